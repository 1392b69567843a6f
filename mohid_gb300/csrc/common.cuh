// common.cuh -- shared definitions of the GB300 advection-diffusion kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define MOHID_NULL_REAL_D (-9.9e15)   // null_real, ModuleGlobalData.F90:143
#define MOHID_MINVALUE_D 1.e-16       // MinValue,  ModuleGlobalData.F90:1812

// Device status bits, latched with atomicOr and read by the host after a step.
#define MOHID_DEV_ZERO_PIVOT 1u
#define MOHID_DEV_NONFINITE  2u
#define MOHID_DEV_BAD_FACE   4u
#define MOHID_DEV_TIMEOUT    8u
#define MOHID_DEV_OBC_EDGE   16u  // Orlanski: an open boundary point off the work box's edges
#define MOHID_DEV_OBC_READ   32u  // Orlanski: a read outside the layer plane (grids under 3 cells wide)

namespace mohid {

// One discharge term at one cell (SetDischarges, AD:4025-4128): its layer, the
// layer range of a uniform discharge (for the water column), flags (1: uniform
// vertical distribution, 2: bypass), DischFlow, DischConc, DischConcMF.
struct DischTerm {
    int k, kmin, kmax, flags;
    double flow, conc, concMF;
};

// Arguments of the plain FP64 step: Fortran layout over the Size box
// (0:ni+1, 0:nj+1, 0:nk+1), i fastest, strides sj = ni+2, sk = (ni+2)(nj+2).
struct PlainArgs {
    int ni, nj, nk;
    long long sj, sk;
    const double* P;
    double* Pout;
    const double *Qx, *Qy, *Qz, *Vold, *V, *ViscH, *DiffV, *AreaU, *AreaV, *DZZ, *DWZ;
    const int *OP, *LP, *WP, *CFU, *CFV, *CFW, *SD;
    const double *DUX, *DVY, *DZX, *DZY;
    const int *KFloor, *BP2D;
    const double* Ref;          // nullptr: closed boundaries
    // Orlanski boundaries (bc 6): the field as OpenBoundaryCondition leaves it
    // (P with the radiated values at the exterior points, orlanski_kernel);
    // the boundary cells read their exterior value there and columns the
    // solve leaves untouched are copied from it.  nullptr otherwise.
    const double* Pobc;
    double DT, schmidtH, schmidtCoefV, schmidtBackV, volumeRelMax, impExpDifV, tdecAux;
    int methodH, limiterH, methodV, limiterV, upwind2H, upwind2V;
    int nullDif, explicitV, docycle, vertical1D, xzflow, bc;
    int impXX, impYY;           // implicit horizontal advection along j (XX) or i (YY)
    int noAdv, noDif;           // NoAdvFlux / NoDifFlux with the masks below
    // AdvectionNudging (AD:1989-2068): the advective terms of a row gather
    // apart and enter scaled by the column's edge factor; nudgeCells as given
    int nudge, nudgeCells;
    const int *NFU, *NFV, *NFW; // NoFluxU/V/W (Size box), or null
    // discharges, or null: terms of column c at dTerms[dStart[c] .. dStart[c+1]),
    // by layer and then in the reference's order (c = i + sj * j)
    const int* dStart;
    const DischTerm* dTerms;
    double *sD, *sE, *sF, *sTI; // rows of the implicit horizontal system (Size box), or null
    // CellFluxes (or null): AdvFluxX/Y/Z and DifFluxX/Y/Z at the west, south and
    // bottom face of each cell, zeroed before the step; the step records the
    // explicit parts, cell_flux_kernel adds the implicit ones after the solve
    double *fAX, *fAY, *fAZ, *fDX, *fDY, *fDZ;
    unsigned int* status;
};

// Steps of the plain kernel (launch_plain_f64 `mode`)
enum PlainMode {
    kPlainFull = 0,         // the whole step, explicit horizontal advection
    kPlainHorizRows = 1,    // 3-D implicit: rows of the horizontal system to sD..sTI
    kPlainVertical = 2,     // 3-D implicit: the column step from the line solution
    kPlainRows2D = 3,       // one layer, implicit: rows with open boundaries and land to sD..sTI
};

// Launchers (plain_f64.cu)
// Orlanski open boundaries (OpenBoundaryCondition AD:5496-5569 with
// OrlanskiCelerity2D FN:4129-4490): the radiated value at the exterior point
// of each open boundary cell, written into S, which must hold a copy of a.P.
// cols: the boundary columns in the reference's order (j outer, i inner).
cudaError_t launch_orlanski(const PlainArgs& a, double* S, const int* cols, int ncols, cudaStream_t s);
cudaError_t launch_plain_f64(const PlainArgs& a, cudaStream_t s, int mode = kPlainFull);
// THOMAS_3D (FN:3760-3876): one tridiagonal system per work-box line along j
// (alongJ) or i, from the first work cell to the halo cell past the last, at
// every layer; rows from D..TI, the halo row D = 0, E = 1, F = 0 and TI = 0
// (null_real on land when landHalo).  W: scratch (Size box); the answer to P,
// which must hold the other cells already.
cudaError_t launch_line_solve(int ni, int nj, int nk, bool alongJ, const double* D, const double* E,
                              const double* F, const double* TI, const int* LP, bool landHalo, double* W,
                              double* P, unsigned int* status, cudaStream_t s);
cudaError_t launch_thomasz_f64(int ni, int nj, int nk, const double* D, const double* E,
                               const double* F, const double* TI, double* RES, const int* WP,
                               unsigned int* status, cudaStream_t s);
cudaError_t launch_check_faces(int ni, int nj, int nk, const int* CFU, const int* CFV,
                               const int* CFW, unsigned int* status, cudaStream_t s);
// CellFluxes, implicit parts (AD:1882-1916): with the new field Pnew and the
// face coefficients of the step (horizontal ones from h.P, vertical ones from
// v.P), into h's flux arrays
cudaError_t launch_cell_fluxes(const PlainArgs& h, const PlainArgs& v, const double* Pnew, double impAdvV,
                               double impDifV, cudaStream_t s);
// Boundary conditions applied after the solve (AD:1874-1880), in place on P
// (Fortran layout).  cols: the 2-D offsets i + sj*j of the boundary columns in
// the reference's sweep order (j outer, i inner), ncols of them.
cudaError_t launch_null_gradient(int ni, int nj, int nk, double* P, const int* CFU, const int* CFV,
                                 const int* KFloor, const int* cols, int ncols, cudaStream_t s);
// rows: the i of the rows whose ends j = 1 and j = nj are both boundary points
// (i = 2..ni-1, in order), then the j of the columns whose ends i = 1 and
// i = ni are (j = 2..nj-1); nrows + ncyc entries.
cudaError_t launch_cyclic(int ni, int nj, int nk, double* P, const double* Ref, const int* KFloor,
                          const int* cols, int ncols, const int* rows, int nrows, int ncyc, cudaStream_t s);

}  // namespace mohid
