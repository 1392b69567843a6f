/*
 * oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * FP64 CPU restatement of MOHID's tracer advection-diffusion step and the
 * seeded synthetic input generators.  It is the checker for the CUDA path
 * (tests/, __graft_entry__.smoke) and the timed CPU baseline of bench.py;
 * nothing in the product (mohid_gb300/, include/) links or calls it.
 *
 * Parity status: UNPINNED.  The reference has no unit tests, golden vectors or
 * result files for this path (its only test case has an empty
 * WaterProperties_1.dat and no outputs), and its Fortran cannot be compiled in
 * this environment (no Fortran compiler).  The restatement is instead checked
 * against (1) an independent pure-Python restatement of the same Fortran
 * (oracle/ref_py.py) on small grids, bit for bit, and (2) analytic known-answer
 * properties (dense tridiagonal solves, constancy preservation, mass
 * conservation, TVD bounds, land/null handling) in tests/.
 *
 * Array layout: Fortran column-major over the Size box (0:ni+1, 0:nj+1, 0:nk+1),
 * i fastest -- the layout MOHID allocates (Size = WorkSize +/- 1).
 */
#ifndef MOHID_ORACLE_H
#define MOHID_ORACLE_H

#include <stdint.h>
#include "../include/mohid_ad.h"

#ifdef __cplusplus
extern "C" {
#endif

/* SetDischarges (ModuleAdvectionDiffusion.F90:978-1030): per discharge
 * (number of them) its cell count, IgnoreDisch, ByPass and DischVert; per
 * discharge cell of the discharges not ignored, in order, its work-box
 * indices I, J, K, Kmin, Kmax (FillValueInt = -9999999 for "not given"),
 * DischFlow, DischConc and DischConcMF. */
typedef struct ora_discharges {
    int number;
    const int *nCells, *ignore, *bypass, *vert;
    const int *I, *J, *K, *Kmin, *Kmax;
    const double *Flow, *Conc, *ConcMF;
} ora_discharges;

typedef struct ora_domain {
    int ni, nj, nk;                    /* WorkSize upper bounds; lower bounds are 1 */
    /* 2-D, Size box (ni+2)*(nj+2) */
    const double *DUX, *DVY, *DZX, *DZY;
    const int *KFloorZ, *BoundaryPoints2D;
    /* 3-D, Size box (ni+2)*(nj+2)*(nk+2) */
    const double *Wflux_X, *Wflux_Y, *Wflux_Z;
    const double *VolumeZOld, *VolumeZ;
    const double *Visc_H, *Diff_V;
    const double *AreaU, *AreaV, *DZZ, *DWZ;
    const int *OpenPoints3D, *LandPoints3D, *WaterPoints3D;
    const int *ComputeFacesU3D, *ComputeFacesV3D, *ComputeFacesW3D;
    const int *SmallDepths;            /* 2-D, may be NULL */
    const int *NoFluxU, *NoFluxV, *NoFluxW;   /* 3-D, may be NULL (NoAdvFlux / NoDifFlux) */
    const ora_discharges* Disch;              /* may be NULL (no discharges) */
    double* PROPOld;                   /* 3-D, may be NULL: with Orlanski boundaries it receives
                                        * the field as OpenBoundaryCondition saw it (AD:5428-5429) */
} ora_domain;

/* Work arrays of one instance (AllocateVariables, AD:537-684). */
typedef struct ora_work ora_work;
ora_work* ora_work_new(int ni, int nj, int nk);
void ora_work_free(ora_work* w);

/* One FP64 step of one property, in place.  Returns a MOHID_AD_* status.
 * `work` may be NULL (a temporary one is allocated); nthreads <= 0 uses the
 * OpenMP default. */
int ora_step_f64(const ora_domain* d, double* PROP, const double* ReferenceProp,
                 const mohid_ad_params* p, ora_work* work, int nthreads);

/* THOMASZ_NewType2 alone (ModuleFunctions.F90:4026-4123) on Size-box arrays. */
int ora_thomasz(int ni, int nj, int nk, const double* D, const double* E, const double* F,
                const double* TI, double* RES, const int* WaterPoints);

/* ComputeAdvectionFace (ModuleFunctions.F90:10702-10894) for one face.
 * Returns 0, or MOHID_AD_ERR_OPTION where the reference stops. */
int ora_advection_face(const double P[4], const double V[4], const double du[4], double dt,
                       double Q, double VolumeRelMax, int method, int limiter,
                       int nearBoundary, int upwind2, double CFace[4]);

/* GetAdvFlux / GetDifFlux (ModuleAdvectionDiffusion.F90:697-860): the face
 * fluxes of the last step made with CellFluxes, which = 0..5 for AdvFluxX,
 * AdvFluxY, AdvFluxZ, DifFluxX, DifFluxY, DifFluxZ (Size box); NULL if none. */
const double* ora_cell_flux(const ora_work* w, int which);

/* Producers (producers.c): ComputeDistances / ComputeVolumes / ComputeAreas /
 * StoreVolumeZOld of ModuleGeometry, in place, and WaterFlux_Z_VarGrid
 * (var_grid != 0) / _FixGrid of ModuleHydrodynamic, in place on Qz. */
void ora_geometry(int ni, int nj, int nk, const double* SZZ, const int* WP, const double* DUX,
                  const double* DVY, const double* DXX, const double* DYY, int faces_option,
                  int store_old, double* DWZ, double* DUZ, double* DVZ, double* DZZ, double* VolumeZ,
                  double* VolumeZOld, double* AreaU, double* AreaV);
void ora_vertical_flux(int ni, int nj, int nk, const double* Qx, const double* Qy, double* Qz, const double* Vnew,
                       const double* Vold, const int* CFU, const int* CFV, const int* WP, double dt, int var_grid);

/* Compensated (Neumaier) FP64 sum of VolumeZ*PROP over water cells of the work box. */
double ora_mass(const ora_domain* d, const double* PROP);
double ora_mass_f32(const ora_domain* d, const float* PROP);

#ifdef __cplusplus
}
#endif
#endif
