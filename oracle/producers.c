/*
 * producers.c -- TEST INFRASTRUCTURE ONLY (checker of the device producers).
 *
 * FP64 restatements of the routines that produce the transport step's
 * geometry and vertical water flux in MOHID Water, in the reference's loop
 * order and expression order, so that the device producers can be compared
 * bit for bit:
 *
 *  - ModuleGeometry (Software/MOHIDBase2/ModuleGeometry.F90, "GEO"):
 *    ComputeDistances GEO:3798-4103 (DWZ, DUZ, DVZ, DZZ; the Lagrangian
 *    thickness gradients are left out), ComputeVolumes GEO:4108-4163 (VolumeZ),
 *    ComputeAreas GEO:4238-4288 (AreaU, AreaV; without impermeability), and
 *    StoreVolumeZOld GEO:4335-4370;
 *  - ModuleHydrodynamic (Software/MOHIDWater/ModuleHydrodynamic.F90, "HD"):
 *    WaterFlux_Z_VarGrid HD:43270-43308 and WaterFlux_Z_FixGrid HD:43315-43349.
 *
 * Arrays are Fortran column-major over the Size box (0:ni+1, 0:nj+1,
 * 0:nk+1), i fastest; the 2-D ones over (0:ni+1, 0:nj+1).  Every output is
 * updated in place where the reference writes it and keeps its value
 * elsewhere, as MOHID's persistent arrays do.  Compile with
 * -ffp-contract=off (the Fortran rounds a*b+c twice).
 */
#include <stddef.h>

#include "oracle.h"

#define S3(i, j, k) ((size_t)(i) + NI * ((size_t)(j) + NJ * (size_t)(k)))
#define S2(i, j) ((size_t)(i) + NI * (size_t)(j))

static inline double dminf(double a, double b) { return (b < a) ? b : a; }   /* Fortran min */

void ora_geometry(int ni, int nj, int nk, const double* SZZ, const int* WP, const double* DUX,
                  const double* DVY, const double* DXX, const double* DYY, int faces_option,
                  int store_old, double* DWZ, double* DUZ, double* DVZ, double* DZZ, double* VolumeZ,
                  double* VolumeZOld, double* AreaU, double* AreaV)
{
    const size_t NI = (size_t)ni + 2, NJ = (size_t)nj + 2;
    /* StoreVolumeZOld (GEO:4335-4370), before the new volumes */
    if (store_old)
        for (int k = 1; k <= nk; ++k)
            for (int j = 1; j <= nj; ++j)
                for (int i = 1; i <= ni; ++i) VolumeZOld[S3(i, j, k)] = VolumeZ[S3(i, j, k)];
    /* DWZ (GEO:3840-3853) */
    for (int k = 1; k <= nk; ++k)
        for (int j = 1; j <= nj; ++j)
            for (int i = 1; i <= ni; ++i)
                if (WP[S3(i, j, k)] == 1) DWZ[S3(i, j, k)] = SZZ[S3(i, j, k - 1)] - SZZ[S3(i, j, k)];
    /* DUZ, DVZ: minimum (GEO:3855-3892) or DUX/DVY-weighted (GEO:3894-3948) thickness */
    for (int k = 1; k <= nk; ++k)
        for (int j = 2; j <= nj; ++j)
            for (int i = 1; i <= ni; ++i)
                if (WP[S3(i, j - 1, k)] == 1 && WP[S3(i, j, k)] == 1) {
                    if (faces_option == MOHID_FACES_MIN_THICKNESS)
                        DUZ[S3(i, j, k)] = dminf(DWZ[S3(i, j - 1, k)], DWZ[S3(i, j, k)]);
                    else
                        DUZ[S3(i, j, k)] = (DWZ[S3(i, j, k)] * DUX[S2(i, j - 1)] + DWZ[S3(i, j - 1, k)] * DUX[S2(i, j)]) /
                                           (DUX[S2(i, j - 1)] + DUX[S2(i, j)]);
                }
    for (int k = 1; k <= nk; ++k)
        for (int j = 1; j <= nj; ++j)
            for (int i = 2; i <= ni; ++i)
                if (WP[S3(i - 1, j, k)] == 1 && WP[S3(i, j, k)] == 1) {
                    if (faces_option == MOHID_FACES_MIN_THICKNESS)
                        DVZ[S3(i, j, k)] = dminf(DWZ[S3(i - 1, j, k)], DWZ[S3(i, j, k)]);
                    else
                        DVZ[S3(i, j, k)] = (DWZ[S3(i, j, k)] * DVY[S2(i - 1, j)] + DWZ[S3(i - 1, j, k)] * DVY[S2(i, j)]) /
                                           (DVY[S2(i - 1, j)] + DVY[S2(i, j)]);
                }
    /* DZZ (GEO:3960-3972): DWZ(k+1) of the top layer is the value held at KUB+1 */
    for (int k = 1; k <= nk; ++k)
        for (int j = 1; j <= nj; ++j)
            for (int i = 1; i <= ni; ++i)
                if (WP[S3(i, j, k)] == 1) DZZ[S3(i, j, k)] = (DWZ[S3(i, j, k + 1)] + DWZ[S3(i, j, k)]) / 2.0;
    /* VolumeZ (GEO:4131-4144): every work-box cell */
    for (int k = 1; k <= nk; ++k)
        for (int j = 1; j <= nj; ++j)
            for (int i = 1; i <= ni; ++i)
                VolumeZ[S3(i, j, k)] = DWZ[S3(i, j, k)] * DUX[S2(i, j)] * DVY[S2(i, j)];
    /* AreaU, AreaV (GEO:4265-4277): every work-box cell */
    for (int k = 1; k <= nk; ++k)
        for (int j = 1; j <= nj; ++j)
            for (int i = 1; i <= ni; ++i) {
                AreaU[S3(i, j, k)] = DUZ[S3(i, j, k)] * DYY[S2(i, j)];
                AreaV[S3(i, j, k)] = DVZ[S3(i, j, k)] * DXX[S2(i, j)];
            }
}

void ora_vertical_flux(int ni, int nj, int nk, const double* Qx, const double* Qy, double* Qz, const double* Vnew,
                       const double* Vold, const int* CFU, const int* CFV, const int* WP, double dt, int var_grid)
{
    const size_t NI = (size_t)ni + 2, NJ = (size_t)nj + 2;
    for (int k = 1; k <= nk; ++k)
        for (int j = 1; j <= nj; ++j)
            for (int i = 1; i <= ni; ++i) {
                const size_t a = S3(i, j, k);
                if (WP[a] != 1) continue;
                const double west = Qx[a] * (double)CFU[a];
                const double east = Qx[S3(i, j + 1, k)] * (double)CFU[S3(i, j + 1, k)];
                const double south = Qy[a] * (double)CFV[a];
                const double north = Qy[S3(i + 1, j, k)] * (double)CFV[S3(i + 1, j, k)];
                if (var_grid) {
                    const double dVdt = (Vnew[a] - Vold[a]) / dt;
                    Qz[S3(i, j, k + 1)] = Qz[a] + west - east + south - north - dVdt;
                } else {
                    Qz[S3(i, j, k + 1)] = Qz[a] + west - east + south - north;
                }
            }
}
