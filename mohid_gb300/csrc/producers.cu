// producers.cu -- device producers of the transport step's inputs: the
// geometry of a new water level (layer thicknesses, distances between cell
// centres, volumes, face areas) and the vertical water flux from continuity.
//
// In MOHID Water these are computed before every transport call by
// ModuleGeometry (Software/MOHIDBase2/ModuleGeometry.F90: ComputeDistances
// GEO:3798-4103, ComputeVolumes GEO:4108-4163, ComputeAreas GEO:4238-4288,
// StoreVolumeZOld GEO:4335-4370) and ModuleHydrodynamic
// (Software/MOHIDWater/ModuleHydrodynamic.F90: WaterFlux_Z_VarGrid
// HD:43270-43308, WaterFlux_Z_FixGrid HD:43315-43349).  Computed here on the
// instance's device arrays, the step's geometry and vertical flux never cross
// the host link: a caller uploads the layer interfaces and horizontal fluxes
// and derives the rest on the GPU.
//
// Every expression is the reference's, in its order, in FP64, compiled with
// --fmad=false (the Fortran rounds a*b+c twice), so the results equal the
// reference's bit for bit.  Each output is written only where the reference
// writes it and keeps its value elsewhere, as MOHID's persistent arrays do.
//
// Layout: Fortran column-major over the Size box (0:ni+1, 0:nj+1, 0:nk+1), i
// fastest.  The geometry passes put one thread on each work-box cell and the
// vertical flux one thread on each column, consecutive threads along i, so
// the loads and stores of a warp are contiguous.
#include <cuda_runtime.h>

#include "../../include/mohid_ad.h"
#include "instance.hpp"

namespace {

constexpr int kThreads = 128;

struct Geo {
    int ni, nj, nk;
    long long NI, sk;                  // Size-box strides along j and k
    const double* SZZ;
    const int* WP;
    const double *DUX, *DVY, *DXX, *DYY;
    int facesOption;
    double *DWZ, *DUZ, *DVZ, *DZZ, *V, *Vold, *AU, *AV;
};

// thread -> work-box cell (i, j, k) of a launch over ni * nj * nk threads
__device__ __forceinline__ bool cell_of(const Geo& g, long long t, int& i, int& j, int& k)
{
    const long long n = (long long)g.ni * g.nj * g.nk;
    if (t >= n) return false;
    i = 1 + (int)(t % g.ni);
    const long long r = t / g.ni;
    j = 1 + (int)(r % g.nj);
    k = 1 + (int)(r / g.nj);
    return true;
}

// StoreVolumeZOld (GEO:4335-4370) and DWZ = SZZ(k-1) - SZZ(k) on water points (GEO:3840-3853)
__global__ void k_geo_dwz(Geo g, int storeOld)
{
    int i, j, k;
    if (!cell_of(g, (long long)blockIdx.x * kThreads + threadIdx.x, i, j, k)) return;
    const long long a = i + g.NI * j + g.sk * k;
    if (storeOld) g.Vold[a] = g.V[a];
    if (g.WP[a] == 1) g.DWZ[a] = g.SZZ[a - g.sk] - g.SZZ[a];
}

// DUZ (j >= 2) and DVZ (i >= 2) between two water points: minimum thickness
// (GEO:3855-3892) or the DUX / DVY-weighted thickness (GEO:3894-3948)
__global__ void k_geo_faces(Geo g)
{
    int i, j, k;
    if (!cell_of(g, (long long)blockIdx.x * kThreads + threadIdx.x, i, j, k)) return;
    const long long a = i + g.NI * j + g.sk * k;
    const bool wp = g.WP[a] == 1;
    if (j >= 2 && wp && g.WP[a - g.NI] == 1) {
        const long long s = a - g.NI, c = i + g.NI * j, cs = c - g.NI;
        if (g.facesOption == MOHID_FACES_MIN_THICKNESS)
            g.DUZ[a] = g.DWZ[a] < g.DWZ[s] ? g.DWZ[a] : g.DWZ[s];    // min(DWZ(j-1), DWZ(j))
        else
            g.DUZ[a] = (g.DWZ[a] * g.DUX[cs] + g.DWZ[s] * g.DUX[c]) / (g.DUX[cs] + g.DUX[c]);
    }
    if (i >= 2 && wp && g.WP[a - 1] == 1) {
        const long long c = i + g.NI * j;
        if (g.facesOption == MOHID_FACES_MIN_THICKNESS)
            g.DVZ[a] = g.DWZ[a] < g.DWZ[a - 1] ? g.DWZ[a] : g.DWZ[a - 1];
        else
            g.DVZ[a] = (g.DWZ[a] * g.DVY[c - 1] + g.DWZ[a - 1] * g.DVY[c]) / (g.DVY[c - 1] + g.DVY[c]);
    }
}

// DZZ on water points (GEO:3960-3972), VolumeZ (GEO:4131-4144) and the face
// areas (GEO:4265-4277) on every work-box cell
__global__ void k_geo_cells(Geo g)
{
    int i, j, k;
    if (!cell_of(g, (long long)blockIdx.x * kThreads + threadIdx.x, i, j, k)) return;
    const long long a = i + g.NI * j + g.sk * k, c = i + g.NI * j;
    if (g.WP[a] == 1) g.DZZ[a] = (g.DWZ[a + g.sk] + g.DWZ[a]) / 2.0;
    g.V[a] = g.DWZ[a] * g.DUX[c] * g.DVY[c];
    g.AU[a] = g.DUZ[a] * g.DYY[c];
    g.AV[a] = g.DVZ[a] * g.DXX[c];
}

// WaterFlux_Z_VarGrid / _FixGrid: one thread per column (i, j), k upwards;
// Qz(k+1) = Qz(k) + West - East + South - North [- dV/dt] on water points.
__global__ void k_vertical_flux(int ni, int nj, int nk, long long NI, long long sk, const double* __restrict__ Qx,
                                const double* __restrict__ Qy, double* __restrict__ Qz,
                                const double* __restrict__ V, const double* __restrict__ Vold,
                                const int* __restrict__ CFU, const int* __restrict__ CFV,
                                const int* __restrict__ WP, double dt, int varGrid)
{
    const long long t = (long long)blockIdx.x * kThreads + threadIdx.x;
    if (t >= (long long)ni * nj) return;
    const int i = 1 + (int)(t % ni), j = 1 + (int)(t / ni);
    for (int k = 1; k <= nk; ++k) {
        const long long a = i + NI * j + sk * k;
        if (WP[a] != 1) continue;
        const double west = Qx[a] * (double)CFU[a];
        const double east = Qx[a + NI] * (double)CFU[a + NI];
        const double south = Qy[a] * (double)CFV[a];
        const double north = Qy[a + 1] * (double)CFV[a + 1];
        double q = Qz[a] + west - east + south - north;
        if (varGrid) q = q - (V[a] - Vold[a]) / dt;
        Qz[a + sk] = q;
    }
}

}  // namespace

using namespace mohid_abi;

extern "C" int mohid_ad_geometry_dev(const int* id, const double* SZZ, const double* DXX, const double* DYY,
                                     const int* faces_option, const int* store_old, int* stat)
{
    TraceRange trace_("mohid_ad_geometry_dev");
    Instance* in = lookup(id);
    if (!in) return fail(MOHID_AD_ERR_ID, stat, "unknown instance id");
    if (!SZZ || !DXX || !DYY || !faces_option || !store_old)
        return fail(MOHID_AD_ERR_NULLPTR, stat, "mohid_ad_geometry_dev: NULL argument");
    if (*faces_option != MOHID_FACES_MIN_THICKNESS && *faces_option != MOHID_FACES_AVERAGE_THICKNESS)
        return fail(MOHID_AD_ERR_OPTION, stat, "faces_option must be MinTickness (3) or AverageTickness (2)");
    if (!in->hydro)
        return fail(MOHID_AD_ERR_OPTION, stat, "set the hydrodynamics (masks) once before the geometry");
    CK(cudaSetDevice(in->device));
    if (!in->DUZ.p) {
        cudaError_t e = in->DUZ.alloc(in->n3);
        if (e == cudaSuccess) e = in->DVZ.alloc(in->n3);
        if (e != cudaSuccess) {
            in->DUZ.release();
            in->DVZ.release();
            return fail(e == cudaErrorMemoryAllocation ? MOHID_AD_ERR_ALLOC : MOHID_AD_ERR_CUDA, stat,
                        cuda_msg("DUZ / DVZ", e));
        }
    }
    Geo g;
    g.ni = in->ni; g.nj = in->nj; g.nk = in->nk;
    g.NI = in->ni + 2;
    g.sk = g.NI * (in->nj + 2);
    g.SZZ = SZZ; g.WP = in->WP.p;
    g.DUX = in->DUX.p; g.DVY = in->DVY.p; g.DXX = DXX; g.DYY = DYY;
    g.facesOption = *faces_option;
    g.DWZ = in->DWZ.p; g.DUZ = in->DUZ.p; g.DVZ = in->DVZ.p; g.DZZ = in->DZZ.p;
    g.V = in->V.p; g.Vold = in->Vold.p; g.AU = in->AreaU.p; g.AV = in->AreaV.p;
    const long long n = (long long)in->ni * in->nj * in->nk;
    const unsigned blocks = (unsigned)((n + kThreads - 1) / kThreads);
    k_geo_dwz<<<blocks, kThreads, 0, in->stream>>>(g, *store_old != 0);
    CK(cudaGetLastError());
    k_geo_faces<<<blocks, kThreads, 0, in->stream>>>(g);
    CK(cudaGetLastError());
    k_geo_cells<<<blocks, kThreads, 0, in->stream>>>(g);
    CK(cudaGetLastError());
    ++in->hydroVersion;
    return ok(stat);
}

extern "C" int mohid_ad_vertical_flux(const int* id, const double* DT, const int* var_grid, int* stat)
{
    TraceRange trace_("mohid_ad_vertical_flux");
    Instance* in = lookup(id);
    if (!in) return fail(MOHID_AD_ERR_ID, stat, "unknown instance id");
    if (!DT || !var_grid) return fail(MOHID_AD_ERR_NULLPTR, stat, "mohid_ad_vertical_flux: NULL argument");
    if (*var_grid && !(*DT > 0.0)) return fail(MOHID_AD_ERR_OPTION, stat, "DT must be > 0 on a variable grid");
    if (!in->hydro) return fail(MOHID_AD_ERR_OPTION, stat, "set the hydrodynamics once before the vertical flux");
    CK(cudaSetDevice(in->device));
    const long long NI = in->ni + 2, sk = NI * (in->nj + 2);
    const long long cols = (long long)in->ni * in->nj;
    k_vertical_flux<<<(unsigned)((cols + kThreads - 1) / kThreads), kThreads, 0, in->stream>>>(
        in->ni, in->nj, in->nk, NI, sk, in->Qx.p, in->Qy.p, in->Qz.p, in->V.p, in->Vold.p, in->CFU.p, in->CFV.p,
        in->WP.p, *DT, *var_grid != 0);
    CK(cudaGetLastError());
    ++in->hydroVersion;
    return ok(stat);
}
