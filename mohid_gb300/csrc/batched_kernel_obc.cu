// batched_kernel_obc.cu -- open-boundary instantiation of the batched step
// (batched_launch.cuh): MassConservation boundary terms compiled in; and the
// boundary mass flux of a step, which the mass fixer's target follows.
#include "batched_launch.cuh"

namespace mohid {
namespace {

constexpr int kFluxThreads = 256;

// v summed over the block in a fixed order (lanes by a shuffle tree, warps in
// order); valid in thread 0
__device__ __forceinline__ double block_sum_fixed(double v, double* red)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    __syncthreads();                               // red may hold an earlier sum
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int q = 0; q < kFluxThreads / 32; ++q) s += red[q];
    return s;
}

// Block (blk, t): tracer t on the boundary columns blk * kFluxThreads + tid,
// strided by the grid.  Each open row of a boundary column gets WFOB from the
// same stored fields and in the same arithmetic as the step (obc_wfob); the
// mass it moves in the step is WFOB * DT times the inflow concentration
// (stored reference, shifted by the fixer's correction, blended with the
// interior value by the decay factor) where WFOB < 0, or times the new stored
// value where WFOB >= 0; both relative to the tracer's constant, whose share
// -(sum of WFOB * DT) * constant the fixer adds.
template <typename QT>
__global__ void __launch_bounds__(kFluxThreads) k_obc_flux(const BatchArgs A, const int* __restrict__ list)
{
    __shared__ double red[kFluxThreads / 32];
    const BLayout& L = A.L;
    const int t = blockIdx.y;
    const int n = list[0];
    const double DT = (double)A.DT;
    const float corr = (float)A.mfix[1 + 2 * A.ntAll + t];
    const long long to = (long long)t * A.ts;
    double z = 0.0, w = 0.0;
    for (int q = blockIdx.x * kFluxThreads + threadIdx.x; q < n; q += gridDim.x * kFluxThreads) {
        const long long c2 = list[1 + q];
        for (int k = A.kfloor[c2]; k <= L.nk; ++k) {
            const long long a = c2 + (long long)k * L.sl;
            const uint8_t fl = A.flag[a];
            if (!(fl & F_OP)) continue;
            const uint8_t flp = k == L.nk ? 0 : A.flag[a + L.sl];
            const uint8_t fw = A.fflag[a], fe = A.fflag[a + L.px], fn = A.fflag[a + 1];
            const float wfob = tile::obc_wfob((fw & FU_ACT) ? tile::ldg_as<QT>(A.Qx, a, A.qsx) : 0.f,
                                              (fe & FU_ACT) ? tile::ldg_as<QT>(A.Qx, a + L.px, A.qsx) : 0.f,
                                              (fw & FV_ACT) ? tile::ldg_as<QT>(A.Qy, a, A.qsy) : 0.f,
                                              (fn & FV_ACT) ? tile::ldg_as<QT>(A.Qy, a + 1, A.qsy) : 0.f,
                                              (fl & F_CFW) ? tile::ldg_as<QT>(A.Qz, a, A.qsz) : 0.f,
                                              (flp & F_CFW) ? tile::ldg_as<QT>(A.Qz, a + L.sl, A.qsz) : 0.f,
                                              A.DVR[a], A.RV[a], A.DT);
            const double wd = (double)wfob * DT;
            const float y = wfob < 0.f ? A.Pin[to + a] * (1.f - A.tdec) + (A.Ref[to + a] - corr) * A.tdec
                                       : A.Pout[to + a];
            z = fma(wd, (double)y, z);
            w += wd;
        }
    }
    z = block_sum_fixed(z, red);
    w = block_sum_fixed(w, red);
    if (threadIdx.x == 0) {
        A.obpart[(long long)t * A.nob + blockIdx.x] = z;
        if (t == 0) A.obpart[(long long)A.ntAll * A.nob + blockIdx.x] = w;
    }
}

}  // namespace

cudaError_t obc_flux(const BatchArgs& a, const int* list, bool halfQ, cudaStream_t s)
{
    if (!a.obpart || !a.Ref || a.t0 != 0 || a.nt != a.ntAll || a.nob < 1) return cudaErrorInvalidValue;
    const dim3 grid(a.nob, a.ntAll);
    if (halfQ) k_obc_flux<__half><<<grid, kFluxThreads, 0, s>>>(a, list);
    else k_obc_flux<float><<<grid, kFluxThreads, 0, s>>>(a, list);
    return cudaGetLastError();
}

cudaError_t launch_batched_open(const BatchArgs& a, const TmaMaps& m, int method, int limiter, bool halfQ,
                                bool halfK, const int2* tiles, int ntl, cudaStream_t s)
{
    return launch_detail::launch_batched_form<true>(a, m, method, limiter, halfQ, halfK, tiles, ntl, s);
}

}  // namespace mohid
