// batched_kernel_obc.cu -- the boundary mass flux of a batched step with
// MassConservation open boundaries, which the mass fixer's target follows.
#include "batched_launch.cuh"

namespace mohid {
namespace {

constexpr int kFluxThreads = 256;

constexpr int kFluxWarps = kFluxThreads / 32;

// v summed over the warp by a fixed shuffle tree; valid in lane 0
__device__ __forceinline__ double warp_sum_fixed(double v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Boundary cells (column q of the list, layer k) are spread over the threads,
// kFluxThreads consecutive cells per block and pass (consecutive columns at one
// layer).  Each open cell gets WFOB once, from the same stored fields and in the
// same arithmetic as the step (obc_wfob).  Every tracer's share is then summed
// over the block in a fixed order.  The mass a cell moves in the step is
// WFOB * DT times the inflow concentration where WFOB < 0 (stored reference,
// shifted by the fixer's correction, blended with the interior value by the
// decay factor), or times the new stored value where WFOB >= 0.  Both are
// relative to the tracer's constant, whose share -(sum of WFOB * DT) *
// constant the fixer adds.  Shared memory: per-tracer running sums
// (ntAll + 1 doubles, the last for WFOB * DT), the warps' sums of one pass
// ((ntAll + 1) x kFluxWarps doubles) and the corrections (ntAll floats).
template <typename QT>
__global__ void __launch_bounds__(kFluxThreads) k_obc_flux(const BatchArgs A, const int* __restrict__ list)
{
    extern __shared__ double acc[];
    const BLayout& L = A.L;
    const int nt = A.ntAll;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    double* wpart = acc + nt + 1;
    float* corr = reinterpret_cast<float*>(wpart + (size_t)(nt + 1) * kFluxWarps);
    for (int t = threadIdx.x; t <= nt; t += kFluxThreads) {
        acc[t] = 0.0;
        if (t < nt) corr[t] = (float)A.mfix[1 + 2 * nt + t];
    }
    __syncthreads();
    const int n = list[0];
    const long long ncell = (long long)n * L.nk;
    const double DT = (double)A.DT;
    for (long long base = (long long)blockIdx.x * kFluxThreads; base < ncell;
         base += (long long)gridDim.x * kFluxThreads) {
        const long long e = base + threadIdx.x;
        double wd = 0.0;
        long long a = 0, r = 0;
        bool act = false, in = false;
        if (e < ncell) {
            const long long c2 = list[1 + (int)(e % n)];
            const int k = 1 + (int)(e / n);
            a = c2 + (long long)k * L.sl;
            r = (long long)A.refIdx[c2] * A.rk + k;   // the cell's reference (boundary columns only)
            if (k >= A.kfloor[c2] && (A.flag[a] & F_OP)) {
                const uint8_t fl = A.flag[a];
                const uint8_t flp = k == L.nk ? 0 : A.flag[a + L.sl];
                const uint8_t fw = A.fflag[a], fe = A.fflag[a + L.px], fn = A.fflag[a + 1];
                const float wfob = tile::obc_wfob((fw & FU_ACT) ? tile::ldg_as<QT>(A.Qx, a, A.qsx) : 0.f,
                                                  (fe & FU_ACT) ? tile::ldg_as<QT>(A.Qx, a + L.px, A.qsx) : 0.f,
                                                  (fw & FV_ACT) ? tile::ldg_as<QT>(A.Qy, a, A.qsy) : 0.f,
                                                  (fn & FV_ACT) ? tile::ldg_as<QT>(A.Qy, a + 1, A.qsy) : 0.f,
                                                  (fl & F_CFW) ? tile::ldg_as<QT>(A.Qz, a, A.qsz) : 0.f,
                                                  (flp & F_CFW) ? tile::ldg_as<QT>(A.Qz, a + L.sl, A.qsz) : 0.f,
                                                  A.DVR[a], A.RV[a], A.DT);
                wd = (double)wfob * DT;
                act = true;
                in = wfob < 0.f;
            }
        }
        // per tracer a warp sum (no barrier, so the tracers' loads overlap),
        // then the warps' sums in order
        const double ws = warp_sum_fixed(wd);
        if (lane == 0) wpart[(size_t)nt * kFluxWarps + warp] = ws;
        for (int t = 0; t < nt; ++t) {
            double v = 0.0;
            if (act) {
                const long long ta = (long long)t * A.ts + a;
                const float y = in ? A.Pin[ta] * (1.f - A.tdec) + (A.Ref[(long long)t * A.rts + r] - corr[t]) * A.tdec
                                   : A.Pout[ta];
                v = wd * (double)y;
            }
            v = warp_sum_fixed(v);
            if (lane == 0) wpart[(size_t)t * kFluxWarps + warp] = v;
        }
        __syncthreads();
        for (int t = threadIdx.x; t <= nt; t += kFluxThreads) {
            double z = 0.0;
            for (int w = 0; w < kFluxWarps; ++w) z += wpart[(size_t)t * kFluxWarps + w];
            acc[t] += z;
        }
        __syncthreads();                           // wpart is rewritten by the next pass
    }
    __syncthreads();
    for (int t = threadIdx.x; t < nt; t += kFluxThreads) A.obpart[(long long)t * A.nob + blockIdx.x] = acc[t];
    if (threadIdx.x == 0) A.obpart[(long long)nt * A.nob + blockIdx.x] = acc[nt];
}

}  // namespace

cudaError_t obc_flux(const BatchArgs& a, const int* list, bool halfQ, cudaStream_t s)
{
    if (!a.obpart || !a.Ref || a.t0 != 0 || a.nt != a.ntAll || a.nob < 1) return cudaErrorInvalidValue;
    const size_t smem = sizeof(double) * (size_t)(a.ntAll + 1) * (1 + kFluxWarps) + sizeof(float) * (size_t)a.ntAll;
    if (smem > 48 * 1024) return cudaErrorInvalidValue;
    if (halfQ) k_obc_flux<__half><<<a.nob, kFluxThreads, smem, s>>>(a, list);
    else k_obc_flux<float><<<a.nob, kFluxThreads, smem, s>>>(a, list);
    return cudaGetLastError();
}

}  // namespace mohid
