// batched_pack.cu -- conversions between the Fortran FP64 Size-box arrays and
// the batched layout, tracer anomaly bookkeeping, continuity check and the
// compensated mass budget of the batched form.
//
// Every 3-D pass walks rows (j, k) of the Size box: one block per row at a
// time, threads along i, so the Fortran reads and the batched-layout writes
// are both contiguous and no thread divides a 64-bit index.
#include "batched.cuh"
#include "common.cuh"

namespace mohid {
namespace {

constexpr int kRowThreads = 256;

// rows (j, k), j = 0..NJ-1, k = 0..nz-1 of the Size box, shared out over the grid;
// f(e, g, i, j, k): e Fortran index, g batched-layout index
template <typename F>
__device__ __forceinline__ void for_rows(const BLayout& L, int k0, int nz, F f)
{
    const int NI = L.ni + 2, NJ = L.nj + 2;
    const int rows = NJ * nz;
    for (int r = blockIdx.x; r < rows; r += gridDim.x) {
        const int j = r % NJ, k = k0 + r / NJ;
        const long long e0 = (long long)NI * ((long long)j + (long long)NJ * k);
        const long long g0 = L.at(0, j, k);
        for (int i = threadIdx.x; i < NI; i += blockDim.x) f(e0 + i, g0 + i, i, j, k);
    }
}

inline unsigned row_blocks(const BLayout& L, int nz)
{
    const long long rows = (long long)(L.nj + 2) * nz;
    return (unsigned)(rows < 1 ? 1 : (rows > 16384 ? 16384 : rows));
}

// FP64 -> FP32, rounded to nearest even, with integer instructions only (GB300
// runs FP64 instructions at a small fraction of the integer rate).  Values
// below the FP32 normal range (|x| < 2^-126) become a signed zero; overflow
// gives a signed infinity, NaN stays NaN.
__device__ __forceinline__ float f64_to_f32(double x)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
    const int e = (int)((b >> 52) & 0x7ff);
    const unsigned long long m = b & 0xfffffffffffffull;
    if (e == 0x7ff) return __uint_as_float(sign | 0x7f800000u | (m ? 0x400000u : 0u));
    const int ef = e - 1023 + 127;
    if (ef >= 255) return __uint_as_float(sign | 0x7f800000u);
    if (ef <= 0) return __uint_as_float(sign);
    const unsigned mf = (unsigned)(m >> 29);
    const unsigned long long rem = m & 0x1fffffffull;
    unsigned r = ((unsigned)ef << 23) | mf;
    if (rem > 0x10000000ull || (rem == 0x10000000ull && (mf & 1u))) r += 1u;   // a carry may reach infinity
    return __uint_as_float(sign | r);
}

// the 64-bit patterns of two doubles are equal (no FP64 instruction)
__device__ __forceinline__ bool same_bits(double a, double b)
{
    return __double_as_longlong(a) == __double_as_longlong(b);
}

// |x| as its bit pattern (orders like |x| for non-NaN values, no FP64 instruction)
__device__ __forceinline__ unsigned long long abs_bits(double x)
{
    return (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull;
}

// v - (double)vh rounded to FP32, vh = f64_to_f32(v) (the low part of the
// volume pair v ~ vh + vlo), with integer instructions: at v's scale
// 2^(e - 1075) the difference is an integer D of at most 29 bits, converted
// with one rounding to nearest and scaled by a power of two (exact).  Values
// whose pair leaves the FP32 normal range take the FP64 path.
__device__ __forceinline__ float f64_lo_f32(double v, float vh)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    const int e = (int)((b >> 52) & 0x7ff);
    const unsigned hb = __float_as_uint(vh);
    const int ef = (int)((hb >> 23) & 0xff);
    if (e < 949 || e > 1150 || ef == 0 || ef == 255) return f64_to_f32(v - (double)vh);
    const long long M = (long long)((b & 0xfffffffffffffull) | (1ull << 52));
    const int c = ef - (e - 896);                  // 1 where rounding carried into the exponent
    const long long H = (long long)((hb & 0x7fffffu) | 0x800000u) << (29 + c);
    const long long D = (b >> 63) ? H - M : M - H; // v - vh in units of 2^(e - 1075), |D| <= 2^28
    return __int2float_rn((int)D) * __int_as_float((e - 1075 + 127) << 23);
}

// The constant-preservation check of one cell without FP64 arithmetic: the
// budget R = qw - qe + qs - qn + qb - qt - dv (or R = qt alone, on the top cell
// of an open boundary column) summed exactly as 64-bit integers at the scale
// of the largest term (its 53-bit mantissa at bits 5..57, so seven terms
// cannot overflow; bits below 2^-57 of it are dropped).  Returns |R| - tol *
// max |term| where that is positive (the cell fails the check), else 0.
// u (< 2^62) as FP32 from its two 32-bit halves (64-bit conversions would
// run on the FP64 pipe)
__device__ __forceinline__ float u64_to_f32(unsigned long long u)
{
    return fmaf(__uint2float_rn((unsigned)(u >> 32)), 4294967296.f, __uint2float_rn((unsigned)u));
}

__device__ __forceinline__ double budget_excess(const double (&x)[7], bool bp, float tol)
{
    // the largest exponent (a zero term counts as exponent 1), then each term
    // at that scale, its fields taken again from its bits
    int emax = 1;
#pragma unroll
    for (int q = 0; q < 7; ++q)
        emax = max(emax, (int)((unsigned long long)__double_as_longlong(x[q]) >> 52) & 0x7ff);
    if (emax == 0x7ff) return 1.0;                 // Inf or NaN: fails
    long long S = 0;
    unsigned long long mx = 0;
#pragma unroll
    for (int q = 0; q < 7; ++q) {
        const unsigned long long b = (unsigned long long)__double_as_longlong(x[q]);
        const int e = (int)((b >> 52) & 0x7ff);
        const unsigned long long m = (b & 0xfffffffffffffull) | (e ? (1ull << 52) : 0ull);
        const int sh = emax - (e ? e : 1);
        const unsigned long long v = sh > 57 ? 0ull : (m << 5) >> sh;
        mx = v > mx ? v : mx;
        // qe, qn, qt and dv enter with a minus sign
        const bool neg = ((b >> 63) != 0) != (q == 1 || q == 3 || q == 5 || q == 6);
        if (!bp || q == 5) S += neg ? -(long long)v : (long long)v;
    }
    const unsigned long long aS = S < 0 ? (unsigned long long)(-S) : (unsigned long long)S;
    const float d = u64_to_f32(aS) - tol * u64_to_f32(mx);
    if (!(d > 0.f)) return 0.0;
    // rare: back to absolute units, 2^(emax - 1080)
    return (double)d * (emax > 57 ? __longlong_as_double((long long)(emax - 57) << 52) : 1e-300);
}

// Neumaier-compensated accumulation s + c += x
__device__ __forceinline__ void neu_add(double& s, double& c, double x)
{
    const double t = s + x;
    if (fabs(s) >= fabs(x)) c += (s - t) + x; else c += (x - t) + s;
    s = t;
}

// Neumaier pairs (s, c) of a warp combined in a fixed order; lane 0 holds the result
__device__ __forceinline__ void warp_neu(double& s, double& c)
{
    for (int o = 16; o > 0; o >>= 1) {
        const double os = __shfl_down_sync(0xffffffffu, s, o), oc = __shfl_down_sync(0xffffffffu, c, o);
        neu_add(s, c, os);
        c += oc;
    }
}

// (s, c) of all kRowThreads threads combined in a fixed order; the sum is valid in thread 0
__device__ __forceinline__ double block_neu(double s, double c)
{
    __shared__ double ws[kRowThreads / 32], wc[kRowThreads / 32];
    warp_neu(s, c);
    if ((threadIdx.x & 31) == 0) { ws[threadIdx.x >> 5] = s; wc[threadIdx.x >> 5] = c; }
    __syncthreads();
    double S = 0.0, C = 0.0;
    if (threadIdx.x == 0)
        for (int q = 0; q < kRowThreads / 32; ++q) { neu_add(S, C, ws[q]); C += wc[q]; }
    return S + C;
}

// ------------------------------------------------------------------ hydrodynamic fields
struct PackIn {
    const double *Qx, *Qy, *Qz, *V, *Vold, *Vis, *Dif, *AU, *AV, *DZZ;
    const int *WP, *OP, *LP, *CFU, *CFV, *CFW;
};
struct PackOut {
    void *Qx, *Qy, *Qz, *Vis, *Dif;     // float, or __half (scaled) when halfQ / halfK
    const float* inv;                   // 1/scale of the __half fields (device, 5), or null
    int halfQ, halfK;
    float *AU, *AV, *rDZZ, *RV, *DVR, *Vhi, *Vlo;
    uint8_t *flag, *fflag;
    unsigned* moving;                   // set when VolumeZ != VolumeZOld on any cell
};

__device__ __forceinline__ void put(void* dst, bool half, float inv, long long g, double v)
{
    const float f = f64_to_f32(v);
    if (half) reinterpret_cast<__half*>(dst)[g] = __float2half_rn(f * inv);
    else reinterpret_cast<float*>(dst)[g] = f;
}

// one pass over every cell of the Size box: transports and diffusivities
// (FP32 or scaled FP16), areas, 1/DZZ, 1/V, (V - Vold)/V with the difference
// formed in FP64 (thin layers make it cancel), VolumeZ as an FP32 pair,
// the cell flag byte and the face flag byte.  Face flags restate the per-face
// conditions of ComputeAdvection1D_V2 (FN:10559: both cells open; NearBoundary
// when the cell upstream of the upwind cell is not open) and the compute-face
// masks; faces on the j = JUB+1 / i = IUB+1 planes are never applied by the
// reference.
__global__ void __launch_bounds__(kRowThreads) k_pack_fields(PackIn in, PackOut out, BLayout L)
{
    const int NI = L.ni + 2, NJ = L.nj + 2;
    float iv[5] = {1.f, 1.f, 1.f, 1.f, 1.f};
    if (out.inv)
        for (int q = 0; q < 5; ++q) iv[q] = out.inv[q];
    for_rows(L, 0, L.nk + 2, [&](long long e, long long g, int i, int j, int k) {
        put(out.Qx, out.halfQ, iv[0], g, in.Qx[e]);
        put(out.Qy, out.halfQ, iv[1], g, in.Qy[e]);
        put(out.Qz, out.halfQ, iv[2], g, in.Qz[e]);
        put(out.Vis, out.halfK, iv[3], g, in.Vis[e]);
        put(out.Dif, out.halfK, iv[4], g, in.Dif[e]);
        out.AU[g] = f64_to_f32(in.AU[e]);
        out.AV[g] = f64_to_f32(in.AV[e]);
        const float dz = f64_to_f32(in.DZZ[e]);
        out.rDZZ[g] = dz != 0.f ? __frcp_rn(dz) : 0.f;
        const double v = in.V[e], vo = in.Vold[e];
        const float vh = f64_to_f32(v);
        out.Vhi[g] = vh;
        if (same_bits(v, vo)) {
            out.Vlo[g] = f64_lo_f32(v, vh);
            out.RV[g] = vh != 0.f ? __frcp_rn(vh) : 0.f;
            out.DVR[g] = 0.f;
        } else {
            *out.moving = 1u;
            out.Vlo[g] = f64_lo_f32(v, vh);
            const float rv = vh != 0.f ? __frcp_rn(vh) : 0.f;
            out.RV[g] = rv;
            out.DVR[g] = f64_to_f32(v - vo) * rv;
        }
        const bool cfu = in.CFU[e] == 1 && j != L.nj + 1, cfv = in.CFV[e] == 1 && i != L.ni + 1;
        const bool op = in.OP[e] == 1;
        uint8_t f = 0;
        if (in.WP[e] == 1) f |= F_WP;
        if (op) f |= F_OP;
        if (cfu) f |= F_CFU;
        if (cfv) f |= F_CFV;
        if (in.CFW[e] == 1) f |= F_CFW;
        if (in.LP[e] == 1) f |= F_LP;
        out.flag[g] = f;
        auto opn = [&](int di, int dj) -> bool {
            const int ii = i + di, jj = j + dj;
            return ii >= 0 && ii < NI && jj >= 0 && jj < NJ && in.OP[e + di + (long long)NI * dj] == 1;
        };
        uint8_t ff = 0;
        if (cfu) { ff |= FU_ACT; if (op && opn(0, -1)) ff |= FU_ADV; }
        if (opn(0, -2)) ff |= FU_TVDP;
        if (opn(0, 1)) ff |= FU_TVDN;
        if (cfv) { ff |= FV_ACT; if (op && opn(-1, 0)) ff |= FV_ADV; }
        if (opn(-2, 0)) ff |= FV_TVDP;
        if (opn(1, 0)) ff |= FV_TVDN;
        out.fflag[g] = ff;
    });
}

// The repack of a new hydrodynamic state in one pass over the Fortran-layout
// FP64 fields (k_pack_fields' conversions) that also
//  * flags a bit-level change of VolumeZ against the last pack (Vprev, updated
//    where it changed);
//  * sums VolumeZ over water cells of the work box (per-thread FP64, blocks
//    by a fixed-order compensated tree; partials to vpart[2 b], vpart[2 b + 1] = 0);
//  * when rDT > 0, checks that the step maps constants onto themselves (the
//    check of k_continuity): on open non-boundary water cells
//    R = Qx(w) - Qx(e) + Qy(s) - Qy(n) + Qz(k) - Qz(k+1) - (V - Vold)/DT over
//    the faces the step applies, on the top cell of open boundary columns R =
//    Qz(KUB+1); *cont = max(0, max of |R| - tol * m), m the largest magnitude
//    among the cell's terms (compared on the bit patterns, no FP64 work).
// MASKS: the masks changed since the last pack and the flag bytes are formed
// from them; otherwise the stored flag bytes are kept and read instead.
struct FuseArgs {
    double* Vprev;
    unsigned* vchanged;
    double* vpart;
    const int* BP2D;
    double rDT, tol;
    unsigned long long* cont;
};

template <bool MASKS>
__global__ void __launch_bounds__(kRowThreads, 6) k_pack_state(PackIn in, PackOut out, BLayout L, FuseArgs f)
{
    const int NI = L.ni + 2, NJ = L.nj + 2, nk = L.nk;
    const long long sk = (long long)NI * NJ;
    float iv[5] = {1.f, 1.f, 1.f, 1.f, 1.f};
    if (out.inv)
        for (int q = 0; q < 5; ++q) iv[q] = out.inv[q];
    double vs = 0.0, cm = 0.0;
    bool changed = false;
    const float tolf = (float)f.tol;
    for_rows(L, 0, L.nk + 2, [&](long long e, long long g, int i, int j, int k) {
        put(out.Qx, out.halfQ, iv[0], g, in.Qx[e]);
        put(out.Qy, out.halfQ, iv[1], g, in.Qy[e]);
        put(out.Qz, out.halfQ, iv[2], g, in.Qz[e]);
        put(out.Vis, out.halfK, iv[3], g, in.Vis[e]);
        put(out.Dif, out.halfK, iv[4], g, in.Dif[e]);
        out.AU[g] = f64_to_f32(in.AU[e]);
        out.AV[g] = f64_to_f32(in.AV[e]);
        const float dz = f64_to_f32(in.DZZ[e]);
        out.rDZZ[g] = dz != 0.f ? __frcp_rn(dz) : 0.f;
        const double v = in.V[e], vo = in.Vold[e];
        const float vh = f64_to_f32(v);
        out.Vhi[g] = vh;
        out.Vlo[g] = f64_lo_f32(v, vh);
        const float rv = vh != 0.f ? __frcp_rn(vh) : 0.f;
        out.RV[g] = rv;
        const bool still = same_bits(v, vo);
        if (still) {
            out.DVR[g] = 0.f;
        } else {
            *out.moving = 1u;
            out.DVR[g] = f64_to_f32(v - vo) * rv;
        }
        if (!same_bits(v, f.Vprev[e])) { changed = true; f.Vprev[e] = v; }
        uint8_t fl;
        if (MASKS) {
            const bool cfu = in.CFU[e] == 1 && j != L.nj + 1, cfv = in.CFV[e] == 1 && i != L.ni + 1;
            const bool op = in.OP[e] == 1;
            fl = 0;
            if (in.WP[e] == 1) fl |= F_WP;
            if (op) fl |= F_OP;
            if (cfu) fl |= F_CFU;
            if (cfv) fl |= F_CFV;
            if (in.CFW[e] == 1) fl |= F_CFW;
            if (in.LP[e] == 1) fl |= F_LP;
            out.flag[g] = fl;
            auto opn = [&](int di, int dj) -> bool {
                const int ii = i + di, jj = j + dj;
                return ii >= 0 && ii < NI && jj >= 0 && jj < NJ && in.OP[e + di + (long long)NI * dj] == 1;
            };
            uint8_t ff = 0;
            if (cfu) { ff |= FU_ACT; if (op && opn(0, -1)) ff |= FU_ADV; }
            if (opn(0, -2)) ff |= FU_TVDP;
            if (opn(0, 1)) ff |= FU_TVDN;
            if (cfv) { ff |= FV_ACT; if (op && opn(-1, 0)) ff |= FV_ADV; }
            if (opn(-2, 0)) ff |= FV_TVDP;
            if (opn(1, 0)) ff |= FV_TVDN;
            out.fflag[g] = ff;
        } else {
            fl = out.flag[g];
        }
        const bool work = i >= 1 && i <= L.ni && j >= 1 && j <= L.nj && k >= 1 && k <= nk;
        if (!work) return;
        if (fl & F_WP) vs += v;
        if (f.rDT > 0.0 && (fl & F_OP)) {
            // the east / north / top neighbours' flags: written by other
            // threads in MASKS mode, so formed here from the masks
            bool cfe, cfn, cft;
            if (MASKS) {
                cfe = in.CFU[e + NI] == 1 && j + 1 != L.nj + 1;
                cfn = in.CFV[e + 1] == 1 && i + 1 != L.ni + 1;
                cft = in.CFW[e + sk] == 1;
            } else {
                cfe = out.flag[g + L.px] & F_CFU;
                cfn = out.flag[g + 1] & F_CFV;
                cft = out.flag[g + L.sl] & F_CFW;
            }
            const bool bp = f.BP2D && f.BP2D[i + (long long)NI * j] == 1;
            if (bp && k != nk) return;
            const double qw = (fl & F_CFU) ? in.Qx[e] : 0.0, qe = cfe ? in.Qx[e + NI] : 0.0;
            const double qs = (fl & F_CFV) ? in.Qy[e] : 0.0, qn = cfn ? in.Qy[e + 1] : 0.0;
            const double qb = (fl & F_CFW) ? in.Qz[e] : 0.0;
            const double qt = (k < nk) ? (cft ? in.Qz[e + sk] : 0.0) : in.Qz[e + sk];
            const double dv = still ? 0.0 : (v - vo) * f.rDT;
            const double terms[7] = {qw, qe, qs, qn, qb, qt, dv};
            const double x = budget_excess(terms, bp, tolf);
            if (__double_as_longlong(x) != 0 && x > cm) cm = x;   // x != 0 only where the check fails
        }
    });
    if (__any_sync(0xffffffffu, changed) && (threadIdx.x & 31) == 0) *f.vchanged = 1u;
    if (f.rDT > 0.0) {
        for (int o = 16; o > 0; o >>= 1) cm = fmax(cm, __shfl_xor_sync(0xffffffffu, cm, o));
        if ((threadIdx.x & 31) == 0 && cm > 0.0) atomicMax(f.cont, (unsigned long long)__double_as_longlong(cm));
    }
    const double S = block_neu(vs, 0.0);
    if (threadIdx.x == 0) {
        f.vpart[2 * blockIdx.x] = S;
        f.vpart[2 * blockIdx.x + 1] = 0.0;
    }
}

__global__ void __launch_bounds__(kRowThreads) k_pack_shift_f32(const double* __restrict__ src, float* __restrict__ dst,
                                                               const int* __restrict__ WP, double shift, BLayout L)
{
    for_rows(L, 0, L.nk + 2, [&](long long e, long long g, int, int, int) {
        dst[g] = (float)(src[e] - (WP[e] == 1 ? shift : 0.0));
    });
}

// mean over water cells: per-block sums and counts, then one ordered final pass
// (deterministic, so the stored anomalies are reproducible bit for bit)
__global__ void __launch_bounds__(kRowThreads) k_water_sum(const double* src, const int* WP, BLayout L, double* partial)
{
    __shared__ int scount[kRowThreads / 32];
    double s = 0.0;
    int cnt = 0;
    for_rows(L, 0, L.nk + 2, [&](long long e, long long, int, int, int) {
        if (WP[e] == 1) { s += src[e]; ++cnt; }
    });
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, o);
    if ((threadIdx.x & 31) == 0) scount[threadIdx.x >> 5] = cnt;
    const double S = block_neu(s, 0.0);
    if (threadIdx.x == 0) {
        long long C = 0;
        for (int q = 0; q < kRowThreads / 32; ++q) C += scount[q];
        partial[2 * blockIdx.x] = S;
        partial[2 * blockIdx.x + 1] = (double)C;
    }
}

// one warp: partial[2q] summed (compensated, fixed order), and partial[2q+1] summed
__device__ void warp_partials(const double* partial, int nb, double& sum, double& second)
{
    const int lane = threadIdx.x & 31;
    double s = 0.0, c = 0.0, t = 0.0;
    for (int q = lane; q < nb; q += 32) { neu_add(s, c, partial[2 * q]); t += partial[2 * q + 1]; }
    warp_neu(s, c);
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
    sum = s + c;
    second = t;
}

__global__ void k_water_mean(const double* partial, int nb, double* out)
{
    double S, Cn;
    warp_partials(partial, nb, S, Cn);
    if (threadIdx.x == 0) *out = Cn > 0.0 ? S / Cn : 0.0;
}

// Continuity over open, non-boundary water cells, with the fluxes the step
// applies (Fortran-layout FP64 inputs):
//   R = Qx(w) - Qx(e) + Qy(s) - Qy(n) + Qz(k) - Qz(k+1) - (V - Vold)/DT
// over the faces the step applies, and on the top cell of each open boundary
// column R = Qz(KUB+1); the result is max(0, max over cells of |R| - tol *
// the largest magnitude among the terms).  When it is 0 the step maps a
// constant field onto itself to round-off.
__global__ void __launch_bounds__(kRowThreads) k_continuity(const double* Qx, const double* Qy, const double* Qz,
                                                          const double* V, const double* Vold, const int* OP,
                                                          const int* CFU, const int* CFV, const int* CFW,
                                                          const int* BP2D, double rDT, double tol, BLayout L,
                                                          unsigned long long* out)
{
    const int NI = L.ni + 2, nk = L.nk;
    const long long sk = (long long)NI * (L.nj + 2);
    double m = 0.0;
    for_rows(L, 1, nk, [&](long long a, long long, int i, int j, int k) {
        if (i < 1 || i > L.ni || j < 1 || j > L.nj) return;
        if (OP[a] != 1) return;
        // an open boundary cell maps constants onto themselves (its reference
        // shifted with them) when its exterior-face balance WFOB takes up the
        // rest, except for the surface face, which the step applies at the
        // top cell but WFOB leaves out: that flux must vanish there
        const bool bp = BP2D && BP2D[i + (long long)NI * j] == 1;
        if (bp && k != nk) return;
        // the faces the step applies: compute faces, those on the j = JUB+1 /
        // i = IUB+1 planes excepted
        const double qw = CFU[a] == 1 ? Qx[a] : 0.0;
        const double qe = (CFU[a + NI] == 1 && j + 1 != L.nj + 1) ? Qx[a + NI] : 0.0;
        const double qs = CFV[a] == 1 ? Qy[a] : 0.0;
        const double qn = (CFV[a + 1] == 1 && i + 1 != L.ni + 1) ? Qy[a + 1] : 0.0;
        const double qb = CFW[a] == 1 ? Qz[a] : 0.0;
        const double qt = (k < nk && CFW[a + sk] == 1) ? Qz[a + sk] : (k == nk ? Qz[a + sk] : 0.0);
        const double dv = (V[a] - Vold[a]) * rDT;
        unsigned long long mb = abs_bits(qw);
        mb = max(mb, abs_bits(qe)); mb = max(mb, abs_bits(qs)); mb = max(mb, abs_bits(qn));
        mb = max(mb, abs_bits(qb)); mb = max(mb, abs_bits(qt)); mb = max(mb, abs_bits(dv));
        const double r = bp ? qt : qw - qe + qs - qn + qb - qt - dv;   // bp: the boundary column's surface flux
        m = fmax(m, fma(-tol, __longlong_as_double((long long)mb), fabs(r)));   // > 0 where |R| > tol * max |term|
    });
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, (unsigned long long)__double_as_longlong(m));
}

// open-boundary references of the boundary columns (element e = q * nk2 + k)
__global__ void k_pack_ref(const double* __restrict__ src, const int* __restrict__ WP, const int* __restrict__ cols,
                           long long n, int nk2, long long sk, double shift, float* __restrict__ dst)
{
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const long long c = cols[e / nk2] + sk * (e % nk2);
        dst[e] = (float)(src[c] - (WP[c] == 1 ? shift : 0.0));
    }
}
__global__ void k_unshift_ref(float* R, const int* __restrict__ WP, const int* __restrict__ cols, long long n,
                              int nk2, long long sk, double shift)
{
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const long long c = cols[e / nk2] + sk * (e % nk2);
        if (WP[c] == 1) R[e] = (float)((double)R[e] + shift);
    }
}
__global__ void k_ref_index(const int* __restrict__ cols, int ncols, int sj, BLayout L, int* idx)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= ncols) return;
    const int c = cols[q];
    idx[L.at2(c % sj, c / sj)] = q;
}

// ImposeNullGradient on the batched tracers: thread (k, t) walks the boundary
// columns in the reference's order at layer k (k = 0..KUB from |KFloorZ|), so
// a cell sees the new values of the boundary cells swept before it.  The
// neighbours across compute faces are water cells, stored relative to the
// same constant as the boundary cell, so their mean is taken as stored.  The
// compute faces come from the cell flags (F_CFU of a cell is its west face,
// F_CFV its south face), which the NoFlux masks leave alone.
__global__ void k_null_gradient_b(float* P, long long ts, int nt, const uint8_t* __restrict__ flag,
                                  const int* __restrict__ cols, int ncols, const int* __restrict__ KFloor, BLayout L)
{
    const int nk1 = L.nk + 1;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nk1 * nt) return;
    const int k = e % nk1, t = e / nk1, sj = L.ni + 2;
    float* Pt = P + (long long)t * ts;
    for (int q = 0; q < ncols; ++q) {
        const int c = cols[q];
        const int kf = KFloor[c];
        if (k < (kf < 0 ? -kf : kf)) continue;
        const long long a = L.at(c % sj, c / sj, k);
        const float cv1 = (flag[a + 1] & F_CFV) ? 1.f : 0.f, cv0 = (flag[a] & F_CFV) ? 1.f : 0.f;
        const float cu1 = (flag[a + L.px] & F_CFU) ? 1.f : 0.f, cu0 = (flag[a] & F_CFU) ? 1.f : 0.f;
        const float aux = cv1 + cv0 + cu1 + cu0;
        if (aux <= 0.f) continue;
        Pt[a] = (Pt[a + 1] * cv1 + Pt[a - 1] * cv0 + Pt[a + L.px] * cu1 + Pt[a - L.px] * cu0) / aux;
    }
}

// Prop_CyclicBoundary (AD:2121-2224) on nt batched FP32 tracers, after the
// solve, in two launches.  First every boundary column takes its reference at
// k = 1..KUB: thread (q, k, t), the reference stored relative to the tracer's
// constant, less the mass fixer's correction of it (corr[t]) as in the walk.
__global__ void k_cyclic_ref_b(float* P, long long ts, int nt, const float* __restrict__ Ref, long long rts,
                               int rk, const double* __restrict__ corr, const int* __restrict__ cols, int ncols,
                               BLayout L)
{
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const int nk = L.nk;
    if (e >= (long long)ncols * nk * nt) return;
    const int k = 1 + (int)(e % nk), q = (int)((e / nk) % ncols), t = (int)(e / ((long long)nk * ncols));
    const int c = cols[q], sj = L.ni + 2;
    P[(long long)t * ts + L.at(c % sj, c / sj, k)] = Ref[(long long)t * rts + (long long)q * rk + k] - (float)corr[t];
}
// Then each row i = 2..IUB-1 whose two ends (j = 1, JUB) are boundary points
// copies the interior values next to the opposite end, and likewise each
// column j = 2..JUB-1 with i = 1, IUB, from the source column's KFloorZ up
// (clamped to the box, AD:2160-2215).  No copy reads a cell another copy
// writes (the row copies write j = 1, JUB and read j = 2, JUB-1 of rows
// 2..IUB-1; the column copies write i = 1, IUB), so one thread per (copy, k,
// tracer) keeps the reference's result.  Copy m: m < 2 (ni-2) rows (even m the
// j = 1 end), then columns.
__global__ void k_cyclic_copy_b(float* P, long long ts, int nt, const int* __restrict__ BP,
                                const int* __restrict__ KF, BLayout L)
{
    const int ni = L.ni, nj = L.nj, nk1 = L.nk + 1, sj = ni + 2;
    const long long nrow = 2LL * (ni > 2 ? ni - 2 : 0), ncol = 2LL * (nj > 2 ? nj - 2 : 0);
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= (nrow + ncol) * nk1 * nt) return;
    const int k = (int)(e % nk1);
    const long long m = (e / nk1) % (nrow + ncol);
    const int t = (int)(e / ((nrow + ncol) * nk1));
    int di, dj, si, sjj;                         // destination and source cells
    if (m < nrow) {
        const int i = 2 + (int)(m / 2);
        if (BP[i + sj] != 1 || BP[i + sj * nj] != 1) return;
        di = i; si = i;
        if (m % 2 == 0) { dj = 1; sjj = nj - 1; } else { dj = nj; sjj = 2; }
    } else {
        const int j = 2 + (int)((m - nrow) / 2);
        if (BP[1 + sj * j] != 1 || BP[ni + sj * j] != 1) return;
        dj = j; sjj = j;
        if ((m - nrow) % 2 == 0) { di = 1; si = ni - 1; } else { di = ni; si = 2; }
    }
    const int kf = KF[si + sj * sjj];
    if (k < (kf < 0 ? 0 : kf)) return;
    float* Pt = P + (long long)t * ts;
    Pt[L.at(di, dj, k)] = Pt[L.at(si, sjj, k)];
}

// NoAdvFlux / NoDifFlux folded into the flag bytes over the work box, where
// the reference zeroes the masked faces' coefficients: the advective bit of a
// west (south) face is cleared where NoFluxU (NoFluxV) == 1 and NoAdvFlux is
// on (AD:4434-4443, AD:4804-4813), its compute bit, which carries the
// diffusion, where NoDifFlux is on (AD:2496-2500, AD:2527-2531); F_NDW marks
// a bottom face with NoFluxW == 1 under NoDifFlux (AD:2741-2745), F_NAW one
// under NoAdvFlux on a column open at KUB, from KFloorZ up (AD:3004-3013).
// Both bits of each face are formed again from the masks first, so noAdv =
// noDif = 0 restores the unmasked flags (the TVD bits are left as they are).
__global__ void __launch_bounds__(kRowThreads)
k_noflux_flags(const int* __restrict__ OP, const int* __restrict__ CFU, const int* __restrict__ CFV,
               const int* __restrict__ NFU, const int* __restrict__ NFV, const int* __restrict__ NFW,
               const int* __restrict__ KF, int noAdv, int noDif, uint8_t* flag, uint8_t* fflag, BLayout L)
{
    const int NI = L.ni + 2;
    const long long sk = (long long)NI * (L.nj + 2);
    for_rows(L, 1, L.nk, [&](long long e, long long g, int i, int j, int k) {
        if (i < 1 || i > L.ni || j < 1 || j > L.nj) return;
        const bool op = OP[e] == 1;
        const bool cfu = CFU[e] == 1 && j != L.nj + 1, cfv = CFV[e] == 1 && i != L.ni + 1;
        uint8_t ff = fflag[g] & (uint8_t)(FU_TVDP | FU_TVDN | FV_TVDP | FV_TVDN);
        if (cfu) {
            if (!(noDif && NFU[e] == 1)) ff |= FU_ACT;
            if (op && OP[e - NI] == 1 && !(noAdv && NFU[e] == 1)) ff |= FU_ADV;
        }
        if (cfv) {
            if (!(noDif && NFV[e] == 1)) ff |= FV_ACT;
            if (op && OP[e - 1] == 1 && !(noAdv && NFV[e] == 1)) ff |= FV_ADV;
        }
        fflag[g] = ff;
        uint8_t fl = flag[g] & (uint8_t)~(F_NDW | F_NAW);
        if (noDif && NFW[e] == 1) fl |= F_NDW;
        if (noAdv && NFW[e] == 1) {
            const long long c = i + (long long)NI * j;
            const int kf = KF[c];
            if (OP[c + sk * L.nk] == 1 && k >= (kf < 0 ? 0 : kf)) fl |= F_NAW;
        }
        flag[g] = fl;
    });
}

// add the stored constant back: anomaly -> absolute values (water cells)
__global__ void k_unshift(float* P, const uint8_t* flag, double shift, long long n)
{
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
        if (flag[e] & F_WP) P[e] = (float)((double)P[e] + shift);
}

// per-column data and per-face 2-D constants
__global__ void k_pack_cols(const double* DUX, const double* DVY, const double* DZX, const double* DZY,
                            const int* KF, const int* BP, const int* WP, const int* OP, const int* CFW,
                            const int* SD, float4* fc, float* areaCol, int* kfloor,
                            uint8_t* cflag, BLayout L)
{
    const int NI = L.ni + 2, NJ = L.nj + 2;
    const long long sk = (long long)NI * NJ;
    const long long n = sk;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(e % NI), j = (int)(e / NI);
        const long long g = L.at2(i, j);
        auto d2 = [&](const double* a, int ii, int jj) -> double {
            ii = ii < 0 ? 0 : (ii > NI - 1 ? NI - 1 : ii);
            jj = jj < 0 ? 0 : (jj > NJ - 1 ? NJ - 1 : jj);
            return a[ii + (long long)NI * jj];
        };
        // Kx weights (Convert_Visc_Dif_Horizontal, AD:2487-2494) over the
        // distance between the centres (HorizontalDiffusionXX, AD:5185), and
        // the TVD slope ratio (du_dn + du_up) / (du_up + du_upup) of
        // ComputeAdvectionFace (FN:10785-10822) for either flow direction
        auto face = [&](double a, double b, double aa, double bb, double dz) -> float4 {
            const double rdz = dz != 0.0 ? 1.0 / dz : 0.0;
            const double s = a + b;
            float4 c;
            c.x = s != 0.0 ? (float)(a / s * rdz) : 0.f;            // weight of Visc(b), the cell's own
            c.y = s != 0.0 ? (float)(b / s * rdz) : 0.f;            // weight of Visc(a)
            c.z = (a + aa) != 0.0 ? (float)(s / (a + aa)) : 0.f;    // Q > 0: upwind a, upup aa
            c.w = (b + bb) != 0.0 ? (float)(s / (b + bb)) : 0.f;    // Q <= 0: upwind b, upup bb
            return c;
        };
        // west face of (i,j): a = (i, j-1), b = (i, j); du = DUX along j
        fc[g] = face(d2(DUX, i, j - 1), d2(DUX, i, j), d2(DUX, i, j - 2), d2(DUX, i, j + 1), d2(DZX, i, j - 1));
        // south face of (i,j): a = (i-1, j), b = (i, j); du = DVY along i
        fc[L.n2 + g] = face(d2(DVY, i - 1, j), d2(DVY, i, j), d2(DVY, i - 2, j), d2(DVY, i + 1, j),
                            d2(DZY, i - 1, j));
        areaCol[g] = (float)(DUX[e] * DVY[e]);
        kfloor[g] = KF[e];
        uint8_t c = 0;
        const bool interior = i >= 1 && i <= L.ni && j >= 1 && j <= L.nj;
        if (interior && WP[e + sk * L.nk] == 1) c |= C_SOLVE;
        if (interior && OP[e + sk * L.nk] == 1) c |= C_OPTOP;
        if (interior && CFW[e + sk * L.nk] == 1) c |= C_CFWTOP;
        if (interior && BP[e] == 1) c |= C_BP;
        if (interior && SD && SD[e] != 0) c |= C_SD;
        cflag[g] = c;
    }
}


// tracer: Fortran FP64 -> batched FP32 in both ping-pong buffers; cells below
// KFloor of solved columns hold null_real and row KUB+1 holds 0, which is what
// one reference step leaves there.
__global__ void __launch_bounds__(kRowThreads) k_pack_tracer(const double* src, float* A, float* B, const int* KF,
                                                           const int* WP, double shift, BLayout L)
{
    const int NI = L.ni + 2;
    const long long sk = (long long)NI * (L.nj + 2);
    for_rows(L, 0, L.nk + 2, [&](long long e, long long g, int i, int j, int k) {
        const long long c = i + (long long)NI * j;
        double v = src[e];
        const bool interior = i >= 1 && i <= L.ni && j >= 1 && j <= L.nj;
        if (interior && WP[c + sk * L.nk] == 1) {
            if (k == L.nk + 1) v = 0.0;
            else if (k >= 1 && k < KF[c]) v = MOHID_NULL_REAL_D;
        }
        if (WP[e] == 1) v -= shift;               // water cells hold the anomaly P - shift
        A[g] = (float)v;
        if (B) B[g] = (float)v;
    });
}

__global__ void __launch_bounds__(kRowThreads) k_unpack_tracer(const float* src, double* dst, const double* orig,
                                                             const int* WP, const int* KF, double shift0,
                                                             const double* corr, BLayout L)
{
    const double shift = shift0 + (corr ? *corr : 0.0);
    const int NI = L.ni + 2;
    const long long sk = (long long)NI * (L.nj + 2);
    for_rows(L, 0, L.nk + 2, [&](long long e, long long g, int i, int j, int k) {
        const long long c = i + (long long)NI * j;
        const bool interior = i >= 1 && i <= L.ni && j >= 1 && j <= L.nj;
        const bool solved = interior && WP[c + sk * L.nk] == 1 && k >= 1;
        if (solved) {
            if (k >= KF[c] && k <= L.nk) dst[e] = (double)src[g] + (WP[e] == 1 ? shift : 0.0);
            else if (k > L.nk) dst[e] = 0.0;
            else dst[e] = MOHID_NULL_REAL_D;
        } else {
            dst[e] = orig ? orig[e] : (double)src[g];
        }
    });
}

__global__ void k_absmax(const double* src, long long n, unsigned long long* out)
{
    double m = 0.0;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
        m = fmax(m, fabs(src[e]));
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, (unsigned long long)__double_as_longlong(m));
}

// Neumaier-compensated FP64 sum of V*P over water cells: per-thread compensated
// partial sums, exact-order block reduction, then one deterministic final pass.
__global__ void __launch_bounds__(kRowThreads) k_mass(const float* P, const double* V, const uint8_t* flag,
                                                    double shift0, const double* corr, BLayout L, double* partial)
{
    const double shift = shift0 + (corr ? *corr : 0.0);
    double s = 0.0, c = 0.0;
    for_rows(L, 1, L.nk, [&](long long f, long long g, int i, int j, int) {
        if (i >= 1 && i <= L.ni && j >= 1 && j <= L.nj && (flag[g] & F_WP))
            neu_add(s, c, V[f] * ((double)P[g] + shift));
    });
    const double S = block_neu(s, c);
    if (threadIdx.x == 0) {
        partial[2 * blockIdx.x] = S;
        partial[2 * blockIdx.x + 1] = 0.0;
    }
}

__global__ void k_mass_finish(const double* partial, int nb, double* out)
{
    double S, Z;
    warp_partials(partial, nb, S, Z);
    if (threadIdx.x == 0) *out = S;
}

// ------------------------------------------------------------------ mass fixer
// FP64 sums over water cells of the Fortran-layout arrays: V (P == null) or
// V * P.  Each thread sums its cells (a few dozen) in FP64; the threads' and
// blocks' sums are combined with Neumaier compensation in a fixed order.
__global__ void __launch_bounds__(kRowThreads) k_water_vsum(const double* V, const double* P, const int* WP,
                                                          BLayout L, double* partial)
{
    double s = 0.0;
    for_rows(L, 1, L.nk, [&](long long f, long long, int i, int j, int) {
        if (i >= 1 && i <= L.ni && j >= 1 && j <= L.nj && WP[f] == 1) s = P ? fma(V[f], P[f], s) : s + V[f];
    });
    const double S = block_neu(s, 0.0);
    if (threadIdx.x == 0) {
        partial[2 * blockIdx.x] = S;
        partial[2 * blockIdx.x + 1] = 0.0;
    }
}

// volume: mfix[0] = sum; load: target, constant, zero correction of tracer t
__global__ void k_fix_set(const double* partial, int nb, double* mfix, int mode, int t, int nt, double shift)
{
    double S, Z;
    warp_partials(partial, nb, S, Z);
    if (threadIdx.x != 0) return;
    if (mode == 0) {
        mfix[0] = S;
    } else {
        mfix[1 + t] = S;
        mfix[1 + nt + t] = shift;
        mfix[1 + 2 * nt + t] = 0.0;
        mfix[1 + 3 * nt + t] = 0.0;
    }
}

// One block per tracer: the tiles' sums of VolumeZ * stored value (each
// thread a strided share in FP64, the threads combined by a compensated tree in
// a fixed order), then correction += (target - mass) / volume, where mass = that
// sum + (constant + correction) * volume.  Adding the correction to every water
// cell (through the constant) leaves the step's result otherwise unchanged:
// the fixer only runs when the step maps constants onto themselves.  With open
// boundaries (obpart != null) the target first takes the step's boundary flux
//   phi = -(sum of WFOB * DT) * (constant + correction) - sum of WFOB * DT * value,
// the value being the stored inflow concentration where WFOB < 0 and the new
// stored value where WFOB >= 0 (obc_flux).  Without tile sums (mpart null:
// not the last step of a step call) only the target follows the flux; the
// correction, which the flux reads, stays as it is.  A tracer whose target was
// dropped (NaN) is left alone.
__device__ void fix_tracer(const double* mpart, int ntiles, int nt, int t, double* mfix, const double* obpart,
                           int nob)
{
    double s = 0.0;
    if (mpart)
        for (int q = threadIdx.x; q < ntiles; q += blockDim.x) s += mpart[(long long)t * ntiles + q];
    const double sum = block_neu(s, 0.0);
    double zs = 0.0, ws = 0.0;
    if (obpart) {
        double z = 0.0, w = 0.0;
        for (int q = threadIdx.x; q < nob; q += blockDim.x) {
            z += obpart[(long long)t * nob + q];
            w += obpart[(long long)nt * nob + q];
        }
        __syncthreads();                         // block_neu's shared words are reused
        zs = block_neu(z, 0.0);
        __syncthreads();
        ws = block_neu(w, 0.0);
    }
    if (threadIdx.x == 0) {
        const double W = mfix[0];
        double target = mfix[1 + t];
        if (W > 0.0 && !isnan(target)) {
            const double cnow = mfix[1 + nt + t] + mfix[1 + 2 * nt + t];
            if (obpart) {
                const double phi = -(ws * cnow) - zs;
                target += phi;
                mfix[1 + t] = target;
                mfix[1 + 3 * nt + t] += phi;
            }
            if (mpart) mfix[1 + 2 * nt + t] += (target - (sum + cnow * W)) / W;
        }
    }
}

// block t: tracer t of the batch
__global__ void __launch_bounds__(kRowThreads) k_fix_step(const double* mpart, int ntiles, int nt, double* mfix,
                                                         const double* obpart, int nob)
{
    fix_tracer(mpart, ntiles, nt, blockIdx.x, mfix, obpart, nob);
}

// block (b, t): tracer t of batch b (blocks past a batch's tracer count, and
// batches with neither tile sums nor a boundary flux this step, return)
__global__ void __launch_bounds__(kRowThreads) k_fix_step_many(const BatchArgs* As)
{
    const BatchArgs& a = As[blockIdx.x];
    if ((!a.mpart && !a.obpart) || (int)blockIdx.y >= a.ntAll) return;
    fix_tracer(a.mpart, a.ntiles, a.ntAll, blockIdx.y, a.mfix, a.obpart, a.nob);
}

// targets and boundary fluxes dropped
__global__ void k_fix_drop(double* mfix, int nt)
{
    const double nan = __longlong_as_double(0x7ff8000000000000LL);
    for (int t = threadIdx.x; t < nt; t += blockDim.x) {
        mfix[1 + t] = nan;
        mfix[1 + 3 * nt + t] = nan;
    }
}

// ------------------------------------------------------------------ open-boundary columns
__device__ __forceinline__ bool obc_column(uint8_t c)
{
    return (c & (C_SOLVE | C_BP)) == (C_SOLVE | C_BP);
}

// block b counts the boundary columns of its chunk [b * chunk, (b + 1) * chunk)
__global__ void __launch_bounds__(kRowThreads) k_obc_count(const uint8_t* __restrict__ cflag, long long n2,
                                                          long long chunk, int* cnt)
{
    __shared__ int wsum[kRowThreads / 32];
    const long long b0 = blockIdx.x * chunk, b1 = min(n2, b0 + chunk);
    int c = 0;
    for (long long e = b0 + threadIdx.x; e < b1; e += blockDim.x) c += obc_column(cflag[e]) ? 1 : 0;
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        int n = 0;
        for (int q = 0; q < kRowThreads / 32; ++q) n += wsum[q];
        cnt[blockIdx.x] = n;
    }
}

// block b writes its chunk's boundary columns, in order, after those of blocks 0 .. b-1
__global__ void __launch_bounds__(kRowThreads) k_obc_write(const uint8_t* __restrict__ cflag, long long n2,
                                                          long long chunk, const int* __restrict__ cnt, int* list)
{
    __shared__ int wsum[kRowThreads / 32];
    __shared__ int base;
    if (threadIdx.x == 0) {
        int o = 0;
        for (int q = 0; q < (int)blockIdx.x; ++q) o += cnt[q];
        base = o;
        if (blockIdx.x == gridDim.x - 1) list[0] = o + cnt[blockIdx.x];
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const long long b0 = blockIdx.x * chunk, b1 = min(n2, b0 + chunk);
    for (long long e0 = b0; e0 < b1; e0 += blockDim.x) {
        const long long e = e0 + threadIdx.x;
        const bool f = e < b1 && obc_column(cflag[e]);
        const unsigned m = __ballot_sync(0xffffffffu, f);
        if (lane == 0) wsum[w] = __popc(m);
        __syncthreads();
        int off = base;
        for (int q = 0; q < w; ++q) off += wsum[q];
        if (f) list[1 + off + __popc(m & ((1u << lane) - 1u))] = (int)e;
        __syncthreads();
        if (threadIdx.x == 0) {
            int n = 0;
            for (int q = 0; q < kRowThreads / 32; ++q) n += wsum[q];
            base += n;
        }
        __syncthreads();
    }
}

// new hydrodynamics: flag any cell whose VolumeZ differs (bit for bit) from the
// last pack's, and keep the new volumes for the next comparison
__global__ void k_vol_changed(const double* __restrict__ Vnew, double* __restrict__ Vprev, long long n,
                              unsigned* changed)
{
    bool c = false;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const double v = Vnew[e];
        if (!same_bits(v, Vprev[e])) { c = true; Vprev[e] = v; }
    }
    if (__any_sync(0xffffffffu, c) && (threadIdx.x & 31) == 0) *changed = 1u;
}

// FP16 storage scales: the largest magnitude of a field maps to 2^14, so that
// FP16 keeps 11 significant bits; scale[q] = absmax / 2^14, inv[q] = 1 / scale[q]
__global__ void k_scales(const double* absmax, int n, float* scale, float* inv)
{
    const int q = threadIdx.x;
    if (q >= n) return;
    const double m = absmax[q];
    const float sc = m > 0 ? (float)(m / 16384.0) : 1.0f;
    scale[q] = sc;
    inv[q] = 1.0f / sc;
}

inline unsigned blocks_for(long long n) { long long b = (n + 255) / 256; return (unsigned)(b > 65535 * 8 ? 65535 * 8 : (b < 1 ? 1 : b)); }

}  // namespace

cudaError_t pack_fields(const double* Qx, const double* Qy, const double* Qz, const double* V, const double* Vold,
                        const double* Vis, const double* Dif, const double* AU, const double* AV, const double* DZZ,
                        const int* WP, const int* OP, const int* LP, const int* CFU, const int* CFV, const int* CFW,
                        void* oQx, void* oQy, void* oQz, void* oVis, void* oDif, bool halfQ, bool halfK,
                        const float* dinv, float* oAU, float* oAV, float* orDZZ, float* oRV, float* oDVR,
                        float* oVhi, float* oVlo, uint8_t* oflag, uint8_t* offlag, unsigned* moving,
                        const BLayout& L, cudaStream_t s)
{
    PackIn in{Qx, Qy, Qz, V, Vold, Vis, Dif, AU, AV, DZZ, WP, OP, LP, CFU, CFV, CFW};
    PackOut out{oQx, oQy, oQz, oVis, oDif, dinv, halfQ ? 1 : 0, halfK ? 1 : 0,
                oAU, oAV, orDZZ, oRV, oDVR, oVhi, oVlo, oflag, offlag, moving};
    cudaError_t e = cudaMemsetAsync(moving, 0, sizeof(unsigned), s);
    if (e != cudaSuccess) return e;
    k_pack_fields<<<row_blocks(L, L.nk + 2), kRowThreads, 0, s>>>(in, out, L);
    return cudaGetLastError();
}
cudaError_t pack_state(const double* Qx, const double* Qy, const double* Qz, const double* V, const double* Vold,
                       const double* Vis, const double* Dif, const double* AU, const double* AV, const double* DZZ,
                       const int* WP, const int* OP, const int* LP, const int* CFU, const int* CFV, const int* CFW,
                       const int* BP2D, bool masks, void* oQx, void* oQy, void* oQz, void* oVis, void* oDif,
                       bool halfQ, bool halfK, const float* dinv, float* oAU, float* oAV, float* orDZZ, float* oRV,
                       float* oDVR, float* oVhi, float* oVlo, uint8_t* oflag, uint8_t* offlag, unsigned* moving,
                       double* Vprev, unsigned* vchanged, double* vpart, int nvblocks, double* mfix, double DT,
                       double tol, double* cont, const BLayout& L, cudaStream_t s)
{
    PackIn in{Qx, Qy, Qz, V, Vold, Vis, Dif, AU, AV, DZZ, WP, OP, LP, CFU, CFV, CFW};
    PackOut out{oQx, oQy, oQz, oVis, oDif, dinv, halfQ ? 1 : 0, halfK ? 1 : 0,
                oAU, oAV, orDZZ, oRV, oDVR, oVhi, oVlo, oflag, offlag, moving};
    FuseArgs f{Vprev, vchanged, vpart, BP2D, DT > 0.0 ? 1.0 / DT : 0.0, tol,
               reinterpret_cast<unsigned long long*>(cont)};
    cudaError_t e = cudaMemsetAsync(moving, 0, sizeof(unsigned), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(vchanged, 0, sizeof(unsigned), s);
    if (e == cudaSuccess && DT > 0.0) e = cudaMemsetAsync(cont, 0, sizeof(double), s);
    if (e != cudaSuccess) return e;
    const unsigned nb = (unsigned)nvblocks;
    if (masks) k_pack_state<true><<<nb, kRowThreads, 0, s>>>(in, out, L, f);
    else k_pack_state<false><<<nb, kRowThreads, 0, s>>>(in, out, L, f);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    k_fix_set<<<1, 32, 0, s>>>(vpart, nvblocks, mfix, 0, 0, 0, 0.0);
    return cudaGetLastError();
}
cudaError_t pack_columns(const double* DUX, const double* DVY, const double* DZX, const double* DZY,
                         const int* KFloor, const int* BP2D, const int* WP, const int* OP,
                         const int* CFW, const int* SD, float4* fc, float* areaCol,
                         int* kfloor, uint8_t* cflag, const BLayout& L, cudaStream_t s)
{
    k_pack_cols<<<blocks_for((long long)(L.ni + 2) * (L.nj + 2)), 256, 0, s>>>(
        DUX, DVY, DZX, DZY, KFloor, BP2D, WP, OP, CFW, SD, fc, areaCol, kfloor, cflag, L);
    return cudaGetLastError();
}
cudaError_t pack_tracer(const double* src, float* dA, float* dB, const int* KFloor, const int* WP,
                        double shift, const BLayout& L, cudaStream_t s)
{
    k_pack_tracer<<<row_blocks(L, L.nk + 2), kRowThreads, 0, s>>>(src, dA, dB, KFloor, WP, shift, L);
    return cudaGetLastError();
}
cudaError_t unpack_tracer(const float* src, double* dst, const double* orig, const int* WP,
                          const int* KFloor, double shift, const double* corr, const BLayout& L, cudaStream_t s)
{
    k_unpack_tracer<<<row_blocks(L, L.nk + 2), kRowThreads, 0, s>>>(src, dst, orig, WP, KFloor, shift, corr, L);
    return cudaGetLastError();
}
cudaError_t pack_shift_f32(const double* src, float* dst, const int* WP, double shift, const BLayout& L,
                           cudaStream_t s)
{
    k_pack_shift_f32<<<row_blocks(L, L.nk + 2), kRowThreads, 0, s>>>(src, dst, WP, shift, L);
    return cudaGetLastError();
}
cudaError_t continuity_residual(const double* Qx, const double* Qy, const double* Qz, const double* V,
                                const double* Vold, const int* OP, const int* CFU, const int* CFV,
                                const int* CFW, const int* BP2D, double DT, double tol, const BLayout& L,
                                double* out, cudaStream_t s)
{
    cudaError_t e = cudaMemsetAsync(out, 0, sizeof(double), s);
    if (e != cudaSuccess) return e;
    k_continuity<<<row_blocks(L, L.nk), kRowThreads, 0, s>>>(Qx, Qy, Qz, V, Vold, OP, CFU, CFV, CFW, BP2D, 1.0 / DT, tol,
                                                              L, reinterpret_cast<unsigned long long*>(out));
    return cudaGetLastError();
}
cudaError_t pack_ref(const double* src, const int* WP, const int* cols, int ncols, int ni, int nj, int nk,
                     double shift, float* dst, cudaStream_t s)
{
    const long long n = (long long)ncols * (nk + 2);
    if (n <= 0) return cudaSuccess;
    const long long sk = (long long)(ni + 2) * (nj + 2);
    k_pack_ref<<<blocks_for(n) > 4096 ? 4096 : blocks_for(n), 256, 0, s>>>(src, WP, cols, n, nk + 2, sk, shift, dst);
    return cudaGetLastError();
}
cudaError_t unshift_ref(float* R, const int* WP, const int* cols, int ncols, int ni, int nj, int nk, double shift,
                        cudaStream_t s)
{
    const long long n = (long long)ncols * (nk + 2);
    if (n <= 0) return cudaSuccess;
    const long long sk = (long long)(ni + 2) * (nj + 2);
    k_unshift_ref<<<blocks_for(n) > 4096 ? 4096 : blocks_for(n), 256, 0, s>>>(R, WP, cols, n, nk + 2, sk, shift);
    return cudaGetLastError();
}
cudaError_t ref_index(const int* cols, int ncols, int ni, const BLayout& L, int* idx, cudaStream_t s)
{
    cudaError_t e = cudaMemsetAsync(idx, 0xff, sizeof(int) * (size_t)L.n2, s);
    if (e != cudaSuccess || ncols <= 0) return e;
    k_ref_index<<<(ncols + 255) / 256, 256, 0, s>>>(cols, ncols, ni + 2, L, idx);
    return cudaGetLastError();
}
cudaError_t null_gradient_batched(float* P, long long ts, int nt, const uint8_t* flag, const int* cols, int ncols,
                                  const int* KFloor, const BLayout& L, cudaStream_t s)
{
    if (ncols <= 0 || nt <= 0) return cudaSuccess;
    const int n = (L.nk + 1) * nt;
    k_null_gradient_b<<<(n + 63) / 64, 64, 0, s>>>(P, ts, nt, flag, cols, ncols, KFloor, L);
    return cudaGetLastError();
}
cudaError_t cyclic_batched(float* P, long long ts, int nt, const float* Ref, long long rts, int rk,
                           const double* corr, const int* cols, int ncols, const int* BP, const int* KFloor,
                           const BLayout& L, cudaStream_t s)
{
    if (nt <= 0) return cudaSuccess;
    const long long n1 = (long long)ncols * L.nk * nt;
    if (n1 > 0) {
        k_cyclic_ref_b<<<(unsigned)((n1 + 255) / 256), 256, 0, s>>>(P, ts, nt, Ref, rts, rk, corr, cols, ncols, L);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    const long long lines = 2LL * (L.ni > 2 ? L.ni - 2 : 0) + 2LL * (L.nj > 2 ? L.nj - 2 : 0);
    const long long n2 = lines * (L.nk + 1) * nt;
    if (n2 <= 0) return cudaSuccess;
    k_cyclic_copy_b<<<(unsigned)((n2 + 255) / 256), 256, 0, s>>>(P, ts, nt, BP, KFloor, L);
    return cudaGetLastError();
}
cudaError_t noflux_flags(const int* OP, const int* CFU, const int* CFV, const int* NFU, const int* NFV,
                         const int* NFW, const int* KF, bool noAdv, bool noDif, uint8_t* flag, uint8_t* fflag,
                         const BLayout& L, cudaStream_t s)
{
    if (L.nk < 1) return cudaSuccess;
    if ((noAdv || noDif) && (!NFU || !NFV || !NFW)) return cudaErrorInvalidValue;
    k_noflux_flags<<<row_blocks(L, L.nk), kRowThreads, 0, s>>>(OP, CFU, CFV, NFU, NFV, NFW, KF, noAdv ? 1 : 0,
                                                                noDif ? 1 : 0, flag, fflag, L);
    return cudaGetLastError();
}
cudaError_t unshift(float* P, const uint8_t* flag, double shift, long long n, cudaStream_t s)
{
    k_unshift<<<blocks_for(n) > 8192 ? 8192 : blocks_for(n), 256, 0, s>>>(P, flag, shift, n);
    return cudaGetLastError();
}
cudaError_t water_mean(const double* src, const int* WP, const BLayout& L, double* partial, int nblocks,
                       double* out, cudaStream_t s)
{
    k_water_sum<<<nblocks, kRowThreads, 0, s>>>(src, WP, L, partial);
    k_water_mean<<<1, 32, 0, s>>>(partial, nblocks, out);
    return cudaGetLastError();
}
cudaError_t absmax_f64(const double* src, long long n, double* out, cudaStream_t s)
{
    cudaError_t e = cudaMemsetAsync(out, 0, sizeof(double), s);
    if (e != cudaSuccess) return e;
    k_absmax<<<blocks_for(n) > 4096 ? 4096 : blocks_for(n), 256, 0, s>>>(src, n, reinterpret_cast<unsigned long long*>(out));
    return cudaGetLastError();
}
cudaError_t mass_batched(const float* P, const double* V, const uint8_t* flag, double shift, const double* corr,
                         const BLayout& L, double* partial, int nblocks, cudaStream_t s)
{
    k_mass<<<nblocks, kRowThreads, 0, s>>>(P, V, flag, shift, corr, L, partial);
    return cudaGetLastError();
}
cudaError_t mass_finish(const double* partial, int nblocks, double* out, cudaStream_t s)
{
    k_mass_finish<<<1, 32, 0, s>>>(partial, nblocks, out);
    return cudaGetLastError();
}

cudaError_t water_volume(const double* V, const int* WP, const BLayout& L, double* partial, int nblocks,
                         double* mfix, cudaStream_t s)
{
    k_water_vsum<<<nblocks, kRowThreads, 0, s>>>(V, nullptr, WP, L, partial);
    k_fix_set<<<1, 32, 0, s>>>(partial, nblocks, mfix, 0, 0, 0, 0.0);
    return cudaGetLastError();
}
cudaError_t mass_fix_load(const double* P, const double* V, const int* WP, const BLayout& L, double* partial,
                          int nblocks, double shift, int t, int nt, double* mfix, cudaStream_t s)
{
    k_water_vsum<<<nblocks, kRowThreads, 0, s>>>(V, P, WP, L, partial);
    k_fix_set<<<1, 32, 0, s>>>(partial, nblocks, mfix, 1, t, nt, shift);
    return cudaGetLastError();
}
cudaError_t mass_fix_step(const double* mpart, int ntiles, int nt, double* mfix, const double* obpart, int nob,
                          cudaStream_t s)
{
    k_fix_step<<<nt, kRowThreads, 0, s>>>(mpart, ntiles, nt, mfix, obpart, nob);
    return cudaGetLastError();
}
cudaError_t mass_fix_drop(double* mfix, int nt, cudaStream_t s)
{
    k_fix_drop<<<1, 128, 0, s>>>(mfix, nt);
    return cudaGetLastError();
}
cudaError_t obc_columns(const uint8_t* cflag, const BLayout& L, int* cnt, int* list, cudaStream_t s)
{
    const long long chunk = (L.n2 + kObcBlocks - 1) / kObcBlocks;
    k_obc_count<<<kObcBlocks, kRowThreads, 0, s>>>(cflag, L.n2, chunk, cnt);
    k_obc_write<<<kObcBlocks, kRowThreads, 0, s>>>(cflag, L.n2, chunk, cnt, list);
    return cudaGetLastError();
}
cudaError_t mass_fix_step_many(const BatchArgs* As, int nb, int ntmax, cudaStream_t s)
{
    k_fix_step_many<<<dim3(nb, ntmax), kRowThreads, 0, s>>>(As);
    return cudaGetLastError();
}

cudaError_t vol_changed(const double* Vnew, double* Vprev, long long n, unsigned* changed, cudaStream_t s)
{
    cudaError_t e = cudaMemsetAsync(changed, 0, sizeof(unsigned), s);
    if (e != cudaSuccess) return e;
    k_vol_changed<<<blocks_for(n) > 4096 ? 4096 : blocks_for(n), 256, 0, s>>>(Vnew, Vprev, n, changed);
    return cudaGetLastError();
}
cudaError_t fp16_scales(const double* const* fields, int nf, long long n, double* absmax, float* scale, float* inv,
                        cudaStream_t s)
{
    for (int q = 0; q < nf; ++q) {
        cudaError_t e = absmax_f64(fields[q], n, absmax + q, s);
        if (e != cudaSuccess) return e;
    }
    k_scales<<<1, 32, 0, s>>>(absmax, nf, scale, inv);
    return cudaGetLastError();
}

}  // namespace mohid
