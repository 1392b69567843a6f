// batched_pack.cu -- conversions between the Fortran FP64 Size-box arrays and
// the batched layout, tracer anomaly bookkeeping, continuity check and the
// compensated mass budget of the batched form.
#include "batched.cuh"
#include "common.cuh"

namespace mohid {
namespace {

// ------------------------------------------------------------------ packing kernels
__global__ void k_pack_f32(const double* __restrict__ src, float* __restrict__ dst, BLayout L, int nz)
{
    const long long n = (long long)(L.ni + 2) * (L.nj + 2) * nz;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(e % (L.ni + 2));
        const int j = (int)((e / (L.ni + 2)) % (L.nj + 2));
        const int k = (int)(e / ((long long)(L.ni + 2) * (L.nj + 2)));
        dst[L.at(i, j, k)] = (float)src[e];
    }
}

__global__ void k_pack_recip(const double* __restrict__ src, float* __restrict__ dst, BLayout L)
{
    const long long n = (long long)(L.ni + 2) * (L.nj + 2) * (L.nk + 2);
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(e % (L.ni + 2));
        const int j = (int)((e / (L.ni + 2)) % (L.nj + 2));
        const int k = (int)(e / ((long long)(L.ni + 2) * (L.nj + 2)));
        dst[L.at(i, j, k)] = src[e] != 0.0 ? (float)(1.0 / src[e]) : 0.f;
    }
}

__global__ void k_pack_f16(const double* __restrict__ src, __half* __restrict__ dst, float inv, BLayout L)
{
    const long long n = (long long)(L.ni + 2) * (L.nj + 2) * (L.nk + 2);
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(e % (L.ni + 2));
        const int j = (int)((e / (L.ni + 2)) % (L.nj + 2));
        const int k = (int)(e / ((long long)(L.ni + 2) * (L.nj + 2)));
        dst[L.at(i, j, k)] = __float2half_rn((float)(src[e] * (double)inv));
    }
}

__global__ void k_pack_shift_f32(const double* __restrict__ src, float* __restrict__ dst,
                                 const int* __restrict__ WP, double shift, BLayout L)
{
    const long long n = (long long)(L.ni + 2) * (L.nj + 2) * (L.nk + 2);
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(e % (L.ni + 2));
        const int j = (int)((e / (L.ni + 2)) % (L.nj + 2));
        const int k = (int)(e / ((long long)(L.ni + 2) * (L.nj + 2)));
        dst[L.at(i, j, k)] = (float)(src[e] - (WP[e] == 1 ? shift : 0.0));
    }
}

// mean over water cells: per-block sums and counts, then one ordered final pass
// (deterministic, so the stored anomalies are reproducible bit for bit)
__global__ void k_water_sum(const double* src, const int* WP, long long n, double* partial)
{
    __shared__ double ss[256];
    __shared__ double sc[256];
    double s = 0.0, cnt = 0.0;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
        if (WP[e] == 1) { s += src[e]; cnt += 1.0; }
    ss[threadIdx.x] = s; sc[threadIdx.x] = cnt;
    __syncthreads();
    if (threadIdx.x == 0) {
        double S = 0.0, Cn = 0.0;
        for (int q = 0; q < (int)blockDim.x; ++q) { S += ss[q]; Cn += sc[q]; }
        partial[2 * blockIdx.x] = S;
        partial[2 * blockIdx.x + 1] = Cn;
    }
}

__global__ void k_water_mean(const double* partial, int nb, double* out)
{
    double S = 0.0, Cn = 0.0;
    for (int q = 0; q < nb; ++q) { S += partial[2 * q]; Cn += partial[2 * q + 1]; }
    *out = Cn > 0.0 ? S / Cn : 0.0;
}

// Largest relative continuity residual over open, non-boundary water cells,
// with the fluxes the step applies (Fortran-layout FP64 inputs):
//   R = Qx(w) - Qx(e) + Qy(s) - Qy(n) + Qz(k) - Qz(k+1) - (V - Vold)/DT
// over compute faces, relative to the sum of the magnitudes.  When it is at
// round-off level the step maps a constant field onto itself.
__global__ void k_continuity(const double* Qx, const double* Qy, const double* Qz, const double* V,
                             const double* Vold, const int* OP, const int* CFU, const int* CFV,
                             const int* CFW, const int* BP2D, double DT, int ni, int nj, int nk,
                             unsigned long long* out)
{
    const long long NI = ni + 2, NJ = nj + 2, sk = NI * NJ;
    const long long n = (long long)ni * nj * nk;
    double m = 0.0;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const int i = 1 + (int)(e % ni);
        const int j = 1 + (int)((e / ni) % nj);
        const int k = 1 + (int)(e / ((long long)ni * nj));
        const long long a = i + NI * j + sk * k, c2 = i + NI * j;
        if (OP[a] != 1 || BP2D[c2] == 1) continue;
        double r = 0.0, s = 0.0, f;
        f = CFU[a] == 1 ? Qx[a] : 0.0; r += f; s += fabs(f);
        f = CFU[a + NI] == 1 ? Qx[a + NI] : 0.0; r -= f; s += fabs(f);
        f = CFV[a] == 1 ? Qy[a] : 0.0; r += f; s += fabs(f);
        f = CFV[a + 1] == 1 ? Qy[a + 1] : 0.0; r -= f; s += fabs(f);
        f = CFW[a] == 1 ? Qz[a] : 0.0; r += f; s += fabs(f);
        f = (k < nk && CFW[a + sk] == 1) ? Qz[a + sk] : (k == nk ? Qz[a + sk] : 0.0); r -= f; s += fabs(f);
        f = (V[a] - Vold[a]) / DT; r -= f; s += fabs(f);
        const double rel = fabs(r) / (s + 1e-300);
        m = fmax(m, rel);
    }
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, (unsigned long long)__double_as_longlong(m));
}

// add the stored constant back: anomaly -> absolute values (water cells)
__global__ void k_unshift(float* P, const uint8_t* flag, double shift, long long n)
{
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
        if (flag[e] & F_WP) P[e] = (float)((double)P[e] + shift);
}

// relative volume change (V - Vold)/V formed in FP64, stored as FP32
__global__ void k_pack_dvr(const double* __restrict__ V, const double* __restrict__ Vo, float* __restrict__ dst,
                           BLayout L)
{
    const long long n = (long long)(L.ni + 2) * (L.nj + 2) * (L.nk + 2);
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(e % (L.ni + 2));
        const int j = (int)((e / (L.ni + 2)) % (L.nj + 2));
        const int k = (int)(e / ((long long)(L.ni + 2) * (L.nj + 2)));
        dst[L.at(i, j, k)] = V[e] != 0.0 ? (float)((V[e] - Vo[e]) / V[e]) : 0.f;
    }
}

__global__ void k_pack_f64(const double* __restrict__ src, double* __restrict__ dst, BLayout L)
{
    const long long n = (long long)(L.ni + 2) * (L.nj + 2) * (L.nk + 2);
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(e % (L.ni + 2));
        const int j = (int)((e / (L.ni + 2)) % (L.nj + 2));
        const int k = (int)(e / ((long long)(L.ni + 2) * (L.nj + 2)));
        dst[L.at(i, j, k)] = src[e];
    }
}

__global__ void k_pack_flags(const int* WP, const int* OP, const int* CFU, const int* CFV, const int* CFW,
                             const int* LP, uint8_t* dst, BLayout L)
{
    const long long n = (long long)(L.ni + 2) * (L.nj + 2) * (L.nk + 2);
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(e % (L.ni + 2));
        const int j = (int)((e / (L.ni + 2)) % (L.nj + 2));
        const int k = (int)(e / ((long long)(L.ni + 2) * (L.nj + 2)));
        uint8_t f = 0;
        if (WP[e] == 1) f |= F_WP;
        if (OP[e] == 1) f |= F_OP;
        if (CFU[e] == 1) f |= F_CFU;
        if (CFV[e] == 1) f |= F_CFV;
        if (CFW[e] == 1) f |= F_CFW;
        if (LP[e] == 1) f |= F_LP;
        // faces only inside the work box (the reference never applies the
        // faces on the j = JUB+1 / i = IUB+1 planes)
        if (j == L.nj + 1) f &= (uint8_t)~F_CFU;
        if (i == L.ni + 1) f &= (uint8_t)~F_CFV;
        dst[L.at(i, j, k)] = f;
    }
}

// face flag bits of every cell's west (U) and south (V) faces.  The bits restate
// the per-face conditions of ComputeAdvection1D_V2 (FN:10559: both cells open;
// NearBoundary when the cell upstream of the upwind cell is not open) and the
// compute-face masks, so the step reads one byte per face.  Faces on the
// j = JUB+1 / i = IUB+1 planes are never applied by the reference.
__global__ void k_pack_face_flags(const int* OP, const int* CFU, const int* CFV, uint8_t* dst, BLayout L)
{
    const int NI = L.ni + 2, NJ = L.nj + 2;
    const long long sk = (long long)NI * NJ;
    const long long n = sk * (L.nk + 2);
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(e % NI);
        const int j = (int)((e / NI) % NJ);
        const int k = (int)(e / sk);
        auto op = [&](int ii, int jj) -> bool {
            return ii >= 0 && ii < NI && jj >= 0 && jj < NJ && OP[ii + (long long)NI * jj + sk * k] == 1;
        };
        uint8_t f = 0;
        if (CFU[e] == 1 && j != L.nj + 1) {
            f |= FU_ACT;
            if (op(i, j - 1) && op(i, j)) f |= FU_ADV;
        }
        if (op(i, j - 2)) f |= FU_TVDP;
        if (op(i, j + 1)) f |= FU_TVDN;
        if (CFV[e] == 1 && i != L.ni + 1) {
            f |= FV_ACT;
            if (op(i - 1, j) && op(i, j)) f |= FV_ADV;
        }
        if (op(i - 2, j)) f |= FV_TVDP;
        if (op(i + 1, j)) f |= FV_TVDN;
        dst[L.at(i, j, k)] = f;
    }
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
__global__ void k_pack_tracer(const double* src, float* A, float* B, const int* KF, const int* WP,
                              double shift, BLayout L)
{
    const int NI = L.ni + 2, NJ = L.nj + 2;
    const long long sk = (long long)NI * NJ;
    const long long n = sk * (L.nk + 2);
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(e % NI);
        const int j = (int)((e / NI) % NJ);
        const int k = (int)(e / sk);
        const long long c = i + (long long)NI * j;
        double v = src[e];
        const bool interior = i >= 1 && i <= L.ni && j >= 1 && j <= L.nj;
        if (interior && WP[c + sk * L.nk] == 1) {
            if (k == L.nk + 1) v = 0.0;
            else if (k >= 1 && k < KF[c]) v = MOHID_NULL_REAL_D;
        }
        if (WP[e] == 1) v -= shift;               // water cells hold the anomaly P - shift
        const long long g = L.at(i, j, k);
        A[g] = (float)v;
        if (B) B[g] = (float)v;
    }
}

__global__ void k_unpack_tracer(const float* src, double* dst, const double* orig, const int* WP,
                                const int* KF, double shift, BLayout L)
{
    const int NI = L.ni + 2, NJ = L.nj + 2;
    const long long sk = (long long)NI * NJ;
    const long long n = sk * (L.nk + 2);
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(e % NI);
        const int j = (int)((e / NI) % NJ);
        const int k = (int)(e / sk);
        const long long c = i + (long long)NI * j;
        const bool interior = i >= 1 && i <= L.ni && j >= 1 && j <= L.nj;
        const bool solved = interior && WP[c + sk * L.nk] == 1 && k >= 1;
        if (solved) {
            if (k >= KF[c] && k <= L.nk) dst[e] = (double)src[L.at(i, j, k)] + (WP[e] == 1 ? shift : 0.0);
            else if (k > L.nk) dst[e] = 0.0;
            else dst[e] = MOHID_NULL_REAL_D;
        } else {
            dst[e] = orig ? orig[e] : (double)src[L.at(i, j, k)];
        }
    }
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
__device__ __forceinline__ void neu_add(double& s, double& c, double x)
{
    const double t = s + x;
    if (fabs(s) >= fabs(x)) c += (s - t) + x; else c += (x - t) + s;
    s = t;
}

__global__ void k_mass(const float* P, const double* V, const uint8_t* flag, double shift, BLayout L,
                       double* partial)
{
    __shared__ double ss[256], sc[256];
    double s = 0.0, c = 0.0;
    const long long n = (long long)L.ni * L.nj * L.nk;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const int i = 1 + (int)(e % L.ni);
        const int j = 1 + (int)((e / L.ni) % L.nj);
        const int k = 1 + (int)(e / ((long long)L.ni * L.nj));
        const long long g = L.at(i, j, k);
        const long long f = i + (long long)(L.ni + 2) * (j + (long long)(L.nj + 2) * k);
        if (flag[g] & F_WP) neu_add(s, c, V[f] * ((double)P[g] + shift));
    }
    ss[threadIdx.x] = s; sc[threadIdx.x] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        double S = 0.0, C = 0.0;
        for (int q = 0; q < (int)blockDim.x; ++q) { neu_add(S, C, ss[q]); C += sc[q]; }
        partial[2 * blockIdx.x] = S;
        partial[2 * blockIdx.x + 1] = C;
    }
}

__global__ void k_mass_finish(const double* partial, int nb, double* out)
{
    double S = 0.0, C = 0.0;
    for (int q = 0; q < nb; ++q) { neu_add(S, C, partial[2 * q]); C += partial[2 * q + 1]; }
    *out = S + C;
}

inline unsigned blocks_for(long long n) { long long b = (n + 255) / 256; return (unsigned)(b > 65535 * 8 ? 65535 * 8 : (b < 1 ? 1 : b)); }

}  // namespace

cudaError_t pack_f64_to_f32(const double* src, float* dst, const BLayout& L, int nz, cudaStream_t s)
{
    k_pack_f32<<<blocks_for((long long)(L.ni + 2) * (L.nj + 2) * nz), 256, 0, s>>>(src, dst, L, nz);
    return cudaGetLastError();
}
cudaError_t pack_recip_f32(const double* src, float* dst, const BLayout& L, cudaStream_t s)
{
    k_pack_recip<<<blocks_for((long long)(L.ni + 2) * (L.nj + 2) * (L.nk + 2)), 256, 0, s>>>(src, dst, L);
    return cudaGetLastError();
}
cudaError_t pack_f64_to_f16(const double* src, __half* dst, float inv, const BLayout& L, cudaStream_t s)
{
    k_pack_f16<<<blocks_for((long long)(L.ni + 2) * (L.nj + 2) * (L.nk + 2)), 256, 0, s>>>(src, dst, inv, L);
    return cudaGetLastError();
}
cudaError_t pack_dvr(const double* V, const double* Vold, float* dst, const BLayout& L, cudaStream_t s)
{
    k_pack_dvr<<<blocks_for((long long)(L.ni + 2) * (L.nj + 2) * (L.nk + 2)), 256, 0, s>>>(V, Vold, dst, L);
    return cudaGetLastError();
}
cudaError_t pack_f64_to_f64(const double* src, double* dst, const BLayout& L, cudaStream_t s)
{
    k_pack_f64<<<blocks_for((long long)(L.ni + 2) * (L.nj + 2) * (L.nk + 2)), 256, 0, s>>>(src, dst, L);
    return cudaGetLastError();
}
cudaError_t pack_flags(const int* WP, const int* OP, const int* CFU, const int* CFV, const int* CFW,
                       const int* LP, uint8_t* dst, const BLayout& L, cudaStream_t s)
{
    k_pack_flags<<<blocks_for((long long)(L.ni + 2) * (L.nj + 2) * (L.nk + 2)), 256, 0, s>>>(WP, OP, CFU, CFV, CFW, LP, dst, L);
    return cudaGetLastError();
}
cudaError_t pack_face_flags(const int* OP, const int* CFU, const int* CFV, uint8_t* dst, const BLayout& L,
                            cudaStream_t s)
{
    k_pack_face_flags<<<blocks_for((long long)(L.ni + 2) * (L.nj + 2) * (L.nk + 2)), 256, 0, s>>>(OP, CFU, CFV,
                                                                                                 dst, L);
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
    k_pack_tracer<<<blocks_for((long long)(L.ni + 2) * (L.nj + 2) * (L.nk + 2)), 256, 0, s>>>(src, dA, dB, KFloor, WP, shift, L);
    return cudaGetLastError();
}
cudaError_t unpack_tracer(const float* src, double* dst, const double* orig, const int* WP,
                          const int* KFloor, double shift, const BLayout& L, cudaStream_t s)
{
    k_unpack_tracer<<<blocks_for((long long)(L.ni + 2) * (L.nj + 2) * (L.nk + 2)), 256, 0, s>>>(src, dst, orig, WP, KFloor, shift, L);
    return cudaGetLastError();
}
cudaError_t pack_shift_f32(const double* src, float* dst, const int* WP, double shift, const BLayout& L,
                           cudaStream_t s)
{
    k_pack_shift_f32<<<blocks_for((long long)(L.ni + 2) * (L.nj + 2) * (L.nk + 2)), 256, 0, s>>>(src, dst, WP, shift, L);
    return cudaGetLastError();
}
cudaError_t continuity_residual(const double* Qx, const double* Qy, const double* Qz, const double* V,
                                const double* Vold, const int* OP, const int* CFU, const int* CFV,
                                const int* CFW, const int* BP2D, double DT, int ni, int nj, int nk,
                                double* out, cudaStream_t s)
{
    cudaError_t e = cudaMemsetAsync(out, 0, sizeof(double), s);
    if (e != cudaSuccess) return e;
    const long long n = (long long)ni * nj * nk;
    k_continuity<<<blocks_for(n) > 4096 ? 4096 : blocks_for(n), 256, 0, s>>>(
        Qx, Qy, Qz, V, Vold, OP, CFU, CFV, CFW, BP2D, DT, ni, nj, nk, reinterpret_cast<unsigned long long*>(out));
    return cudaGetLastError();
}
cudaError_t unshift(float* P, const uint8_t* flag, double shift, long long n, cudaStream_t s)
{
    k_unshift<<<blocks_for(n) > 8192 ? 8192 : blocks_for(n), 256, 0, s>>>(P, flag, shift, n);
    return cudaGetLastError();
}
cudaError_t water_mean(const double* src, const int* WP, long long n, double* partial, int nblocks,
                       double* out, cudaStream_t s)
{
    k_water_sum<<<nblocks, 256, 0, s>>>(src, WP, n, partial);
    k_water_mean<<<1, 1, 0, s>>>(partial, nblocks, out);
    return cudaGetLastError();
}
cudaError_t absmax_f64(const double* src, long long n, double* out, cudaStream_t s)
{
    cudaError_t e = cudaMemsetAsync(out, 0, sizeof(double), s);
    if (e != cudaSuccess) return e;
    k_absmax<<<blocks_for(n) > 4096 ? 4096 : blocks_for(n), 256, 0, s>>>(src, n, reinterpret_cast<unsigned long long*>(out));
    return cudaGetLastError();
}
cudaError_t mass_batched(const float* P, const double* V, const uint8_t* flag, double shift,
                         const BLayout& L, double* partial, int nblocks, cudaStream_t s)
{
    k_mass<<<nblocks, 256, 0, s>>>(P, V, flag, shift, L, partial);
    return cudaGetLastError();
}
cudaError_t mass_finish(const double* partial, int nblocks, double* out, cudaStream_t s)
{
    k_mass_finish<<<1, 1, 0, s>>>(partial, nblocks, out);
    return cudaGetLastError();
}

}  // namespace mohid
