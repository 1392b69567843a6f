// batched_f32.cu -- batched FP32 multi-tracer transport step.
//
// Same operator as the plain FP64 drop-in (ModuleAdvectionDiffusion's
// AdvectionDiffusion: VolumeVariation, explicit horizontal diffusion and
// advection with ComputeAdvectionFace coefficients, implicit vertical
// diffusion and upwind advection, MassConservation open boundaries, THOMASZ),
// re-organised for many tracers sharing one hydrodynamic state:
//
//  * a CTA owns a 32 x 8 tile of water columns and walks k upwards; each layer
//    of every tracer is staged in shared memory with a 2-cell halo;
//  * every horizontal face is evaluated once per layer: its tracer-independent
//    part (Courant number, upwind side, limiter weights, diffusive conductance)
//    once, then the tracer-dependent flux for each tracer; cells gather the
//    four face fluxes from shared memory;
//  * the vertical tridiagonal matrix does not depend on the tracer (upwind
//    vertical advection + diffusion, AD:2708-2784, AD:3066-3117), so each row
//    is factorised once (W, 1/pivot) and every tracer only runs
//    G = (TI - D*G_prev) / pivot and the back-substitution (THOMASZ,
//    FN:4026-4123); W lives in shared memory, G is parked in the output array;
//  * the volume ratio Vold/V is formed as 1 - (V - Vold)/V with the difference
//    taken in FP64 (thin layers make it cancel); everything else is FP32;
//  * rows below KFloor are never touched (they hold null_real, as after any
//    reference step), so a z-level column costs what it holds.
#include "batched.cuh"
#include "common.cuh"

namespace mohid {
namespace {

// Velocity storage: float, or half with a per-field scale (Q = scale * q).
template <typename QT> struct QLoad;
template <> struct QLoad<float> {
    __device__ static float get(const float* p, long long a, float) { return __ldg(p + a); }
};
template <> struct QLoad<__half> {
    __device__ static float get(const __half* p, long long a, float s) { return s * __half2float(p[a]); }
};

constexpr int TX = kTX, TY = kTY, NTH = TX * TY;
constexpr int PW = TX + 4, PH = TY + 4;     // tracer / flag tile with 2-cell halo
constexpr int VW = TX + 2, VH = TY + 2;     // halo-1 tiles

template <int NT>
struct Tiles {
    float P[NT][PH][PW];
    float V[VH][VW];
    float Vis[VH][VW];
    float QX[TY + 1][TX];     // west faces of cells (i0..i0+TX-1, j0..j0+TY)
    float AU[TY + 1][TX];
    float QY[TY][TX + 1];     // south faces of cells (i0..i0+TX, j0..j0+TY-1)
    float AV[TY][TX + 1];
    float FX[NT][TY + 1][TX];
    float FY[NT][TY][TX + 1];
    float CX[6][TY + 1][TX];
    float CY[6][TY][TX + 1];
    uint8_t F[PH][PW];
    int kmin;
};

template <int LIM>
__device__ __forceinline__ float limiter(float r, float pa, float pb, float p2, float pcr)
{
    // ComputeAdvectionFace limiters, FN:10823-10856
    if (LIM == 1) return fmaxf(0.f, fminf(1.f, r));
    if (LIM == 2) return r < 0.f ? 0.f : 2.f * r / (1.f + r);
    if (LIM == 3) return fmaxf(0.f, fminf(fminf(2.f, 2.f * r), (1.f + r) * 0.5f));
    if (LIM == 4) return fmaxf(fmaxf(0.f, fminf(1.f, 2.f * r)), fminf(r, 2.f));
    // PDM: pa, pb from |Cr|, p2 = 2/(1-Cr'), pcr = 2/Cr'
    return fmaxf(0.f, fminf(fminf(pa + pb * r, p2), r * pcr));
}

template <typename QT>
__device__ __forceinline__ float ldq(const void* p, long long a, float s)
{
    return QLoad<QT>::get(reinterpret_cast<const QT*>(p), a, s);
}

// One horizontal face: tracer-independent preparation, then the flux of each
// tracer into shared memory.  `a`/`b` are the lower/upper cells along the face
// normal in the P tile, `st` the tile stride along that normal, `va`/`vb` the
// same cells in the halo-1 tiles; q, area and the 2-D constants `cc` (stride
// cs) are the face's.
template <int NT, int METHOD, int LIM>
__device__ __forceinline__ void face_flux(Tiles<NT>& S, const BatchArgs& A, int ja, int ia, int jb, int ib,
                                          int dj, int di, int vja, int via, int vjb, int vib,
                                          bool act, float q, float area, const float* cc, int cs,
                                          float* out, int ostride)
{
    if (!act) {
        for (int t = 0; t < NT; ++t) out[t * ostride] = 0.f;
        return;
    }
    const uint8_t fa = S.F[ja][ia], fb = S.F[jb][ib];
    const bool adv = (fa & F_OP) && (fb & F_OP);
    const bool pos = q > 0.f;
    // diffusive conductance: Kx*Area/DZX (Convert_Visc_Dif_Horizontal AD:2487-2494)
    float K = A.schmidtH * (S.Vis[vjb][vib] * cc[0] + S.Vis[vja][via] * cc[cs]);
    if (A.nullDif && q == 0.f) K = 0.f;
    const float auxK = K * area * cc[2 * cs];
    float c = 0.f, gup = 0.f, gdn = 0.f, pa = 0.f, pb = 0.f, p2 = 0.f, pcr = 0.f;
    bool tvd = false;
    int juu = 0, iuu = 0;
    if (METHOD == 4 && adv) {
        juu = pos ? ja - dj : jb + dj;
        iuu = pos ? ia - di : ib + di;
        const bool nb = !(S.F[juu][iuu] & F_OP);
        if (!nb) {
            tvd = true;
            const float vup = pos ? S.V[vja][via] : S.V[vjb][vib];
            float Cr = q * A.DT / vup;
            gdn = cc[4 * cs];
            gup = pos ? cc[3 * cs] : cc[5 * cs];
            if (LIM == 5) {
                const float t6 = (1.f - 2.f * fabsf(Cr)) / 6.f;
                pa = 0.5f + t6;
                pb = 0.5f - t6;
                if (fabsf(Cr) < 1e-16f) Cr = 1e-16f;
                p2 = 2.f / (1.f - Cr);
                pcr = 2.f / Cr;
            }
            c = 0.5f * (1.f - Cr);
        }
    }
    for (int t = 0; t < NT; ++t) {
        const float Pa = S.P[t][ja][ia], Pb = S.P[t][jb][ib];
        float F = -auxK * (Pb - Pa);
        if (adv) {
            const float Pup = pos ? Pa : Pb, Pdn = pos ? Pb : Pa;
            float theta = 0.f;
            if (METHOD == 4 && tvd) {
                const float Puu = S.P[t][juu][iuu];
                float dC = (Pdn - Pup) * gdn;
                if (fabsf(dC) < 1e-16f) dC = dC >= 0.f ? 1e-16f : -1e-16f;
                const float r = __fdividef((Pup - Puu) * gup, dC);
                theta = limiter<LIM>(r, pa, pb, p2, pcr) * c;
            }
            F += q * (Pup + theta * (Pdn - Pup));
        }
        out[t * ostride] = F;
    }
}

template <int NT, int METHOD, int LIM, typename QT, typename KT>
__global__ void __launch_bounds__(NTH)
batched_kernel(const BatchArgs A)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Tiles<NT>& S = *reinterpret_cast<Tiles<NT>*>(smem_raw);
    float* Wcol = reinterpret_cast<float*>(smem_raw + ((sizeof(Tiles<NT>) + 15) / 16) * 16);

    const BLayout& L = A.L;
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TX + tx;
    const int i0 = 1 + blockIdx.x * TX, j0 = 1 + blockIdx.y * TY;
    const int i = i0 + tx, j = j0 + ty;
    const bool inside = i <= L.ni && j <= L.nj;
    const long long c2 = L.at2(i, j);
    const uint8_t cf = inside ? A.cflag[c2] : 0;
    const bool solve = cf & C_SOLVE;
    const int kb = solve ? A.kfloor[c2] : L.nk + 1;

    if (tid == 0) S.kmin = L.nk + 1;
    // 2-D face constants of this tile
    for (int e = tid; e < (TY + 1) * TX; e += NTH) {
        const int a = e / TX, b = e % TX;
        const long long g = L.at2(i0 + b, j0 + a);
        for (int q = 0; q < 6; ++q) S.CX[q][a][b] = A.fx[q * L.n2 + g];
    }
    for (int e = tid; e < TY * (TX + 1); e += NTH) {
        const int a = e / (TX + 1), b = e % (TX + 1);
        const long long g = L.at2(i0 + b, j0 + a);
        for (int q = 0; q < 6; ++q) S.CY[q][a][b] = A.fy[q * L.n2 + g];
    }
    __syncthreads();
    if (solve) atomicMin(&S.kmin, kb);
    __syncthreads();
    const int kmin = S.kmin;
    if (kmin > L.nk) return;                       // no water column in this tile

    const float DT = A.DT;
    const float areaCol = solve ? A.areaCol[c2] : 0.f;
    const bool sd = cf & C_SD, opTop = cf & C_OPTOP, cfwTop = cf & C_CFWTOP, bp = cf & C_BP;
    const bool horiz = !A.vertical1D;

    // own-column sliding window
    float qz = 0.f, dv = 0.f, dzzm = 1.f;
    uint8_t flm = 0;                               // flag of layer k-1
    if (solve) {
        const long long a = L.at(i, j, kb);
        qz = ldq<QT>(A.Qz, a, A.qsz);
        dv = ldq<KT>(A.DiffV, a, A.ksv);
        dzzm = A.DZZ[a - L.sl];
        flm = A.flag[a - L.sl];
    }
    float Gp[NT];
    for (int t = 0; t < NT; ++t) Gp[t] = 0.f;
    float Wp = 0.f;
    unsigned bad = 0;

    for (int k = kmin; k <= L.nk; ++k) {
        __syncthreads();
        // ---- stage layer k
        for (int e = tid; e < PH * PW; e += NTH) {
            const int a = e / PW, b = e % PW;
            const long long g = L.at(i0 - 2 + b, j0 - 2 + a, k);
            S.F[a][b] = A.flag[g];
            for (int t = 0; t < NT; ++t) S.P[t][a][b] = A.Pin[t * A.ts + g];
        }
        for (int e = tid; e < VH * VW; e += NTH) {
            const int a = e / VW, b = e % VW;
            const long long g = L.at(i0 - 1 + b, j0 - 1 + a, k);
            S.V[a][b] = (float)A.V[g];
            S.Vis[a][b] = ldq<KT>(A.ViscH, g, A.ksh);
        }
        if (horiz) {
            for (int e = tid; e < (TY + 1) * TX; e += NTH) {
                const int a = e / TX, b = e % TX;
                const long long g = L.at(i0 + b, j0 + a, k);
                S.QX[a][b] = ldq<QT>(A.Qx, g, A.qsx);
                S.AU[a][b] = A.AreaU[g];
            }
            for (int e = tid; e < TY * (TX + 1); e += NTH) {
                const int a = e / (TX + 1), b = e % (TX + 1);
                const long long g = L.at(i0 + b, j0 + a, k);
                S.QY[a][b] = ldq<QT>(A.Qy, g, A.qsy);
                S.AV[a][b] = A.AreaV[g];
            }
        }
        __syncthreads();

        // ---- faces owned by this thread (west, south; tile edges also east, north)
        const int jj = ty + 2, ii = tx + 2, vj = ty + 1, vi = tx + 1;
        if (horiz) {
            // west face of (i,j): a = (i, j-1), b = (i, j)
            face_flux<NT, METHOD, LIM>(S, A, jj - 1, ii, jj, ii, 1, 0, vj - 1, vi, vj, vi,
                                       (S.F[jj][ii] & F_CFU) != 0, S.QX[ty][tx], S.AU[ty][tx],
                                       &S.CX[0][ty][tx], (TY + 1) * TX, &S.FX[0][ty][tx], (TY + 1) * TX);
            if (ty == TY - 1)
                face_flux<NT, METHOD, LIM>(S, A, jj, ii, jj + 1, ii, 1, 0, vj, vi, vj + 1, vi,
                                           (S.F[jj + 1][ii] & F_CFU) != 0, S.QX[ty + 1][tx],
                                           S.AU[ty + 1][tx], &S.CX[0][ty + 1][tx], (TY + 1) * TX,
                                           &S.FX[0][ty + 1][tx], (TY + 1) * TX);
            const bool yy = !A.xzflow;
            face_flux<NT, METHOD, LIM>(S, A, jj, ii - 1, jj, ii, 0, 1, vj, vi - 1, vj, vi,
                                       yy && (S.F[jj][ii] & F_CFV) != 0, S.QY[ty][tx], S.AV[ty][tx],
                                       &S.CY[0][ty][tx], TY * (TX + 1), &S.FY[0][ty][tx], TY * (TX + 1));
            if (tx == TX - 1)
                face_flux<NT, METHOD, LIM>(S, A, jj, ii, jj, ii + 1, 0, 1, vj, vi, vj, vi + 1,
                                           yy && (S.F[jj][ii + 1] & F_CFV) != 0, S.QY[ty][tx + 1],
                                           S.AV[ty][tx + 1], &S.CY[0][ty][tx + 1], TY * (TX + 1),
                                           &S.FY[0][ty][tx + 1], TY * (TX + 1));
        }
        __syncthreads();

        if (!solve || k < kb) continue;
        // ---- row k of column (i,j): tracer-independent matrix
        const long long a = L.at(i, j, k);
        const uint8_t fl = S.F[jj][ii];
        const uint8_t flp = (k < L.nk) ? A.flag[a + L.sl] : 0;
        const double Vd = A.V[a], Vod = A.Vold[a];
        const float Vk = (float)Vd;
        const float dtv = DT / Vk;
        const float qzp = ldq<QT>(A.Qz, a + L.sl, A.qsz);
        const float dvp = (k < L.nk) ? ldq<KT>(A.DiffV, a + L.sl, A.ksv) : 0.f;
        const float dzz = A.DZZ[a];
        const bool open = fl & F_OP;
        // VolumeVariation: TI = P*Vold/V = P*(1 - (V-Vold)/V), E(KUB) surface term
        const float ratio = open ? 1.f - (float)(Vd - Vod) / Vk : 1.f;
        float E = 1.f, D = 0.f, Fc = 0.f;
        if (open && k == L.nk) E = 1.f + dtv * qzp;
        if (L.nk > 1) {
            if ((fl & F_CFW) && !sd) {                       // VerticalDiffusion, face k
                float kz = A.coefV * dv + A.backV;
                if (A.nullDif && qz == 0.f) kz = 0.f;
                const float aux2 = kz * areaCol / dzzm * dtv;
                D -= aux2; E += aux2;
            }
            if ((flp & F_CFW) && !sd) {                      // face k+1
                float kz = A.coefV * dvp + A.backV;
                if (A.nullDif && qzp == 0.f) kz = 0.f;
                const float aux1 = kz * areaCol / dzz * dtv;
                E += aux1; Fc -= aux1;
            }
            if (!A.vertical1D && cfwTop) {                   // VerticalAdvection, upwind, implicit
                if (k >= kb + 1 && opTop && (flm & F_OP) && open) {
                    D -= (qz > 0.f ? qz : 0.f) * dtv;
                    E -= (qz > 0.f ? 0.f : qz) * dtv;
                }
                if (k + 1 <= L.nk && opTop && open && (flp & F_OP)) {
                    E += (qzp > 0.f ? qzp : 0.f) * dtv;
                    Fc += (qzp > 0.f ? 0.f : qzp) * dtv;
                }
            }
        }
        // open boundary (MassConservation): net flux through the exterior faces
        float wfob = 0.f;
        const bool obc = bp && A.Ref && open;
        if (obc) {
            const double hz = (double)(((fl & F_CFU) ? S.QX[ty][tx] : 0.f) -
                                       ((S.F[jj + 1][ii] & F_CFU) ? S.QX[ty + 1][tx] : 0.f) +
                                       ((fl & F_CFV) ? S.QY[ty][tx] : 0.f) -
                                       ((S.F[jj][ii + 1] & F_CFV) ? S.QY[ty][tx + 1] : 0.f) +
                                       ((fl & F_CFW) ? qz : 0.f) - ((flp & F_CFW) ? qzp : 0.f));
            wfob = (float)(hz - (Vd - Vod) / (double)DT);
            if (wfob >= 0.f) E += wfob * dtv;
        }
        // THOMASZ factorisation of row k
        const float aux = E + D * Wp;
        float inv;
        if (aux != 0.f) inv = 1.f / aux; else { inv = 0.f; bad |= MOHID_DEV_ZERO_PIVOT; }
        const float W = -Fc * inv;
        Wcol[k * NTH + tid] = W;
        Wp = W;
        for (int t = 0; t < NT; ++t) {
            const float P = S.P[t][jj][ii];
            float TI = P * ratio;
            if (horiz) TI += dtv * (S.FX[t][ty][tx] - S.FX[t][ty + 1][tx] + S.FY[t][ty][tx] - S.FY[t][ty][tx + 1]);
            if (obc && wfob < 0.f) {
                const float ext = P * (1.f - A.tdec) + A.Ref[t * A.ts + a] * A.tdec;
                TI -= wfob * ext * dtv;
            }
            const float G = (TI - D * Gp[t]) * inv;
            Gp[t] = G;
            A.Pout[t * A.ts + a] = G;
        }
        // slide the column window
        qz = qzp; dv = dvp; dzzm = dzz; flm = fl;
    }

    // ---- back-substitution (row KUB+1 solves to 0)
    if (solve) {
        for (int t = 0; t < NT; ++t) {
            float x = 0.f;
            float* Po = A.Pout + t * A.ts;
            for (int k = L.nk; k >= kb; --k) {
                const long long a = L.at(i, j, k);
                x = Wcol[k * NTH + tid] * x + Po[a];
                Po[a] = x;
                if (!isfinite(x)) bad |= MOHID_DEV_NONFINITE;
            }
        }
    }
    if (bad) atomicOr(A.status, bad);
}

template <int NT, int METHOD, int LIM, typename QT, typename KT>
cudaError_t launch_t(const BatchArgs& a, cudaStream_t s)
{
    const size_t tiles = ((sizeof(Tiles<NT>) + 15) / 16) * 16;
    const size_t smem = tiles + sizeof(float) * (size_t)(a.L.nk + 2) * NTH;
    auto kern = batched_kernel<NT, METHOD, LIM, QT, KT>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    dim3 grd((unsigned)((a.L.ni + TX - 1) / TX), (unsigned)((a.L.nj + TY - 1) / TY));
    kern<<<grd, dim3(TX, TY), smem, s>>>(a);
    return cudaGetLastError();
}

template <int NT, typename QT, typename KT>
cudaError_t launch_m(const BatchArgs& a, int method, int limiter, cudaStream_t s)
{
    if (method == 1) return launch_t<NT, 1, 0, QT, KT>(a, s);
    switch (limiter) {
    case 1: return launch_t<NT, 4, 1, QT, KT>(a, s);
    case 2: return launch_t<NT, 4, 2, QT, KT>(a, s);
    case 3: return launch_t<NT, 4, 3, QT, KT>(a, s);
    case 4: return launch_t<NT, 4, 4, QT, KT>(a, s);
    default: return launch_t<NT, 4, 5, QT, KT>(a, s);
    }
}

template <int NT>
cudaError_t launch_n(const BatchArgs& a, int method, int limiter, bool halfQ, bool halfK, cudaStream_t s)
{
    if (halfQ && halfK) return launch_m<NT, __half, __half>(a, method, limiter, s);
    if (halfQ) return launch_m<NT, __half, float>(a, method, limiter, s);
    return launch_m<NT, float, float>(a, method, limiter, s);
}

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

// per-column data and per-face 2-D constants
__global__ void k_pack_cols(const double* DUX, const double* DVY, const double* DZX, const double* DZY,
                            const int* KF, const int* BP, const int* WP, const int* OP, const int* CFW,
                            const int* SD, float* fx, float* fy, float* areaCol, int* kfloor,
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
        // west face of (i,j): a = (i, j-1), b = (i, j); du = DUX along j
        {
            const double ua = d2(DUX, i, j - 1), ub = d2(DUX, i, j);
            const double uaa = d2(DUX, i, j - 2), ubb = d2(DUX, i, j + 1);
            fx[0 * L.n2 + g] = (float)(ua / (ub + ua));       // weight of Visc(b)
            fx[1 * L.n2 + g] = (float)(ub / (ub + ua));       // weight of Visc(a)
            fx[2 * L.n2 + g] = (float)(1.0 / d2(DZX, i, j - 1));
            fx[3 * L.n2 + g] = (float)(1.0 / (ua + uaa));
            fx[4 * L.n2 + g] = (float)(1.0 / (ub + ua));
            fx[5 * L.n2 + g] = (float)(1.0 / (ub + ubb));
        }
        {
            const double va = d2(DVY, i - 1, j), vb = d2(DVY, i, j);
            const double vaa = d2(DVY, i - 2, j), vbb = d2(DVY, i + 1, j);
            fy[0 * L.n2 + g] = (float)(va / (vb + va));
            fy[1 * L.n2 + g] = (float)(vb / (vb + va));
            fy[2 * L.n2 + g] = (float)(1.0 / d2(DZY, i - 1, j));
            fy[3 * L.n2 + g] = (float)(1.0 / (va + vaa));
            fy[4 * L.n2 + g] = (float)(1.0 / (vb + va));
            fy[5 * L.n2 + g] = (float)(1.0 / (vb + vbb));
        }
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
        if (flag[g] & F_WP) neu_add(s, c, V[g] * ((double)P[g] + shift));
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

cudaError_t launch_batched(const BatchArgs& a, int method, int limiter, bool halfQ, bool halfK,
                           cudaStream_t s)
{
    if (a.nt == 4) return launch_n<4>(a, method, limiter, halfQ, halfK, s);
    if (a.nt == 2) return launch_n<2>(a, method, limiter, halfQ, halfK, s);
    if (a.nt == 1) return launch_n<1>(a, method, limiter, halfQ, halfK, s);
    return cudaErrorInvalidValue;
}

cudaError_t pack_f64_to_f32(const double* src, float* dst, const BLayout& L, int nz, cudaStream_t s)
{
    k_pack_f32<<<blocks_for((long long)(L.ni + 2) * (L.nj + 2) * nz), 256, 0, s>>>(src, dst, L, nz);
    return cudaGetLastError();
}
cudaError_t pack_f64_to_f16(const double* src, __half* dst, float inv, const BLayout& L, cudaStream_t s)
{
    k_pack_f16<<<blocks_for((long long)(L.ni + 2) * (L.nj + 2) * (L.nk + 2)), 256, 0, s>>>(src, dst, inv, L);
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
cudaError_t pack_columns(const double* DUX, const double* DVY, const double* DZX, const double* DZY,
                         const int* KFloor, const int* BP2D, const int* WP, const int* OP,
                         const int* CFW, const int* SD, float* fx, float* fy, float* areaCol,
                         int* kfloor, uint8_t* cflag, const BLayout& L, cudaStream_t s)
{
    k_pack_cols<<<blocks_for((long long)(L.ni + 2) * (L.nj + 2)), 256, 0, s>>>(
        DUX, DVY, DZX, DZY, KFloor, BP2D, WP, OP, CFW, SD, fx, fy, areaCol, kfloor, cflag, L);
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
