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
struct Stage {                // one layer of the tile, staged from global memory
    float P[NT][PH][PW];
    float V[VH][VW];
    float Vis[VH][VW];
    float QX[TY + 1][TX];     // west faces of cells (i0..i0+TX-1, j0..j0+TY)
    float AU[TY + 1][TX];
    float QY[TY][TX + 1];     // south faces of cells (i0..i0+TX, j0..j0+TY-1)
    float AV[TY][TX + 1];
    uint8_t F[PH][PW];
};

template <int NT>
struct Tiles {
    Stage<NT> st[2];          // double buffer: layer k+1 is staged while k is solved
    float FX[NT][TY + 1][TX];
    float FY[NT][TY][TX + 1];
    float CX[6][TY + 1][TX];
    float CY[6][TY][TX + 1];
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

// A face of the tile, fixed for the whole walk: pb is the P/F-tile index of its
// upper cell b (lower cell a = pb - st), vb the V-tile index of b (a = vb - vst),
// fi the index in the face arrays (QX/AU/CX/FX for west faces, QY/AV/CY/FY for
// south faces).
struct FaceRef {
    int pb, vb, fi;
    bool west, valid;
};

// One face at one layer: tracer-independent preparation (upwind side, Courant
// number, limiter weights, diffusive conductance), then the flux of every
// tracer, F = q*P_up + (q*theta + kd)*(P_dn - P_up), into shared memory.
// The reference's face coefficients: ComputeAdvectionFace FN:10702-10894
// (first-order upwind, P2_TVD limiters), the diffusive flux of
// HorizontalDiffusionXX/YY AD:5185-5196 with Kx from AD:2487-2494.
template <int NT, int METHOD, int LIM>
__device__ __forceinline__ void face_flux(const Stage<NT>& T, float* FX, float* FY, const float* CX,
                                          const float* CY, const BatchArgs& A, const FaceRef& f)
{
    constexpr int NWF = (TY + 1) * TX, NSF = TY * (TX + 1);
    const int st = f.west ? PW : 1, vst = f.west ? VW : 1;
    const int cs = f.west ? NWF : NSF;
    const float* cc = (f.west ? CX : CY) + f.fi;
    float* out = (f.west ? FX : FY) + f.fi;
    const int pa = f.pb - st;
    const uint8_t* Fl = &T.F[0][0];
    const uint8_t fb = Fl[f.pb], fa = Fl[pa];
    const bool act = f.west ? (fb & F_CFU) && !A.vertical1D : (fb & F_CFV) && !A.vertical1D && !A.xzflow;
    const float q = f.west ? (&T.QX[0][0])[f.fi] : (&T.QY[0][0])[f.fi];
    const float area = f.west ? (&T.AU[0][0])[f.fi] : (&T.AV[0][0])[f.fi];
    const bool adv = act && (fa & F_OP) && (fb & F_OP);
    const bool pos = q > 0.f;
    // diffusive conductance Kx*Area/DZX; F_dif = -auxK*(Pb - Pa) = kd*(Pdn - Pup)
    float K = A.schmidtH * ((&T.Vis[0][0])[f.vb] * cc[0] + (&T.Vis[0][0])[f.vb - vst] * cc[cs]);
    if (A.nullDif && q == 0.f) K = 0.f;
    const float auxK = act ? K * area * cc[2 * cs] : 0.f;
    const float kd = pos ? -auxK : auxK;
    const float qv = adv ? q : 0.f;
    const int iup = pos ? pa : f.pb, idn = pos ? f.pb : pa;
    int iuu = iup;
    float c = 0.f, gup = 0.f, gdn = 0.f, pa5 = 0.f, pb5 = 0.f, p2 = 0.f, pcr = 0.f;
    bool tvd = false;
    if (METHOD == 4 && adv) {
        iuu = pos ? pa - st : f.pb + st;
        if (Fl[iuu] & F_OP) {                      // not near a boundary
            tvd = true;
            const float vup = (&T.V[0][0])[pos ? f.vb - vst : f.vb];
            float Cr = __fdividef(q * A.DT, vup);
            gdn = cc[4 * cs];
            gup = pos ? cc[3 * cs] : cc[5 * cs];
            if (LIM == 5) {
                const float t6 = (1.f - 2.f * fabsf(Cr)) / 6.f;
                pa5 = 0.5f + t6;
                pb5 = 0.5f - t6;
                if (fabsf(Cr) < 1e-16f) Cr = 1e-16f;
                p2 = 2.f / (1.f - Cr);
                pcr = 2.f / Cr;
            }
            c = 0.5f * (1.f - Cr);
        }
    }
#pragma unroll
    for (int t = 0; t < NT; ++t) {
        const float* Pt = &T.P[t][0][0];
        const float Pup = Pt[iup], Pdn = Pt[idn];
        const float dd = Pdn - Pup;
        float coef = kd;
        if (METHOD == 4) {
            const float du = Pup - Pt[iuu];
            float dC = dd * gdn;
            if (fabsf(dC) < 1e-16f) dC = copysignf(1e-16f, dC);
            const float r = du * gup * __frcp_rn(dC);
            const float th = tvd ? limiter<LIM>(r, pa5, pb5, p2, pcr) * c : 0.f;
            coef = fmaf(qv, th, kd);
        }
        out[t * cs] = fmaf(coef, dd, qv * Pup);
    }
}

// Staging slots: every thread moves up to two elements of each layer tile;
// their shared-memory index and layer-0 global offset are fixed for the walk.
struct Slot2 {
    int s[2];
    long long g[2];
    bool v[2];
};

template <int NT, int METHOD, int LIM, typename QT, typename KT>
__global__ void __launch_bounds__(NTH, 2)
batched_kernel(const BatchArgs A)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Tiles<NT>& S = *reinterpret_cast<Tiles<NT>*>(smem_raw);
    float* Wcol = reinterpret_cast<float*>(smem_raw + ((sizeof(Tiles<NT>) + 15) / 16) * 16);
    constexpr int NWF = (TY + 1) * TX, NSF = TY * (TX + 1);

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
    for (int e = tid; e < NWF; e += NTH) {
        const int a = e / TX, b = e % TX;
        const long long g = L.at2(i0 + b, j0 + a);
        for (int q = 0; q < 6; ++q) S.CX[q][a][b] = A.fx[q * L.n2 + g];
    }
    for (int e = tid; e < NSF; e += NTH) {
        const int a = e / (TX + 1), b = e % (TX + 1);
        const long long g = L.at2(i0 + b, j0 + a);
        for (int q = 0; q < 6; ++q) S.CY[q][a][b] = A.fy[q * L.n2 + g];
    }
    __syncthreads();
    if (solve) atomicMin(&S.kmin, kb);
    __syncthreads();
    const int kmin = S.kmin;
    if (kmin > L.nk) return;                       // no water column in this tile

    const bool horiz = !A.vertical1D;
    // ---- this thread's faces for the whole walk (west faces, then south faces)
    FaceRef fr[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        const int f = tid + q * NTH;
        fr[q].valid = horiz && f < NWF + NSF;
        if (f < NWF) {
            const int a = f / TX, b = f % TX;
            fr[q].west = true;
            fr[q].pb = (a + 2) * PW + b + 2;
            fr[q].vb = (a + 1) * VW + b + 1;
            fr[q].fi = a * TX + b;
        } else {
            const int g = f - NWF, a = g / (TX + 1), b = g % (TX + 1);
            fr[q].west = false;
            fr[q].pb = (a + 2) * PW + b + 2;
            fr[q].vb = (a + 1) * VW + b + 1;
            fr[q].fi = fr[q].valid ? a * (TX + 1) + b : 0;
        }
    }
    // ---- staging slots (P and flags: halo 2; V, Visc: halo 1; faces)
    Slot2 sp, sv, sx, sy;
#pragma unroll
    for (int q = 0; q < 2; ++q) {
        int e = tid + q * NTH;
        sp.v[q] = e < PH * PW;
        sp.s[q] = sp.v[q] ? e : 0;
        sp.g[q] = sp.v[q] ? L.at(i0 - 2 + e % PW, j0 - 2 + e / PW, 0) : 0;
        sv.v[q] = e < VH * VW;
        sv.s[q] = sv.v[q] ? e : 0;
        sv.g[q] = sv.v[q] ? L.at(i0 - 1 + e % VW, j0 - 1 + e / VW, 0) : 0;
        sx.v[q] = horiz && e < NWF;
        sx.s[q] = sx.v[q] ? e : 0;
        sx.g[q] = sx.v[q] ? L.at(i0 + e % TX, j0 + e / TX, 0) : 0;
        sy.v[q] = horiz && e < NSF;
        sy.s[q] = sy.v[q] ? e : 0;
        sy.g[q] = sy.v[q] ? L.at(i0 + e % (TX + 1), j0 + e / (TX + 1), 0) : 0;
    }
    float rP[NT][2], rV[2], rVis[2], rQX[2], rAU[2], rQY[2], rAV[2];
    uint8_t rF[2];
    auto fetch = [&](int k) {
        const long long ko = (long long)k * L.sl;
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            if (sp.v[q]) {
                rF[q] = A.flag[sp.g[q] + ko];
#pragma unroll
                for (int t = 0; t < NT; ++t) rP[t][q] = __ldg(A.Pin + t * A.ts + sp.g[q] + ko);
            }
            if (sv.v[q]) {
                rV[q] = (float)__ldg(A.V + sv.g[q] + ko);
                rVis[q] = ldq<KT>(A.ViscH, sv.g[q] + ko, A.ksh);
            }
            if (sx.v[q]) {
                rQX[q] = ldq<QT>(A.Qx, sx.g[q] + ko, A.qsx);
                rAU[q] = __ldg(A.AreaU + sx.g[q] + ko);
            }
            if (sy.v[q]) {
                rQY[q] = ldq<QT>(A.Qy, sy.g[q] + ko, A.qsy);
                rAV[q] = __ldg(A.AreaV + sy.g[q] + ko);
            }
        }
    };
    auto stage = [&](Stage<NT>& T) {
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            if (sp.v[q]) {
                (&T.F[0][0])[sp.s[q]] = rF[q];
#pragma unroll
                for (int t = 0; t < NT; ++t) (&T.P[t][0][0])[sp.s[q]] = rP[t][q];
            }
            if (sv.v[q]) {
                (&T.V[0][0])[sv.s[q]] = rV[q];
                (&T.Vis[0][0])[sv.s[q]] = rVis[q];
            }
            if (sx.v[q]) {
                (&T.QX[0][0])[sx.s[q]] = rQX[q];
                (&T.AU[0][0])[sx.s[q]] = rAU[q];
            }
            if (sy.v[q]) {
                (&T.QY[0][0])[sy.s[q]] = rQY[q];
                (&T.AV[0][0])[sy.s[q]] = rAV[q];
            }
        }
    };

    const float DT = A.DT;
    const float areaCol = solve ? A.areaCol[c2] : 0.f;
    const bool sd = cf & C_SD, opTop = cf & C_OPTOP, cfwTop = cf & C_CFWTOP, bp = cf & C_BP;

    // own-column window: values of rows k-1 / k slide, the next row is prefetched
    float qz = 0.f, dv = 0.f, dzzm = 1.f;
    uint8_t flm = 0;
    double nV = 1.0, nVo = 1.0;
    float nQz = 0.f, nDv = 0.f, nDzz = 1.f;
    uint8_t nFl = 0;
    const long long cb = L.at(i, j, 0);
    auto fetch_col = [&](int k) {                  // values first needed by row k
        const long long a = cb + (long long)k * L.sl;
        nV = __ldg(A.V + a);
        nVo = __ldg(A.Vold + a);
        nQz = ldq<QT>(A.Qz, a + L.sl, A.qsz);
        nDv = (k < L.nk) ? ldq<KT>(A.DiffV, a + L.sl, A.ksv) : 0.f;
        nDzz = __ldg(A.DZZ + a);
        nFl = (k < L.nk) ? A.flag[a + L.sl] : 0;
    };
    if (solve) {
        const long long a = cb + (long long)kb * L.sl;
        qz = ldq<QT>(A.Qz, a, A.qsz);
        dv = ldq<KT>(A.DiffV, a, A.ksv);
        dzzm = __ldg(A.DZZ + a - L.sl);
        flm = A.flag[a - L.sl];
        fetch_col(kb);
    }
    float Gp[NT];
#pragma unroll
    for (int t = 0; t < NT; ++t) Gp[t] = 0.f;
    float Wp = 0.f;
    unsigned bad = 0;
    const int jj = ty + 2, ii = tx + 2;
    const int fw = ty * TX + tx, fs = ty * (TX + 1) + tx;

    fetch(kmin);
    stage(S.st[kmin & 1]);
    if (kmin < L.nk) fetch(kmin + 1);
    for (int k = kmin; k <= L.nk; ++k) {
        Stage<NT>& T = S.st[k & 1];
        __syncthreads();                           // layer k staged; previous layer's rows done
        const bool active = solve && k >= kb;
        const double Vd = nV, Vod = nVo;
        const float qzp = nQz, dvp = nDv, dzz = nDzz;
        const uint8_t flp = nFl;
        if (active && k < L.nk) fetch_col(k + 1);

        // ---- the tile's faces at layer k
#pragma unroll
        for (int q = 0; q < 3; ++q)
            if (fr[q].valid)
                face_flux<NT, METHOD, LIM>(T, &S.FX[0][0][0], &S.FY[0][0][0], &S.CX[0][0][0],
                                           &S.CY[0][0][0], A, fr[q]);
        // stage layer k+1 into the other buffer (its readers finished before
        // the barrier above) and start fetching layer k+2
        if (k < L.nk) {
            stage(S.st[(k + 1) & 1]);
            if (k + 1 < L.nk) fetch(k + 2);
        }
        __syncthreads();                           // face fluxes of layer k complete

        if (!active) continue;
        // ---- row k of column (i,j): tracer-independent matrix
        const long long a = cb + (long long)k * L.sl;
        const uint8_t fl = T.F[jj][ii];
        const float Vk = (float)Vd;
        const float dtv = DT / Vk;
        const bool open = fl & F_OP;
        // VolumeVariation: TI = P*Vold/V = P*(1 - (V-Vold)/V), E(KUB) surface term
        const float ratio = open ? 1.f - (float)(Vd - Vod) / Vk : 1.f;
        float E = 1.f, D = 0.f, Fc = 0.f;
        if (open && k == L.nk) E = 1.f + dtv * qzp;
        if (L.nk > 1) {
            if ((fl & F_CFW) && !sd) {                       // VerticalDiffusion, face k
                float kz = A.coefV * dv + A.backV;
                if (A.nullDif && qz == 0.f) kz = 0.f;
                const float aux2 = kz * areaCol * dzzm * dtv;     // dzzm holds 1/DZZ(k-1)
                D -= aux2; E += aux2;
            }
            if ((flp & F_CFW) && !sd) {                      // face k+1
                float kz = A.coefV * dvp + A.backV;
                if (A.nullDif && qzp == 0.f) kz = 0.f;
                const float aux1 = kz * areaCol * dzz * dtv;      // dzz holds 1/DZZ(k)
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
            const double hz = (double)(((fl & F_CFU) ? T.QX[ty][tx] : 0.f) -
                                       ((T.F[jj + 1][ii] & F_CFU) ? T.QX[ty + 1][tx] : 0.f) +
                                       ((fl & F_CFV) ? T.QY[ty][tx] : 0.f) -
                                       ((T.F[jj][ii + 1] & F_CFV) ? T.QY[ty][tx + 1] : 0.f) +
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
#pragma unroll
        for (int t = 0; t < NT; ++t) {
            const float P = T.P[t][jj][ii];
            float TI = P * ratio;
            if (horiz) {
                const float* fx = &S.FX[t][0][0];
                const float* fy = &S.FY[t][0][0];
                TI += dtv * ((fx[fw] - fx[fw + TX]) + (fy[fs] - fy[fs + 1]));
            }
            if (obc && wfob < 0.f) {
                const float ext = P * (1.f - A.tdec) + A.Ref[t * A.ts + a] * A.tdec;
                TI -= wfob * ext * dtv;
            }
            const float G = (TI - D * Gp[t]) * inv;
            Gp[t] = G;
            A.Pout[t * A.ts + a] = G;
        }
        qz = qzp; dv = dvp; dzzm = dzz; flm = fl;
    }

    // ---- back-substitution (row KUB+1 solves to 0), G loads issued 8 rows at a time
    if (solve) {
#pragma unroll 1
        for (int t = 0; t < NT; ++t) {
            float x = 0.f;
            float* Po = A.Pout + t * A.ts + cb;
            for (int k = L.nk; k >= kb; k -= 8) {
                float g[8];
#pragma unroll
                for (int q = 0; q < 8; ++q)
                    if (k - q >= kb) g[q] = __ldcg(Po + (long long)(k - q) * L.sl);
#pragma unroll
                for (int q = 0; q < 8; ++q)
                    if (k - q >= kb) {
                        x = Wcol[(k - q) * NTH + tid] * x + g[q];
                        Po[(long long)(k - q) * L.sl] = x;
                        if (!isfinite(x)) bad |= MOHID_DEV_NONFINITE;
                    }
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
