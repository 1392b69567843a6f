// batched_tile.cuh -- the k-walk of one 32 x 8 tile of the batched FP32
// multi-tracer transport step, shared by the single-domain launch and the
// ensemble launch (many domains in one persistent grid).
//
// Same operator as the plain FP64 drop-in (ModuleAdvectionDiffusion's
// AdvectionDiffusion: VolumeVariation, explicit horizontal diffusion and
// advection with ComputeAdvectionFace coefficients, implicit vertical
// diffusion and upwind advection, MassConservation open boundaries, THOMASZ),
// re-organised for many tracers sharing one hydrodynamic state:
//
//  * a CTA owns a 32 x 8 tile of water columns and walks k upwards.  Each
//    layer's fields (all tracers of the launch with a 2-cell halo, face flags,
//    1/V, viscosity, face transports and areas, and the own-column values of
//    the layer above) arrive in shared memory as tiled bulk-tensor copies
//    (TMA), double-buffered on two mbarriers: layer k+1 streams in while layer
//    k is solved, and the last warp to finish layer k refills its buffer with
//    layer k+2.  One barrier per layer separates the face fluxes (double
//    buffered by layer parity) from the cells that gather them;
//  * every horizontal face is evaluated once per layer: its tracer-independent
//    part (Courant number, upwind side, diffusive conductance) once, then the
//    flux of each tracer, with the TVD limiter in a division-free form;
//  * the vertical tridiagonal matrix does not depend on the tracer (upwind
//    vertical advection + diffusion, AD:2708-2784, AD:3066-3117), so each row
//    is factorised once (W, 1/pivot) and every tracer only runs
//    G = (TI - D*G_prev) / pivot and the back-substitution (THOMASZ,
//    FN:4026-4123); W goes to a per-cell scratch array and G into the output
//    array, both read back from L2 by the same thread on the way down;
//  * the volume ratio Vold/V is applied as 1 - (V - Vold)/V, the relative
//    change (and 1/V) being formed in FP64 when the volumes are packed; the
//    kernel itself runs no FP64 arithmetic outside open-boundary cells, which
//    GB300 issues at a small fraction of the FP32 rate;
//  * rows below KFloor are never touched (they hold null_real, as after any
//    reference step), so a z-level column costs what it holds.
//
// Every wait on an mbarrier is bounded; a stage that never arrives makes the
// whole CTA set MOHID_DEV_TIMEOUT and return.
#pragma once
#include <type_traits>

#include "batched.cuh"
#include "common.cuh"

namespace mohid {
namespace tile {


constexpr int TX = kTX;
// a tile is TX = 32 cells along i (the lanes of a warp) by TY rows along j
// (one warp each): NTH threads, NWF west faces and NSF south faces
template <int TY> struct TileGeom {
    static constexpr int NTH = TX * TY;
    static constexpr int NWF = (TY + 1) * TX, NSF = TY * (TX + 1);
};

// ---- TMA stage layout -------------------------------------------------------
// Box origins sit on 16-byte boundaries of the batched layout (x = i + 31):
// the tracer and 1/V tiles start 4 cells before i0, the viscosity tile 4 (FP32)
// or 8 (FP16) cells before; face, face-flag and own-cell tiles start at i0.
constexpr int PBX = 40, FBX = 48, VBX = 40, OWN = 32, AVX = 36;
template <typename T> struct Box;
template <> struct Box<float> { static constexpr int visX = 40, visOff = 4, qyX = 36; };
template <> struct Box<__half> { static constexpr int visX = 48, visOff = 8, qyX = 40; };

constexpr int al128(int b) { return (b + 127) / 128 * 128; }

template <int NT, typename QT, typename KT, int TY>
struct StageLayout {
    static constexpr int qyX = Box<QT>::qyX, visX = Box<KT>::visX;
    static constexpr int bP = NT * (TY + 4) * PBX * 4;
    static constexpr int bF = (TY + 1) * FBX;
    static constexpr int bV = (TY + 2) * VBX * 4;
    static constexpr int bVis = (TY + 2) * visX * (int)sizeof(KT);
    static constexpr int bQX = (TY + 1) * TX * (int)sizeof(QT);
    static constexpr int bAU = (TY + 1) * TX * 4;
    static constexpr int bQY = TY * qyX * (int)sizeof(QT);
    static constexpr int bAV = TY * AVX * 4;
    static constexpr int bVo = TY * OWN * 4;
    static constexpr int bQz = TY * OWN * (int)sizeof(QT);
    static constexpr int bDv = TY * OWN * (int)sizeof(KT);
    static constexpr int bDz = TY * OWN * 4;
    static constexpr int bFn = TY * OWN;
    static constexpr int oP = 0;
    static constexpr int oF = oP + al128(bP);
    static constexpr int oV = oF + al128(bF);
    static constexpr int oVis = oV + al128(bV);
    static constexpr int oQX = oVis + al128(bVis);
    static constexpr int oAU = oQX + al128(bQX);
    static constexpr int oQY = oAU + al128(bAU);
    static constexpr int oAV = oQY + al128(bQY);
    static constexpr int oVo = oAV + al128(bAV);
    static constexpr int oQz = oVo + al128(bVo);
    static constexpr int oDv = oQz + al128(bQz);
    static constexpr int oDz = oDv + al128(bDv);
    static constexpr int oFn = oDz + al128(bDz);
    static constexpr int size = oFn + al128(bFn);
    static constexpr unsigned tx_bytes =
        bP + bF + bV + bVis + bQX + bAU + bQY + bAV + bVo + bQz + bDv + bDz + bFn;
};

template <int NT, typename QT, typename KT, int TY>
struct Smem {
    using SL = StageLayout<NT, QT, KT, TY>;
    static constexpr int NTH = TileGeom<TY>::NTH, NWF = TileGeom<TY>::NWF, NSF = TileGeom<TY>::NSF;
    static constexpr int oStage0 = 0;
    static constexpr int oStage1 = SL::size;
    // face fluxes, double-buffered by layer parity: [FX | FY] x 2
    static constexpr int FXYStride = al128(NT * NWF * 4) + al128(NT * NSF * 4);
    static constexpr int oFX = 2 * SL::size;
    static constexpr int oFY = oFX + al128(NT * NWF * 4);
    static constexpr int oCX = oFX + 2 * FXYStride;        // face constants (west, south faces)
    static constexpr int oCY = oCX + al128(NWF * 16);
    static constexpr int oRed = oCY + al128(NSF * 16);      // the mass fixer's per-warp sums
    static constexpr int oBar = oRed + al128(TY * NT * 2 * 4);
    static constexpr int oEnd = oBar + 128;
    static constexpr int oDis = oEnd;                       // a row's discharge sources, per thread
    // dis: the discharge instantiation, which also holds oDis
    static size_t bytes(int, bool dis = false) { return (size_t)(dis ? oDis + al128(NTH * NT * 4) : oEnd); }
};

// ---- PTX helpers: mbarrier and bulk tensor copies ---------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// bounded wait: gives up after `limit` polls
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint32_t limit)
{
    for (uint32_t it = 0; it < limit; ++it)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}
__device__ __forceinline__ void tma3(void* dst, const CUtensorMap* map, int x, int y, int z, uint64_t* bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
        ::"r"(smem_u32(dst)), "l"(map), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ void tma4(void* dst, const CUtensorMap* map, int x, int y, int z, int w, uint64_t* bar)
{
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], [%6];"
        ::"r"(smem_u32(dst)), "l"(map), "r"(x), "r"(y), "r"(z), "r"(w), "r"(smem_u32(bar))
        : "memory");
}
// L2 eviction priorities: the THOMASZ scratch (W, G) written on the way up and
// read once on the way down is kept in L2 ahead of the streamed layer inputs
__device__ __forceinline__ uint64_t l2_policy_evict_last()
{
    uint64_t p;
    asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
    return p;
}
__device__ __forceinline__ uint64_t l2_policy_evict_first()
{
    uint64_t p;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
    return p;
}
// (volatile asm keeps these in program order among themselves; the scratch is
// only ever read back by the thread that wrote it, after a data dependence)
__device__ __forceinline__ void st_l2hint(float* a, float v, uint64_t pol)
{
    asm volatile("st.global.L2::cache_hint.f32 [%0], %1, %2;" ::"l"(a), "f"(v), "l"(pol));
}
__device__ __forceinline__ float ld_l2hint(const float* a, uint64_t pol)
{
    float v;
    asm volatile("ld.global.cg.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(v) : "l"(a), "l"(pol));
    return v;
}

constexpr uint32_t kWaitLimit = 1u << 24;

// fetch-add on a shared-memory counter with acquire-release semantics at CTA scope
__device__ __forceinline__ unsigned atom_add_acq_rel_cta(unsigned* p, unsigned v)
{
    unsigned old;
    asm volatile("atom.acq_rel.cta.shared::cta.add.u32 %0, [%1], %2;"
                 : "=r"(old) : "r"(smem_u32(p)), "r"(v) : "memory");
    return old;
}

// psi(r) * d for r = n / d, psi one of the ComputeAdvectionFace limiters
// (FN:10823-10856).  Each min/max of psi(r) is multiplied through by |d|, so
// with a = |d| and b = n * sign(d) no division is needed (VanLeer keeps one);
// d = 0 gives 0, as the reference's theta * 0.
// PDM: pa, pb from |Cr|, p2 = 2/(1-Cr), pcr = 2/Cr.
template <int LIM>
__device__ __forceinline__ float limited_slope(float n, float d, float pa, float pb, float p2, float pcr)
{
    const unsigned sd = __float_as_uint(d) & 0x80000000u;
    const float a = fabsf(d);
    const float b = __uint_as_float(__float_as_uint(n) ^ sd);
    float v;
    if (LIM == 1) v = fmaxf(0.f, fminf(a, b));                                          // MinMod
    else if (LIM == 2) v = b > 0.f ? __fdividef(2.f * a * b, a + b) : 0.f;             // VanLeer
    else if (LIM == 3) v = fmaxf(0.f, fminf(fminf(2.f * a, 2.f * b), 0.5f * (a + b))); // MUSCL
    else if (LIM == 4) v = fmaxf(fmaxf(0.f, fminf(a, 2.f * b)), fminf(b, 2.f * a));    // SuperBee
    else v = fmaxf(0.f, fminf(fminf(fmaf(pb, b, pa * a), p2 * a), pcr * b));          // PDM
    return __uint_as_float(__float_as_uint(v) | sd);
}

template <typename T> __device__ __forceinline__ float tofl(T v, float s);
template <> __device__ __forceinline__ float tofl<float>(float v, float) { return v; }
template <> __device__ __forceinline__ float tofl<__half>(__half v, float s) { return s * __half2float(v); }

template <typename T>
__device__ __forceinline__ float ldg_as(const void* p, long long a, float s)
{
    return tofl<T>(reinterpret_cast<const T*>(p)[a], s);
}

// Net water flux out of a MassConservation open-boundary cell through its
// exterior faces (AD:5680-5742, FluxAtOpenBoundary): the transports into the
// cell through its west, south and bottom faces less those out through east,
// north and top (faces that are not compute faces count zero), less the
// volume change rate (V - Vold) / DT = dvr / (rV * DT).  The face sum is
// formed in FP32 with rounded adds, which are never contracted, so the step
// and the mass fixer's boundary budget get the same value.
__device__ __forceinline__ float obc_wfob(float qw, float qe, float qs, float qn, float qb, float qt, float dvr,
                                          float rV, float DT)
{
    const float h = __fsub_rn(__fadd_rn(__fsub_rn(__fadd_rn(__fsub_rn(qw, qe), qs), qn), qb), qt);
    return (float)((double)h - (double)dvr / ((double)rV * (double)DT));
}

// THOMASZ scratch of the walk, per cell of the batched layout: W in its own
// plane (A.W) and G of the launch's tracers together (A.G, NT floats per
// cell), so that a row's scratch is one scalar and one vector store on the
// way up and the same two loads on the way down.  The lines are discarded
// from L2 once read (they are dead), so they are never written back.
template <int NT> struct GVec;
template <> struct GVec<1> {
    static __device__ __forceinline__ void st(float* a, const float* g, uint64_t pol)
    {
        asm volatile("st.global.L2::cache_hint.f32 [%0], %1, %2;" ::"l"(a), "f"(g[0]), "l"(pol));
    }
    static __device__ __forceinline__ void ld(const float* a, float* g, uint64_t pol)
    {
        asm volatile("ld.global.cg.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(g[0]) : "l"(a), "l"(pol));
    }
};
template <> struct GVec<2> {
    static __device__ __forceinline__ void st(float* a, const float* g, uint64_t pol)
    {
        asm volatile("st.global.L2::cache_hint.v2.f32 [%0], {%1, %2}, %3;" ::"l"(a), "f"(g[0]), "f"(g[1]), "l"(pol));
    }
    static __device__ __forceinline__ void ld(const float* a, float* g, uint64_t pol)
    {
        asm volatile("ld.global.cg.L2::cache_hint.v2.f32 {%0, %1}, [%2], %3;"
                     : "=f"(g[0]), "=f"(g[1]) : "l"(a), "l"(pol));
    }
};
template <> struct GVec<4> {
    static __device__ __forceinline__ void st(float* a, const float* g, uint64_t pol)
    {
        asm volatile("st.global.L2::cache_hint.v4.f32 [%0], {%1, %2, %3, %4}, %5;" ::"l"(a), "f"(g[0]), "f"(g[1]),
                     "f"(g[2]), "f"(g[3]), "l"(pol));
    }
    static __device__ __forceinline__ void ld(const float* a, float* g, uint64_t pol)
    {
        asm volatile("ld.global.cg.L2::cache_hint.v4.f32 {%0, %1, %2, %3}, [%4], %5;"
                     : "=f"(g[0]), "=f"(g[1]), "=f"(g[2]), "=f"(g[3]) : "l"(a), "l"(pol));
    }
};
template <> struct GVec<8> {
    static __device__ __forceinline__ void st(float* a, const float* g, uint64_t pol)
    {
        GVec<4>::st(a, g, pol);
        GVec<4>::st(a + 4, g + 4, pol);
    }
    static __device__ __forceinline__ void ld(const float* a, float* g, uint64_t pol)
    {
        GVec<4>::ld(a, g, pol);
        GVec<4>::ld(a + 4, g + 4, pol);
    }
};

template <> struct GVec<10> {                     // 40 B per cell: 8-byte aligned pairs
    static __device__ __forceinline__ void st(float* a, const float* g, uint64_t pol)
    {
#pragma unroll
        for (int q = 0; q < 5; ++q) GVec<2>::st(a + 2 * q, g + 2 * q, pol);
    }
    static __device__ __forceinline__ void ld(const float* a, float* g, uint64_t pol)
    {
#pragma unroll
        for (int q = 0; q < 5; ++q) GVec<2>::ld(a + 2 * q, g + 2 * q, pol);
    }
};

// the 128-byte L2 line at a holds only dead data: drop it without a write-back
__device__ __forceinline__ void l2_discard(const void* a)
{
    asm volatile("discard.global.L2 [%0], 128;" ::"l"(a) : "memory");
}

// One face of the tile at one layer.  WEST: the face between the cells at P
// offsets pb - PBX and pb (j - 1 and j); otherwise between pb - 1 and pb (i - 1
// and i).  The offsets into the stage (elements): pb into the tracer tile, vb
// into 1/V, visb into Visc_H, qo / ao into the face transports and areas, fo
// into the face-flag bytes; out: the face's flux slot (tracer stride cs).  cf:
// the face's constants (Visc weights with Schmidt and 1/DZ folded in, TVD
// slope ratios).  Tracer-independent part first (upwind side, Courant number,
// diffusive conductance), then for every tracer
// F = q*P_up + kd*(P_dn - P_up) + q*c*psi(r)*(P_dn - P_up) into shared memory.
// Reference face coefficients: ComputeAdvectionFace FN:10702-10894 (upwind,
// P2_TVD limiters, theta = psi*(1-Cr)/2); diffusive flux
// HorizontalDiffusionXX/YY AD:5185-5196 with Kx from
// Convert_Visc_Dif_Horizontal AD:2487-2494.
template <bool WEST, int NT, int METHOD, int LIM, typename QT, typename KT, int TY>
__device__ __forceinline__ void face_flux(const unsigned char* st, float* out, const float4 cf, const BatchArgs& A,
                                          int pb, int vb, int visb, int qo, int ao, int fo)
{
    using SL = StageLayout<NT, QT, KT, TY>;
    constexpr int pst = WEST ? PBX : 1, vst = WEST ? VBX : 1;
    constexpr int visst = WEST ? Box<KT>::visX : 1;
    constexpr int cs = WEST ? TileGeom<TY>::NWF : TileGeom<TY>::NSF;
    constexpr int tst = (TY + 4) * PBX;              // tracer stride of the stage's tracer tile
    constexpr uint8_t ACT = WEST ? FU_ACT : FV_ACT, ADV = WEST ? FU_ADV : FV_ADV;
    constexpr uint8_t TVDP = WEST ? FU_TVDP : FV_TVDP, TVDN = WEST ? FU_TVDN : FV_TVDN;
    const float* P = reinterpret_cast<const float*>(st + SL::oP);
    const KT* Vis = reinterpret_cast<const KT*>(st + SL::oVis);
    float q, area;
    if (WEST) {
        q = tofl<QT>(reinterpret_cast<const QT*>(st + SL::oQX)[qo], A.qsx);
        area = reinterpret_cast<const float*>(st + SL::oAU)[ao];
    } else {
        q = tofl<QT>(reinterpret_cast<const QT*>(st + SL::oQY)[qo], A.qsy);
        area = reinterpret_cast<const float*>(st + SL::oAV)[ao];
    }
    const uint8_t ff = (WEST || !A.xzflow) ? st[SL::oF + fo] : 0;
    const bool pos = q > 0.f;
    float K = tofl<KT>(Vis[visb], A.ksh) * cf.x + tofl<KT>(Vis[visb - visst], A.ksh) * cf.y;
    if (A.nullDif && q == 0.f) K = 0.f;
    const float auxK = (ff & ACT) ? K * area : 0.f;
    const float kd = pos ? -auxK : auxK;
    const float qv = (ff & ADV) ? q : 0.f;
    const float* pup = P + (pos ? pb - pst : pb);
    const float* pdn = P + (pos ? pb : pb - pst);
    const float* puu = P + (pos ? pb - 2 * pst : pb + pst);
    float gr = 0.f, qvc = 0.f, pa5 = 0.f, pb5 = 0.f, p2 = 0.f, pcr = 0.f;
    if (METHOD == 4) {
        const bool tvd = (ff & ADV) && (ff & (pos ? TVDP : TVDN));   // not NearBoundary
        gr = pos ? cf.z : cf.w;
        const float* RVt = reinterpret_cast<const float*>(st + SL::oV);
        float Cr = q * A.DT * RVt[pos ? vb - vst : vb];
        if (LIM == 5) {
            const float t6 = (1.f - 2.f * fabsf(Cr)) / 6.f;
            pa5 = 0.5f + t6;
            pb5 = 0.5f - t6;
            if (fabsf(Cr) < 1e-16f) Cr = 1e-16f;
            p2 = 2.f / (1.f - Cr);
            pcr = 2.f / Cr;
        }
        qvc = tvd ? q * (0.5f - 0.5f * Cr) : 0.f;
    }
#pragma unroll
    for (int t = 0; t < NT; ++t) {
        const float Pup = pup[t * tst];
        const float dd = pdn[t * tst] - Pup;
        float o = fmaf(kd, dd, qv * Pup);
        if (METHOD == 4) o = fmaf(qvc, limited_slope<LIM>((Pup - puu[t * tst]) * gr, dd, pa5, pb5, p2, pcr), o);
        out[t * cs] = o;
    }
}

// The flow of a discharge term into its layer (Discharges AD:4057-4075): the
// cell's flow, or with the uniform vertical distribution its share by layer
// thickness over layers kmin..kmax (FP64 as the reference, rare columns only).
__device__ __forceinline__ float disch_flow(const BatchArgs& A, const DischTerm& T, int i, int j, int k)
{
    if (!(T.flags & 1)) return (float)T.flow;
    const long long NI = A.L.ni + 2, sk = NI * (A.L.nj + 2), c = i + NI * j;
    double wc = 0.0;
    for (int kk = T.kmin; kk <= T.kmax; ++kk) wc = wc + A.DWZ[c + sk * kk];
    return (float)(T.flow * A.DWZ[c + sk * k] / wc);
}

// s + c += a as an unevaluated FP32 pair (Knuth's TwoSum: the rounding error of
// s + a is carried in c); the _rn intrinsics keep the compiler from fusing
__device__ __forceinline__ void two_sum_acc(float& s, float& c, float a)
{
    const float t = __fadd_rn(s, a);
    const float z = __fsub_rn(t, s);
    c = __fadd_rn(c, __fadd_rn(__fsub_rn(s, __fsub_rn(t, z)), __fsub_rn(a, z)));
    s = t;
}

// reciprocal with at most 1 ulp error (PTX rcp.approx), for the pivots
__device__ __forceinline__ float rcp_approx(float x)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// Shared-memory words of the walk outside the staged layers
struct WalkWords {
    uint64_t bar[2];          // stage mbarriers
    int kmin;                 // lowest KFloor of the tile's water columns
    unsigned done;            // warps that finished a layer (the last one refills its stage)
};

// once per CTA, before the first tile walk
template <int NT, typename QT, typename KT, int TY>
__device__ __forceinline__ void walk_init(unsigned char* smem_raw)
{
    using SM = Smem<NT, QT, KT, TY>;
    WalkWords* ww = reinterpret_cast<WalkWords*>(smem_raw + SM::oBar);
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        ww->done = 0;
        mbar_init(&ww->bar[0], 1);
        mbar_init(&ww->bar[1], 1);
        fence_mbar_init();
    }
}

// One transport step of the 32 x TY tile (bx, by) of one domain: the k-walk
// with the face fluxes and the THOMASZ factorisation, then the
// back-substitution.  `phase` carries the stage parities from one walk to the
// next in the same CTA.  Returns false when a stage never arrived (the status
// word then holds MOHID_DEV_TIMEOUT).  The caller must have every warp of the
// CTA past its previous walk before calling (a barrier between walks).
//
// The layer body is compiled once per stage buffer (the walk advances two
// layers per iteration), so every shared-memory access is a per-thread offset
// computed once per tile plus a constant.
//
// OBC selects the form: 0 closed boundaries, 1 with the MassConservation
// open-boundary terms, 2 with every open-boundary treatment and the
// discharges, so that no form carries the registers and code of terms it
// does not apply (form 1 serves MassConservation batches and ensembles).
template <int NT, int METHOD, int LIM, typename QT, typename KT, int OBC, int TY>
__device__ __forceinline__ bool tile_walk(const BatchArgs& A, const TmaMaps& M, int bx, int by,
                                          unsigned char* smem_raw, uint32_t& phase)
{
    using SL = StageLayout<NT, QT, KT, TY>;
    using SM = Smem<NT, QT, KT, TY>;
    constexpr int NTH = TileGeom<TY>::NTH, NWF = TileGeom<TY>::NWF, NSF = TileGeom<TY>::NSF;
    constexpr int visX = Box<KT>::visX, visOff = Box<KT>::visOff;
    WalkWords* ww = reinterpret_cast<WalkWords*>(smem_raw + SM::oBar);
    uint64_t* bar = ww->bar;
    int* kminp = &ww->kmin;
    unsigned* done = &ww->done;

    const BLayout& L = A.L;
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TX + tx;
    const int i0 = 1 + bx * TX, j0 = 1 + by * TY;
    const int i = i0 + tx, j = j0 + ty;
    const bool inside = i <= L.ni && j <= L.nj;
    const long long c2 = L.at2(i, j);
    const uint8_t cf = inside ? A.cflag[c2] : 0;
    const bool solve = cf & C_SOLVE;
    const int kb = solve ? A.kfloor[c2] : L.nk + 1;

    if (tid == 0) *kminp = L.nk + 1;
    // face constants of the tile's faces (Visc weights with Schmidt folded in,
    // TVD slope ratios), tile-invariant, into shared memory
    float4* CX = reinterpret_cast<float4*>(smem_raw + SM::oCX);
    float4* CY = reinterpret_cast<float4*>(smem_raw + SM::oCY);
    for (int e = tid; e < NWF; e += NTH) {
        float4 c = A.fc[L.at2(i0 + e % TX, j0 + e / TX)];
        c.x *= A.schmidtH; c.y *= A.schmidtH;
        CX[e] = c;
    }
    for (int e = tid; e < NSF; e += NTH) {
        float4 c = A.fc[L.n2 + L.at2(i0 + e % (TX + 1), j0 + e / (TX + 1))];
        c.x *= A.schmidtH; c.y *= A.schmidtH;
        CY[e] = c;
    }
    const bool xW = ty == 0, xS = ty == 1 && tx < TY;
    __syncthreads();
    if (solve) atomicMin(kminp, kb);
    __syncthreads();
    const int kmin = *kminp;
    const int tile = by * A.tilesX + bx;
    if (kmin > L.nk) {                             // no water column in this tile
        if (A.mpart && tid < NT) A.mpart[(long long)(A.t0 + tid) * A.ntiles + tile] = 0.0;
        return true;
    }

    // TMA box origins (x on 16-byte boundaries of the batched layout)
    const int xP = i0 + kXOff - 4, xV = i0 + kXOff - 4;
    const int xVis = i0 + kXOff - visOff, xO = i0 + kXOff;
    const int yP = j0 + kYOff - 2, yV = j0 + kYOff - 1, yO = j0 + kYOff;
    auto issue = [&](int k, int s) {               // one thread: stage layer k into buffer s
        unsigned char* d = smem_raw + (s ? SM::oStage1 : SM::oStage0);
        uint64_t* br = &bar[s];
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");   // earlier reads of buffer s
        mbar_expect_tx(br, SL::tx_bytes);
        tma4(d + SL::oP, &M.P, xP, yP, k, A.t0, br);
        tma3(d + SL::oF, &M.F, xO, yO, k, br);
        tma3(d + SL::oV, &M.V, xV, yV, k, br);
        tma3(d + SL::oVis, &M.Vis, xVis, yV, k, br);
        tma3(d + SL::oQX, &M.QX, xO, yO, k, br);
        tma3(d + SL::oAU, &M.AU, xO, yO, k, br);
        tma3(d + SL::oQY, &M.QY, xO, yO, k, br);
        tma3(d + SL::oAV, &M.AV, xO, yO, k, br);
        tma3(d + SL::oVo, &M.Vo, xO, yO, k, br);
        tma3(d + SL::oQz, &M.Qz, xO, yO, k + 1, br);
        tma3(d + SL::oDv, &M.Dv, xO, yO, k + 1, br);
        tma3(d + SL::oDz, &M.Dz, xO, yO, k, br);
        tma3(d + SL::oFn, &M.Fn, xO, yO, k + 1, br);
    };
    if (tid == 0) {
        issue(kmin, kmin & 1);
        if (kmin < L.nk) issue(kmin + 1, (kmin + 1) & 1);
    }

    const bool horiz = !A.vertical1D;
    const float DT = A.DT;
    const float areaCol = solve ? A.areaCol[c2] : 0.f;
    // k-invariant conditions of the column's vertical terms
    const bool vdif = L.nk > 1 && !(cf & C_SD);
    const bool vadv = L.nk > 1 && !A.vertical1D && (cf & C_CFWTOP) && (cf & C_OPTOP);
    // open boundaries are compiled in only where the batch has reference
    // concentrations: the closed form carries none of their instructions
    const bool obcCol = OBC && (cf & C_BP) && A.Ref != nullptr;
    const float* refc = obcCol ? A.Ref + (long long)A.refIdx[c2] * A.rk : nullptr;   // this column's row
    // discharge terms of this column, dq0 .. dq1 (discharge instantiation only)
    int dq0 = 0, dq1 = 0;
    if (OBC == 2 && A.dStart && solve) { dq0 = A.dStart[c2]; dq1 = A.dStart[c2 + 1]; }
    // own-column values of the face below row k slide up the walk: transport,
    // conductance Kz * area / DZZ (AD:2736-2765), cell flags of rows k-1 and k
    float qz = 0.f, kzb = 0.f;
    uint8_t flm = 0, fl = 0;
    const long long cb = L.at(i, j, 0);
    if (solve) {
        const long long a = cb + (long long)kb * L.sl;
        qz = ldg_as<QT>(A.Qz, a, A.qsz);
        fl = A.flag[a];
        flm = A.flag[a - L.sl];
        if (vdif && (fl & (F_CFW | F_NDW)) == F_CFW) {
            float kz = A.coefV * ldg_as<KT>(A.DiffV, a, A.ksv) + A.backV;
            if (A.nullDif && qz == 0.f) kz = 0.f;
            kzb = kz * areaCol * A.DZZ[a - L.sl];          // DZZ holds 1/DZZ
        }
    }
    float Gp[NT];
#pragma unroll
    for (int t = 0; t < NT; ++t) Gp[t] = 0.f;
    float Wp = 0.f;
    unsigned bad = 0;
    // per-thread offsets into a stage (elements), the same for both buffers
    const int pbO = (ty + 2) * PBX + tx + 4;       // tracer tile, own cell
    const int vbO = (ty + 1) * VBX + tx + 4;       // 1/V, own cell
    const int visO = (ty + 1) * visX + tx + visOff;
    const int own = ty * OWN + tx;                 // own-cell boxes, west-face boxes (pitch TX)
    const int qyO = ty * SL::qyX + tx, avO = ty * AVX + tx, fO = ty * FBX + tx;
    const int fs = ty * (TX + 1) + tx;             // own south face in FY
    // closing faces: warp 0 the west faces of row TY, warp 1 the south faces of column TX
    const int xa = xW ? TY : tx, xb = xW ? tx : TX;
    const int pbX = (xa + 2) * PBX + xb + 4, vbX = (xa + 1) * VBX + xb + 4;
    const int visXo = (xa + 1) * visX + xb + visOff;
    const int qoX = xW ? xa * TX + xb : xa * SL::qyX + xb, aoX = xW ? xa * TX + xb : xa * AVX + xb;
    const int foX = xa * FBX + xb, fiX = xW ? xa * TX + xb : xa * (TX + 1) + xb;
    // THOMASZ scratch of row k of this column: W at A.W + cb + k * sl, G at
    // A.G + (cb + k * sl) * NT
    float* wr = A.W + cb + (long long)kmin * L.sl;
    float* gr = A.G + (cb + (long long)kmin * L.sl) * NT;
    const long long wStep = L.sl, gStep = L.sl * NT;
    const uint64_t keep = l2_policy_evict_last(), drop = l2_policy_evict_first();

    // one layer with the stage buffer S; false: a stage never arrived
    auto layer = [&](auto SC, const int k) -> bool {
        constexpr int S = decltype(SC)::value;
        const unsigned char* st = smem_raw + (S ? SM::oStage1 : SM::oStage0);
        float* FX = reinterpret_cast<float*>(smem_raw + SM::oFX + S * SM::FXYStride);
        float* FY = reinterpret_cast<float*>(smem_raw + SM::oFY + S * SM::FXYStride);
        const bool ok = mbar_wait_bounded(&bar[S], (phase >> S) & 1u, kWaitLimit);
        phase ^= 1u << S;

        // ---- faces of the tile at layer k: own west and south faces; the
        //      east row (warp 0) and north column (warp 1) close the tile
        if (horiz && ok) {
            face_flux<true, NT, METHOD, LIM, QT, KT, TY>(st, FX + own, CX[own], A, pbO, vbO, visO, own, own, fO);
            face_flux<false, NT, METHOD, LIM, QT, KT, TY>(st, FY + fs, CY[fs], A, pbO, vbO, visO, qyO, avO, fO);
            if (xW)
                face_flux<true, NT, METHOD, LIM, QT, KT, TY>(st, FX + fiX, CX[fiX], A, pbX, vbX, visXo, qoX, aoX, foX);
            else if (xS)
                face_flux<false, NT, METHOD, LIM, QT, KT, TY>(st, FY + fiX, CY[fiX], A, pbX, vbX, visXo, qoX, aoX,
                                                              foX);
        }
        if (__syncthreads_or(!ok)) {               // a stage never arrived: leave cleanly
            if (tid == 0) {
                atomicOr(A.status, MOHID_DEV_TIMEOUT);
                mbar_wait_bounded(&bar[S ^ 1], (phase >> (S ^ 1)) & 1u, kWaitLimit);
            }
            return false;
        }

        if (solve && k >= kb) {
            // ---- row k of column (i,j): tracer-independent matrix
            const bool top = k == L.nk;
            const uint8_t flp = top ? 0 : (st + SL::oFn)[own];
            const float rVk = reinterpret_cast<const float*>(st + SL::oV)[vbO];
            const float dvr = reinterpret_cast<const float*>(st + SL::oVo)[own];   // (V - Vold)/V
            const float qzp = tofl<QT>(reinterpret_cast<const QT*>(st + SL::oQz)[own], A.qsz);
            const float dtv = DT * rVk;
            const bool open = fl & F_OP;
            // VolumeVariation: TI = P*Vold/V = P*(1 - (V-Vold)/V), E(KUB) surface term;
            // (V-Vold)/V was formed in FP64 when the volumes were packed
            const float ratio = open ? 1.f - dvr : 1.f;
            // VerticalDiffusion, implicit: faces k (below) and k+1 (above)
            float kza = 0.f;
            if (vdif && (flp & (F_CFW | F_NDW)) == F_CFW) {     // NoDifFlux: F_NDW
                float kz = A.coefV * tofl<KT>(reinterpret_cast<const KT*>(st + SL::oDv)[own], A.ksv) + A.backV;
                if (A.nullDif && qzp == 0.f) kz = 0.f;
                kza = kz * areaCol * reinterpret_cast<const float*>(st + SL::oDz)[own];   // 1/DZZ(k)
            }
            const float aux2 = kzb * dtv, aux1 = kza * dtv;
            float D = -aux2, E = 1.f + aux2 + aux1, Fc = -aux1;
            if (open && top) E += dtv * qzp;
            if (vadv && open) {                          // VerticalAdvection, upwind, implicit
                // (faces under NoAdvFlux carry F_NAW on the cell above them)
                if (k > kb && (flm & F_OP) && !(fl & F_NAW)) {
                    D -= fmaxf(qz, 0.f) * dtv;
                    E -= fminf(qz, 0.f) * dtv;
                }
                if (!top && (flp & (F_OP | F_NAW)) == F_OP) {
                    E += fmaxf(qzp, 0.f) * dtv;
                    Fc += fminf(qzp, 0.f) * dtv;
                }
            }
            // discharges (AD:4025-4128), rare rows: withdrawals (not bypassed)
            // from open cells enter E; each tracer's sources gather in shared
            // memory (dsrc, tracer stride NTH), read by the tracer loop below.
            // A water cell that is not open and takes an inflow restarts from
            // P * Vold / V plus the source (dfill).  The _rn intrinsics fix the
            // rounding, so that the walk's two inlined copies (grid and tile
            // list) cannot contract these differently
            bool dis = false, dfill = false;
            float* dsrc = reinterpret_cast<float*>(smem_raw + SM::oDis) + tid;
            if (OBC == 2 && dq1 > dq0) {
                for (int q = dq0; q < dq1; ++q) {
                    const DischTerm T = A.dTerms[q];
                    if (T.k != k) continue;
                    const float fl = disch_flow(A, T, i, j, k);
                    const float fdt = __fmul_rn(fl, dtv);
                    const float* cq = A.dConc + (long long)q * A.ntAll + A.t0;
                    if (!dis) {
                        for (int t = 0; t < NT; ++t) dsrc[t * NTH] = 0.f;
                        dis = true;
                    }
                    if (open) {
                        if ((T.flags & 2) || fl > 0.f) {
                            for (int t = 0; t < NT; ++t)
                                dsrc[t * NTH] = __fadd_rn(dsrc[t * NTH], __fmul_rn(fdt, cq[t]));
                        } else {
                            E = __fsub_rn(E, __fmul_rn(fdt, (float)T.concMF));
                        }
                    } else if (fl > 0.f) {
                        for (int t = 0; t < NT; ++t) dsrc[t * NTH] = __fmul_rn(fdt, cq[t]);
                        dfill = true;
                    }
                }
            }
            // open boundary cells (OpenBoundaryCondition AD:5369-5742).
            // MassConservation (1) and MassConservNullGrad (7): the net flux
            // through the exterior faces, outflow implicit in E; inflow carries
            // the exterior value in (1) or takes the neighbours' mean across
            // compute faces as an identity row (7).  ImposedValue (2), SubModel
            // (5) and NullGradient (4, set after the solve): identity rows with
            // the exterior value, or the old value.
            float wfob = 0.f;
            const bool obc = obcCol && open;
            bool ident = false;
            const uint8_t* ffl = st + SL::oF + fO;
            if (obc) {
                if (OBC == 1 || A.bc == 1 || A.bc == 7) {
                    const QT* qx = reinterpret_cast<const QT*>(st + SL::oQX);
                    const QT* qy = reinterpret_cast<const QT*>(st + SL::oQY);
                    wfob = obc_wfob((ffl[0] & FU_ACT) ? tofl<QT>(qx[own], A.qsx) : 0.f,
                                    (ffl[FBX] & FU_ACT) ? tofl<QT>(qx[own + TX], A.qsx) : 0.f,
                                    (ffl[0] & FV_ACT) ? tofl<QT>(qy[qyO], A.qsy) : 0.f,
                                    (ffl[1] & FV_ACT) ? tofl<QT>(qy[qyO + 1], A.qsy) : 0.f,
                                    (fl & F_CFW) ? qz : 0.f, (flp & F_CFW) ? qzp : 0.f, dvr, rVk, DT);
                    if (wfob >= 0.f) E += wfob * dtv;
                    else ident = OBC == 2 && A.bc == 7;
                } else {
                    ident = OBC == 2;
                }
                if (ident) { D = 0.f; E = 1.f; Fc = 0.f; }
            }

            // THOMASZ factorisation of row k
            const float aux = fmaf(D, Wp, E);
            float inv = rcp_approx(aux);
            if (aux == 0.f) { inv = 0.f; bad |= MOHID_DEV_ZERO_PIVOT; }
            const float W = -Fc * inv;
            Wp = W;
            st_l2hint(wr, W, keep);                      // read back by the back-substitution
            const float* P = reinterpret_cast<const float*>(st + SL::oP);
#pragma unroll
            for (int t = 0; t < NT; ++t) {
                const float Pc = P[t * (TY + 4) * PBX + pbO];
                float TI = Pc * ratio;
                if (OBC == 2 && dis)
                    TI = __fadd_rn(dfill ? __fmul_rn(Pc, __fsub_rn(1.f, dvr)) : TI, dsrc[t * NTH]);
                if (horiz)
                    TI = fmaf(dtv, (FX[t * NWF + own] - FX[t * NWF + own + TX]) +
                                   (FY[t * NSF + fs] - FY[t * NSF + fs + 1]), TI);
                if (OBC == 2 && ident) {
                    const float* Pt = P + t * (TY + 4) * PBX + pbO;   // the neighbours: i +- 1, j +- PBX
                    if (A.bc == 2 || A.bc == 5) {
                        // the interior mean over the neighbours that are open
                        // and not boundary points (AD:5458-5485)
                        const long long a = cb + (long long)k * L.sl;
                        const float w0 = ((A.flag[a + 1] & F_OP) && !(A.cflag[c2 + 1] & C_BP)) ? 1.f : 0.f;
                        const float w1 = ((A.flag[a - 1] & F_OP) && !(A.cflag[c2 - 1] & C_BP)) ? 1.f : 0.f;
                        const float w2 = ((A.flag[a + L.px] & F_OP) && !(A.cflag[c2 + L.px] & C_BP)) ? 1.f : 0.f;
                        const float w3 = ((A.flag[a - L.px] & F_OP) && !(A.cflag[c2 - L.px] & C_BP)) ? 1.f : 0.f;
                        const float ws = w0 + w1 + w2 + w3;
                        const float ref = refc[(long long)t * A.rts + k] -
                                          (float)A.mfix[1 + 2 * A.ntAll + A.t0 + t];
                        if (ws > 0.f) {
                            const float in = (Pt[1] * w0 + Pt[-1] * w1 + Pt[PBX] * w2 + Pt[-PBX] * w3) / ws;
                            TI = in * (1.f - A.tdec) + ref * A.tdec;
                        } else {
                            TI = ref;
                        }
                    } else if (A.bc == 7) {
                        // the mean across the compute faces north, south,
                        // east and west (NullGradProp AD:2071-2110)
                        const float c0 = (ffl[1] & FV_ACT) ? 1.f : 0.f, c1 = (ffl[0] & FV_ACT) ? 1.f : 0.f;
                        const float c2f = (ffl[FBX] & FU_ACT) ? 1.f : 0.f, c3 = (ffl[0] & FU_ACT) ? 1.f : 0.f;
                        const float cs = c0 + c1 + c2f + c3;
                        TI = cs > 0.f ? (Pt[1] * c0 + Pt[-1] * c1 + Pt[PBX] * c2f + Pt[-PBX] * c3) / cs : Pc;
                    } else {
                        TI = Pc;                         // NullGradient: set after the solve
                    }
                } else if (obc && wfob < 0.f) {
                    // the reference is stored relative to the tracer's loaded
                    // constant; the fixer's correction moves it with the field
                    const float ref = refc[(long long)t * A.rts + k] -
                                      (float)A.mfix[1 + 2 * A.ntAll + A.t0 + t];
                    const float ext = Pc * (1.f - A.tdec) + ref * A.tdec;
                    TI -= wfob * ext * dtv;
                }
                Gp[t] = (TI - D * Gp[t]) * inv;
            }
            GVec<NT>::st(gr, Gp, keep);
            qz = qzp; kzb = kza; flm = fl; fl = flp;
        }
        wr += wStep;
        gr += gStep;
        // buffer S is free once every warp has finished row k: the last warp
        // to get here refills it with layer k + 2 (all warps pass the barrier
        // of layer k + 1 only after all of them got here for layer k).  The
        // counter is an acquire-release fetch-add at CTA scope: each warp's
        // reads of buffer S (ordered before its lane 0 by __syncwarp) happen
        // before its release, the last warp's acquire sees all of them, and
        // the proxy fence in issue() then orders them before the bulk copy's
        // async-proxy writes.
        __syncwarp();
        if (tx == 0) {
            const unsigned n = atom_add_acq_rel_cta(done, 1u);
            if ((n & (TY - 1)) == TY - 1 && k + 2 <= L.nk) issue(k + 2, S);
        }
        return true;
    };

    int k = kmin;
    if (k & 1) {
        if (!layer(std::integral_constant<int, 1>{}, k)) return false;
        ++k;
    }
    for (; k <= L.nk; k += 2) {
        if (!layer(std::integral_constant<int, 0>{}, k)) return false;
        if (k + 1 > L.nk) break;
        if (!layer(std::integral_constant<int, 1>{}, k + 1)) return false;
    }

    // ---- back-substitution (row KUB+1 solves to 0); the scratch rows are
    //      loaded RB rows at a time, all tracers of the column together.  With
    //      the mass fixer on, the column's sum of VolumeZ * value is
    //      accumulated as an FP32 pair per tracer from VolumeZ = hi + lo (about
    //      2^-44 relative).
    const bool mf = A.mpart != nullptr;
    constexpr int RB = NT >= 8 ? 2 : 4;            // rows per batch of loads (registers)
    float mh[NT], ml[NT];
#pragma unroll
    for (int t = 0; t < NT; ++t) { mh[t] = 0.f; ml[t] = 0.f; }
    if (solve) {
        float x[NT];
#pragma unroll
        for (int t = 0; t < NT; ++t) x[t] = 0.f;
        float chk = 0.f;                           // NaN / Inf anywhere in the column shows here
        float* const Po = A.Pout + cb;
        for (int k = L.nk; k >= kb; k -= RB) {
            float w[RB], g[RB][NT], vh[RB], vl[RB];
#pragma unroll
            for (int q = 0; q < RB; ++q)
                if (k - q >= kb) {
                    const long long o = (long long)(k - q) * L.sl;
                    w[q] = ld_l2hint(A.W + cb + o, drop);
                    GVec<NT>::ld(A.G + (cb + o) * NT, g[q], drop);
                    if (mf) {
                        vh[q] = ld_l2hint(A.Vhi + cb + o, drop);
                        vl[q] = ld_l2hint(A.Vlo + cb + o, drop);
                    }
                }
#pragma unroll
            for (int q = 0; q < RB; ++q)
                if (k - q >= kb) {
                    const long long o = (long long)(k - q) * L.sl;
#pragma unroll
                    for (int t = 0; t < NT; ++t) {
                        x[t] = fmaf(w[q], x[t], g[q][t]);
                        Po[(long long)t * A.ts + o] = x[t];
                        chk += x[t];
                        if (mf) {
                            const float pr = __fmul_rn(vh[q], x[t]);
                            two_sum_acc(mh[t], ml[t], pr);
                            ml[t] = __fadd_rn(ml[t], __fmaf_rn(vh[q], x[t], -pr) + vl[q] * x[t]);
                        }
                    }
                }
        }
        if (!isfinite(chk)) bad |= MOHID_DEV_NONFINITE;
    }
    // the scratch rows kmin..nk of this warp's 32 cells are dead now: drop
    // their L2 lines (one W line and NT G lines per row) without a write-back.
    // The warp's cells start on a 32-cell boundary of the layout, so these
    // lines hold no other cells.
    __syncwarp();
    {
        const long long c0 = cb - tx;                // the warp's first cell
        const int nl = 1 + NT;                       // lines per row
        const int nrow = L.nk - kmin + 1;
        for (int e = tx; e < nrow * nl; e += TX) {
            const int r = e / nl, q = e - r * nl;
            const long long c = c0 + (long long)(kmin + r) * L.sl;
            l2_discard(q == 0 ? (const void*)(A.W + c) : (const void*)(A.G + c * NT + (q - 1) * 32));
        }
    }
    if (mf) {
        // fixed-order reduction: lanes by a shuffle tree, warps in order
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
#pragma unroll
            for (int t = 0; t < NT; ++t) {
                const float oh = __shfl_down_sync(0xffffffffu, mh[t], o);
                const float ol = __shfl_down_sync(0xffffffffu, ml[t], o);
                two_sum_acc(mh[t], ml[t], oh);
                ml[t] = __fadd_rn(ml[t], ol);
            }
        float* red = reinterpret_cast<float*>(smem_raw + SM::oRed);
        if (tx == 0)
#pragma unroll
            for (int t = 0; t < NT; ++t) {
                red[2 * (ty * NT + t)] = mh[t];
                red[2 * (ty * NT + t) + 1] = ml[t];
            }
        __syncthreads();
        if (tid < NT) {
            double sum = 0.0;
            for (int w = 0; w < TY; ++w) sum += (double)red[2 * (w * NT + tid)] + (double)red[2 * (w * NT + tid) + 1];
            A.mpart[(long long)(A.t0 + tid) * A.ntiles + tile] = sum;
        }
    }
    if (bad) atomicOr(A.status, bad);
    return true;
}


}  // namespace tile
}  // namespace mohid
