// batched_flux.cu -- CellFluxes of the batched form: the face fluxes of one
// tracer's last step (GetAdvFlux / GetDifFlux, ModuleAdvectionDiffusion.F90:
// 697-860), formed on request from the two ping-pong buffers, so the step
// itself does no extra work.  The buffer the next step writes still holds the
// field the last step started from, which the explicit horizontal terms saw;
// the current buffer holds the new field, which the implicit vertical terms
// are recorded with (AD:1882-1916).  Same face terms as the walk, in FP32:
//  * west / south faces (AdvFluxX/Y, DifFluxX/Y): the walk's face flux split
//    into its advective part q * P_up + q * (1 - Cr)/2 * psi(r) * dP (AD:4531,
//    4900 with ComputeAdvectionFace FN:10702) and its diffusive part
//    -K * area * (P - P_west) (CalcHorizontalDifFluxXX/YY AD:3784, 3871);
//  * bottom faces (AdvFluxZ, DifFluxZ): max(Qz, 0) * P(k-1) + min(Qz, 0) * P(k)
//    on faces between open cells of columns open at KUB, where the reference
//    forms the coefficients (AD:2941-3013), and -Kz * DUX * DVY / DZZ(k-1) *
//    (P(k) - P(k-1)) on every compute face from k = 2 (CalcVerticalDifFlux
//    AD:3668-3711; NoDifFlux does not zero it there, Kz being left as it is).
// Fluxes are positive towards the cell; zero away from the faces that carry
// them.  Absolute values are stored + c on water cells; differences need no c.
#include "batched_launch.cuh"

namespace mohid {
namespace {
using namespace tile;

struct FluxIn {
    const float* Po;      // the tracer's stored values before the last step
    const float* Pn;      // after it
    double shift;         // the tracer's constant ...
    const double* corr;   // ... plus the mass fixer's correction (device)
    int adv;              // 1: AdvFluxX/Y/Z, 0: DifFluxX/Y/Z
    double* out;          // X, Y, Z face arrays over the Size box (Fortran layout), n3 apart
    long long n3;
};

template <bool WEST, int METHOD, int LIM, typename QT, typename KT>
__device__ __forceinline__ float hface(const BatchArgs& A, const FluxIn& F, float c, int i, int j, int k)
{
    const BLayout& L = A.L;
    constexpr uint8_t ACT = WEST ? FU_ACT : FV_ACT, ADV = WEST ? FU_ADV : FV_ADV;
    constexpr uint8_t TVDP = WEST ? FU_TVDP : FV_TVDP, TVDN = WEST ? FU_TVDN : FV_TVDN;
    const long long g = L.at(i, j, k);
    const long long s = WEST ? L.px : 1;           // to the cell across the face (j - 1 or i - 1)
    const uint8_t ff = (WEST || !A.xzflow) ? A.fflag[g] : 0;
    if (!(ff & (F.adv ? ADV : ACT))) return 0.f;
    const float q = ldg_as<QT>(WEST ? A.Qx : A.Qy, g, WEST ? A.qsx : A.qsy);
    const float4 cf = A.fc[(WEST ? 0 : L.n2) + L.at2(i, j)];
    const float* P = F.Po;
    if (!F.adv) {
        float K = ldg_as<KT>(A.ViscH, g, A.ksh) * (cf.x * A.schmidtH) +
                  ldg_as<KT>(A.ViscH, g - s, A.ksh) * (cf.y * A.schmidtH);
        if (A.nullDif && q == 0.f) K = 0.f;
        const float area = (WEST ? A.AreaU : A.AreaV)[g];
        return -(K * area) * (P[g] - P[g - s]);
    }
    const bool pos = q > 0.f;
    const long long up = pos ? g - s : g, dn = pos ? g : g - s, uu = pos ? g - 2 * s : g + s;
    const float Pup = P[up];
    float o = q * (Pup + c);
    if (METHOD == 4 && (ff & (pos ? TVDP : TVDN))) {
        float Cr = q * A.DT * A.RV[up];
        float pa5 = 0.f, pb5 = 0.f, p2 = 0.f, pcr = 0.f;
        if (LIM == 5) {
            const float t6 = (1.f - 2.f * fabsf(Cr)) / 6.f;
            pa5 = 0.5f + t6;
            pb5 = 0.5f - t6;
            if (fabsf(Cr) < 1e-16f) Cr = 1e-16f;
            p2 = 2.f / (1.f - Cr);
            pcr = 2.f / Cr;
        }
        const float qvc = q * (0.5f - 0.5f * Cr);
        const float gr = pos ? cf.z : cf.w;
        o = fmaf(qvc, limited_slope<LIM>((Pup - P[uu]) * gr, P[dn] - Pup, pa5, pb5, p2, pcr), o);
    }
    return o;
}

// one block per row (j, k) of the Size box, threads along i
template <int METHOD, int LIM, typename QT, typename KT>
__global__ void __launch_bounds__(256) k_cell_fluxes(const BatchArgs A, const FluxIn F)
{
    const BLayout& L = A.L;
    const int NI = L.ni + 2, NJ = L.nj + 2;
    const float c = (float)(F.shift + (F.corr ? *F.corr : 0.0));
    for (long long r = blockIdx.x; r < (long long)NJ * (L.nk + 2); r += gridDim.x) {
        const int j = (int)(r % NJ), k = (int)(r / NJ);
        for (int i = threadIdx.x; i < NI; i += blockDim.x) {
            const long long e = i + (long long)NI * (j + (long long)NJ * k);
            float fx = 0.f, fy = 0.f, fz = 0.f;
            if (i >= 1 && i <= L.ni && j >= 1 && j <= L.nj && k >= 1 && k <= L.nk) {
                if (!A.vertical1D) {
                    fx = hface<true, METHOD, LIM, QT, KT>(A, F, c, i, j, k);
                    fy = hface<false, METHOD, LIM, QT, KT>(A, F, c, i, j, k);
                }
                const long long g = L.at(i, j, k);
                const uint8_t fl = A.flag[g];
                if (L.nk > 1 && (fl & F_CFW)) {
                    const float qz = ldg_as<QT>(A.Qz, g, A.qsz);
                    const float* P = F.Pn;
                    if (F.adv) {
                        const uint8_t flm = A.flag[g - L.sl];
                        if (!A.vertical1D && (A.cflag[L.at2(i, j)] & C_OPTOP) && (fl & F_OP) && (flm & F_OP) &&
                            !(fl & F_NAW))
                            fz = fmaxf(qz, 0.f) * (P[g - L.sl] + c) + fminf(qz, 0.f) * (P[g] + c);
                    } else if (k >= 2) {
                        float kz = A.coefV * ldg_as<KT>(A.DiffV, g, A.ksv) + A.backV;
                        if (A.nullDif && qz == 0.f) kz = 0.f;
                        fz = -(kz * A.areaCol[L.at2(i, j)] * A.DZZ[g - L.sl]) * (P[g] - P[g - L.sl]);
                    }
                }
            }
            F.out[e] = (double)fx;
            F.out[F.n3 + e] = (double)fy;
            F.out[2 * F.n3 + e] = (double)fz;
        }
    }
}

template <typename QT, typename KT>
cudaError_t launch_fluxes(const BatchArgs& a, const FluxIn& f, int method, int limiter, cudaStream_t s)
{
    const long long rows = (long long)(a.L.nj + 2) * (a.L.nk + 2);
    const unsigned grid = (unsigned)(rows < 16384 ? rows : 16384);
    if (method == 1) k_cell_fluxes<1, 0, QT, KT><<<grid, 256, 0, s>>>(a, f);
    else switch (limiter) {
    case 1: k_cell_fluxes<4, 1, QT, KT><<<grid, 256, 0, s>>>(a, f); break;
    case 2: k_cell_fluxes<4, 2, QT, KT><<<grid, 256, 0, s>>>(a, f); break;
    case 3: k_cell_fluxes<4, 3, QT, KT><<<grid, 256, 0, s>>>(a, f); break;
    case 4: k_cell_fluxes<4, 4, QT, KT><<<grid, 256, 0, s>>>(a, f); break;
    default: k_cell_fluxes<4, 5, QT, KT><<<grid, 256, 0, s>>>(a, f); break;
    }
    return cudaGetLastError();
}

}  // namespace

cudaError_t cell_fluxes_batched(const BatchArgs& a, const float* Pold, const float* Pnew, double shift,
                                const double* corr, bool adv, double* out, long long n3, int method, int limiter,
                                bool halfQ, bool halfK, cudaStream_t s)
{
    FluxIn f{Pold, Pnew, shift, corr, adv ? 1 : 0, out, n3};
    if (halfQ && halfK) return launch_fluxes<__half, __half>(a, f, method, limiter, s);
    if (halfQ) return launch_fluxes<__half, float>(a, f, method, limiter, s);
    return launch_fluxes<float, float>(a, f, method, limiter, s);
}

}  // namespace mohid
