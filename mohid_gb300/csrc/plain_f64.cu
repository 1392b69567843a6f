// plain_f64.cu -- the plain FP64 drop-in step (one property, Fortran layout).
//
// One thread owns one water column (i,j); lanes of a warp run along i, so every
// load of a layer is coalesced.  Walking k = 1..KUB the thread assembles row k
// of the tridiagonal system exactly as ModuleAdvectionDiffusion accumulates it
// over its full-array passes (same operands, same order, no fused multiply-add:
// this file is compiled with --fmad=false), eliminates it at once (THOMASZ
// forward sweep, W in shared memory, G parked in the output array), then
// back-substitutes from KUB+1.  The reference's coefficient arrays (D, E, F,
// TI, 12 flux-coefficient arrays, Kx/Ky/Kz) never exist in memory.
//
// Row k of the system (reference passes, in call order):
//   VolumeVariation                 AD:3966-4021
//   HorizontalDiffusionXX / YY      AD:5156-5214 / AD:5313-5365 (Kx/Ky AD:2453-2595)
//   HorizontalAdvectionXX / YY      AD:4368-4540 / AD:4739-4910
//        face coefficients          FN:10534-10591, FN:10702-10894
//   VerticalDiffusion               AD:2708-2784 (Kz AD:2364-2443)
//   VerticalAdvection               AD:2941-3140
//   OpenBoundaryCondition           AD:5369-5742
//   land -> null_real               AD:1753
//   THOMASZ_NewType2                FN:4026-4123
// then, for NullGradient and Cyclic boundaries, the post-solve passes
//   ImposeNullGradient              AD:1926-1987
//   Prop_CyclicBoundary             AD:2121-2224
#include "common.cuh"

namespace mohid {
namespace {

constexpr int kBX = 32, kBY = 4, kThreads = kBX * kBY;

__device__ __forceinline__ double dmin2(double a, double b) { return (b < a) ? b : a; }
__device__ __forceinline__ double dmax2(double a, double b) { return (b > a) ? b : a; }

// ComputeAdvectionFace (FN:10702-10894) for options validated on the host.
// Stencil values are fetched through `ld(n)` (n = 0..3 <-> cells f-2..f+1)
// only by the methods that read them.
template <class LP, class LV, class LD>
__device__ __forceinline__ void face_coef(double Q, double dt, double VRM, int method, int limiter,
                                          bool nb, bool up2, LP ldP, LV ldV, LD ldU, double CF[4])
{
    double Cup1[4] = {0., 0., 0., 0.};
    if (Q > 0.) Cup1[1] = 1.; else Cup1[2] = 1.;
    if (method == 1 || (nb && up2)) {            // UpwindOrder1: CupHigh = Cup1, Theta = 0
        const double T = 0.;
        for (int n = 0; n < 4; ++n) CF[n] = (1. - T) * Cup1[n] + T * Cup1[n];
        return;
    }
    double Cr = 0., VolumeRel = 0.;
    if (!nb) {
        double v0 = ldV(0), v1 = ldV(1), v2 = ldV(2), v3 = ldV(3);
        if (Q > 0) {
            Cr = Q * dt / v1;
            double Aux = dmin2(dmin2(v0, v1), v2);
            VolumeRel = dmax2(dmax2(v0, v1), v2) / Aux;
        } else {
            Cr = Q * dt / v2;
            double Aux = dmin2(dmin2(v1, v2), v3);
            VolumeRel = dmax2(dmax2(v1, v2), v3) / Aux;
        }
    }
    double CH[4] = {0., 0., 0., 0.};
    double Theta;
    if (method == 2) {                           // FaceConcUpSecondOrder FN:11055
        if (Q > 0) { CH[0] = -1. / 8.; CH[1] = 6. / 8.; CH[2] = 3. / 8.; }
        else if (Q < 0) { CH[3] = -1. / 8.; CH[2] = 6. / 8.; CH[1] = 3. / 8.; }
        else { CH[2] = 1.; }
        Theta = (VolumeRel > VRM) ? 0. : 1.;
    } else if (method == 3) {                    // FaceConcUpThirdOrder FN:11086
        double c = (1 - 2. * fabs(Cr)) / 6.;
        double a = 0.5 + c, b = 0.5 - c, d = (1 - fabs(Cr)) / 2.;
        if (Q > 0) { CH[0] = -d * b; CH[1] = 1 + d * (b - a); CH[2] = d * a; CH[3] = 0.; }
        else if (Q < 0) { CH[3] = -d * b; CH[2] = 1 + d * (b - a); CH[1] = d * a; CH[0] = 0.; }
        else { CH[2] = 1.; }
        Theta = (VolumeRel > VRM) ? 0. : 1.;
    } else if (method == 5 || method == 6) {     // CentralDif / LeapFrog
        double u1 = ldU(1), u2 = ldU(2);
        CH[1] = u2 / (u1 + u2);
        CH[2] = u1 / (u1 + u2);
        Theta = 1.;
    } else {                                     // P2_TVD, not near a boundary
        double p0 = ldP(0), p1 = ldP(1), p2 = ldP(2), p3 = ldP(3);
        double u0 = ldU(0), u1 = ldU(1), u2 = ldU(2), u3 = ldU(3);
        double dC, r;
        if (Q > 0.) {
            CH[2] = 1.;
            dC = (p2 - p1) / (u2 + u1);
            if (fabs(dC) < MOHID_MINVALUE_D) dC = (dC >= 0) ? MOHID_MINVALUE_D : -MOHID_MINVALUE_D;
            r = (p1 - p0) / (u1 + u0) / dC;
        } else {
            CH[1] = 1.;
            dC = (p1 - p2) / (u2 + u1);
            if (fabs(dC) < MOHID_MINVALUE_D) dC = (dC >= 0) ? MOHID_MINVALUE_D : -MOHID_MINVALUE_D;
            r = (p2 - p3) / (u2 + u3) / dC;
        }
        if (limiter == 1) {
            Theta = dmax2(0., dmin2(1., r));
        } else if (limiter == 2) {
            Theta = (r < 0) ? 0. : 2. * r / (1 + r);
        } else if (limiter == 3) {
            Theta = dmax2(0., dmin2(dmin2(2., 2. * r), (1 + r) / 2.));
        } else if (limiter == 4) {
            Theta = dmax2(dmax2(0., dmin2(1., 2. * r)), dmin2(r, 2.));
        } else {
            double a = 0.5 + (1 - 2. * fabs(Cr)) / 6.;
            double b = 0.5 - (1 - 2. * fabs(Cr)) / 6.;
            double Aux = a + b * r;
            if (fabs(Cr) < MOHID_MINVALUE_D) Cr = MOHID_MINVALUE_D;
            Theta = dmax2(0., dmin2(dmin2(Aux, 2. / (1. - Cr)), 2. * r / Cr));
        }
        Theta = 0.5 * Theta * (1. - Cr);
    }
    for (int n = 0; n < 4; ++n) CF[n] = (1. - Theta) * Cup1[n] + Theta * CH[n];
}

// NullGradProp (AD:2071-2110): the mean of the four neighbours of cell `a`
// across compute faces (V faces i, i+1; U faces j, j+1).  Plain loads: the
// post-solve pass reads values it wrote itself.
__device__ __forceinline__ bool null_grad(const double* P, const int* CFU, const int* CFV, size_t a,
                                          long long sj, double& out)
{
    const int cv1 = CFV[a + 1], cv0 = CFV[a], cu1 = CFU[a + sj], cu0 = CFU[a];
    const int Aux = cv1 + cv0 + cu1 + cu0;
    if (Aux <= 0) return false;
    out = (P[a + 1] * (double)cv1 + P[a - 1] * (double)cv0 + P[a + sj] * (double)cu1 +
           P[a - sj] * (double)cu0) / (double)Aux;
    return true;
}

// WaterFluxOBoundary of open boundary cell `a` (FluxAtOpenBoundary,
// AD:5680-5742): transport in through its compute faces less its volume change.
__device__ __forceinline__ double obc_flux(const PlainArgs& A, size_t a, double Vk)
{
    const long long sj = A.sj, sk = A.sk;
    return __ldg(A.Qx + a) * (double)__ldg(A.CFU + a) - __ldg(A.Qx + a + sj) * (double)__ldg(A.CFU + a + sj) +
           __ldg(A.Qy + a) * (double)__ldg(A.CFV + a) - __ldg(A.Qy + a + 1) * (double)__ldg(A.CFV + a + 1) +
           __ldg(A.Qz + a) * (double)__ldg(A.CFW + a) - __ldg(A.Qz + a + sk) * (double)__ldg(A.CFW + a + sk) -
           (Vk - __ldg(A.Vold + a)) / A.DT;
}

// The normal of boundary point (i, j) and its exterior point (ie, je)
// (OpenBoundaryCondition AD:5504-5540): along i on the i = ILB / IUB edges,
// else along j on the j = JLB / JUB edges.  The exterior point is the point at
// -(di, dj) when i = ILB or j = JLB, else at +(di, dj): the corner i = IUB,
// j = JLB therefore takes the interior point (IUB-1, JLB).  false where the
// reference stops ('Orlanski Advection 2').
__device__ __forceinline__ bool orl_normal(int ni, int nj, int i, int j, int& di, int& dj, bool& en, int& ie,
                                           int& je)
{
    if (i == 1 || i == ni) { di = 1; dj = 0; }
    else if (j == 1 || j == nj) { di = 0; dj = 1; }
    else return false;
    en = !(i == 1 || j == 1);
    ie = en ? i + di : i - di;
    je = en ? j + dj : j - dj;
    return true;
}

// OrlanskiCelerity2D (FN:4129-4490) at exterior point (i, j) of the layer
// starting at `lay`, with the arguments OpenBoundaryCondition passes
// (AD:5551-5567): implicit, oblique, computed celerity, the default relaxation
// times (86400 * 300 s), the work box as compute box.  NewField is read from
// NF, OldField from OF and ComputePoints from CP, each at the column-major
// plane offset i + sj * j as the Fortran addresses them (the caller has
// checked that the six unguarded points lie in the plane).  Returns the new
// value at the exterior point.
__device__ double orlanski_value(const double* NF, const double* OF, const double* Ref, const int* CP,
                                 long long sj, long long lay, int ni, int nj, int di, int dj, int i, int j,
                                 bool en, double LimitMax, double DT, double FlowVelX)
{
    auto at = [&](int x, int y) { return (size_t)(lay + x + sj * y); };
    const int s = en ? -1 : 1;                   // from the exterior point into the domain
    const int bi = i + s * di, bj = j + s * dj;  // the first interior point
    const double I1N = NF[at(bi, bj)], I1O = OF[at(bi, bj)];
    const double I2N = NF[at(i + 2 * s * di, j + 2 * s * dj)];
    const double I3N = NF[at(i + 3 * s * di, j + 3 * s * dj)];
    const double I6O = OF[at(bi + dj, bj + di)], I7O = OF[at(bi - dj, bj - di)];
    bool noNE = false, noSW = false;
    if (bi + 3 * dj > ni || bj + 3 * di > nj) noNE = true;
    else if (CP[at(bi + dj, bj + di)] * CP[at(bi + 2 * dj, bj + 2 * di)] * CP[at(bi + 3 * dj, bj + 3 * di)] == 0)
        noNE = true;
    if (bi - 3 * dj < 1 || bj - 3 * di < 1) noSW = true;
    else if (CP[at(bi - dj, bj - di)] * CP[at(bi - 2 * dj, bj - 2 * di)] * CP[at(bi - 3 * dj, bj - 3 * di)] == 0)
        noSW = true;
    const double B5 = OF[at(i, j)];
    // the scheme of Marchesiello et al. (2000), FN:4316-4354
    const double tv = I1N - I1O;
    const double svx = I1N - I2N;
    double svy;
    if ((I6O - I7O) * tv > 0) svy = noSW ? 0. : I1O - I7O;
    else svy = noNE ? 0. : I6O - I1O;
    const double ss = svx * svx + svy * svy;
    double cx = 0., cy = 0.;
    if (ss > 0.) {
        cx = -((tv * svx) / ss);
        cy = -((tv * svy) / ss);
        if (fabs(cx) > LimitMax) cx = LimitMax * cx / fabs(cx);
        if (fabs(cy) > LimitMax) cy = LimitMax * cy / fabs(cy);
    }
    const double refv = Ref[at(i, j)];
    const double trelax = 86400.0 * 300.0;
    cx = cx + FlowVelX;
    double adjx;
    if (cx > 0) {
        cx = 4 * cx;
        adjx = 0.0546875 * I3N - 0.2578125 * I2N + 0.6015625 * I1N;
    } else {
        adjx = refv; cx = 0.; cy = 0.;
    }
    double auxInt = cx * adjx;
    if (cy >= 0 && !noSW) {
        const double B4 = OF[at(i - dj, j - di)], B42 = OF[at(i - 2 * dj, j - 2 * di)];
        const double B43 = OF[at(i - 3 * dj, j - 3 * di)];
        const double adjy = 0.0546875 * B43 - 0.2578125 * B42 + 0.6015625 * B4 + 0.6015625 * B5;
        auxInt = auxInt - 4 * cy * (B5 - adjy);
    } else if (cy < 0 && !noNE) {
        const double B3 = OF[at(i + dj, j + di)], B32 = OF[at(i + 2 * dj, j + 2 * di)];
        const double B33 = OF[at(i + 3 * dj, j + 3 * di)];
        const double adjy = 0.0546875 * B33 - 0.2578125 * B32 + 0.6015625 * B3 + 0.6015625 * B5;
        auxInt = auxInt - 4 * cy * (adjy - B5);
    }
    // OldField(i, j) = NewField(i, j): the exterior point's value as the call found it
    const double old = NF[at(i, j)];
    const double auxBound = 1. + cx * (1 - 0.6015625) + DT / trelax;
    return (old + auxInt + refv * DT / trelax) / auxBound;
}

// Explicit advective flux through the face between cells `m` (= a - s) and `a`
// along stride `s`; `f` is the face index along that axis (1..N), du indexed
// by du(f + n - 2).  Coefficients are computed only where both cells are
// OpenPoints (FN:10559); elsewhere they stay zero, as the reference's arrays.
// nf: the NoFlux mask of these faces when NoAdvFlux is set (AD:4434-4443,
// AD:4804-4813: the face's coefficients are zeroed), else null
template <class DU>
__device__ __forceinline__ void adv_coef(const PlainArgs& A, size_t a, long long s, const double* Q,
                                         const int* nf, int method, int limiter, bool up2, DU du, double C[4])
{
    const double* P = A.P;
    const int* OP = A.OP;
    C[0] = C[1] = C[2] = C[3] = 0.;
    if (__ldg(OP + a - s) == 1 && __ldg(OP + a) == 1) {
        double QF = __ldg(Q + a);
        bool nb = (QF > 0) ? (__ldg(OP + a - 2 * s) != 1) : (__ldg(OP + a + s) != 1);
        double CF[4];
        face_coef(QF, A.DT, A.volumeRelMax, method, limiter, nb, up2,
                  [&](int n) { return __ldg(P + a + (long long)(n - 2) * s); },
                  [&](int n) { return __ldg(A.V + a + (long long)(n - 2) * s); },
                  [&](int n) { return du(n); }, CF);
        for (int n = 0; n < 4; ++n) C[n] = QF * CF[n];
    }
    if (nf && __ldg(nf + a) == 1) C[0] = C[1] = C[2] = C[3] = 0.;
}

template <class DU>
__device__ __forceinline__ double adv_flux(const PlainArgs& A, size_t a, long long s, const double* Q,
                                           const int* nf, int method, int limiter, bool up2, DU du)
{
    const double* P = A.P;
    double C[4];
    adv_coef(A, a, s, Q, nf, method, limiter, up2, du, C);
    return C[0] * __ldg(P + a - 2 * s) + C[1] * __ldg(P + a - s) + C[2] * __ldg(P + a) +
           C[3] * __ldg(P + a + s);
}

// MODE (PlainMode): the full step; or, for implicit horizontal advection
// (AD:4167-4254, AD:1758-1858), the rows of the horizontal system, the column
// step that follows its solution, or the one-layer rows.
template <int MODE>
__global__ void __launch_bounds__(kThreads)
plain_f64_kernel(const PlainArgs A)
{
    constexpr bool kRows = MODE == kPlainHorizRows || MODE == kPlainRows2D;
    extern __shared__ double sW[];               // W(k) at sW[k * kThreads + tid]
    const int tid = threadIdx.y * kBX + threadIdx.x;
    const int i = blockIdx.x * kBX + threadIdx.x;    // 0..ni+1 (Size box)
    const int j = blockIdx.y * kBY + threadIdx.y;    // 0..nj+1
    const int ni = A.ni, nj = A.nj, nk = A.nk;
    if (i > ni + 1 || j > nj + 1) return;
    const long long sj = A.sj, sk = A.sk;
    const size_t c = (size_t)i + (size_t)sj * (size_t)j;     // (i,j,0)
    const double* P = A.P;
    double* Po = A.Pout;

    const bool interior = i >= 1 && i <= ni && j >= 1 && j <= nj;
    if (kRows && !interior) return;               // every work-box cell has a row
    const bool solve = interior && (kRows || __ldg(A.WP + c + (size_t)sk * nk) == 1);
    if (!solve) {                                 // THOMASZ leaves the column untouched
        const double* Pc = A.Pobc ? A.Pobc : P;   // (with the radiated exterior values)
        for (int k = 0; k <= nk + 1; ++k) Po[c + (size_t)sk * k] = __ldg(Pc + c + (size_t)sk * k);
        return;
    }
    if (!kRows) Po[c] = __ldg(P + c);             // row 0 is never solved

    const double DT = A.DT;
    const double DUXc = __ldg(A.DUX + c), DVYc = __ldg(A.DVY + c);
    const int kb = __ldg(A.KFloor + c);
    const bool sd = A.SD != nullptr && __ldg(A.SD + c) != 0;
    const bool colOpenTop = __ldg(A.OP + c + (size_t)sk * nk) == 1;
    const bool colCFWTop = __ldg(A.CFW + c + (size_t)sk * nk) == 1;
    const bool bp = A.Ref != nullptr && __ldg(A.BP2D + c) == 1;
    const int kbp = kb < 0 ? -kb : kb;
    const double ie = A.impExpDifV;
    const bool doVert = nk > 1;
    const bool doVAdv = doVert && !A.vertical1D;
    // AdvectionNudging's factor n of this column: min(in, jn) / nCells, in (jn)
    // = i (j) within nCells of the low edge, IUB - i + 1 (JUB - j + 1) within
    // nCells of the high edge, else nCells, which is what the reference's
    // loop leaves in the distance it does not set when it runs in order
    const bool nud = A.nudge != 0;
    double nudN = 1.0;
    if (nud && A.nudgeCells >= 1) {
        const int nc = A.nudgeCells;
        const int di = i < nc + 1 ? i : (i > ni - nc ? ni - i + 1 : nc);
        const int dj = j < nc + 1 ? j : (j > nj - nc ? nj - j + 1 : nc);
        nudN = (double)(di < dj ? di : dj) / (double)nc;
    }

    // vertical face helpers -------------------------------------------------
    auto Kz = [&](size_t a) {                    // Convert_Dif_Vertical AD:2397-2424
        double kz = A.schmidtCoefV * __ldg(A.DiffV + a) + A.schmidtBackV;
        if (A.nullDif && __ldg(A.Qz + a) == 0.) kz = 0.;
        return kz;
    };
    // vertical advection coefficients of face k (k = 1..nk), AD:2986-3001
    auto vcoef = [&](int k, double C[4]) {
        C[0] = C[1] = C[2] = C[3] = 0.;
        size_t a = c + (size_t)sk * k;
        if (colOpenTop && __ldg(A.OP + a - sk) == 1 && __ldg(A.OP + a) == 1) {
            double QF = __ldg(A.Qz + a);
            bool nb = (QF > 0) ? (__ldg(A.OP + a - 2 * sk) != 1) : (__ldg(A.OP + a + sk) != 1);
            double CF[4];
            face_coef(QF, DT, A.volumeRelMax, A.methodV, A.limiterV, nb, A.upwind2V != 0,
                      [&](int n) { return __ldg(P + a + (long long)(n - 2) * sk); },
                      [&](int n) { return __ldg(A.V + a + (long long)(n - 2) * sk); },
                      [&](int n) { return __ldg(A.DWZ + a + (long long)(n - 2) * sk); }, CF);
            for (int n = 0; n < 4; ++n) C[n] = QF * CF[n];
            if (A.noAdv && __ldg(A.NFW + a) == 1) C[0] = C[1] = C[2] = C[3] = 0.;   // AD:3004-3013
        }
    };

    unsigned int flags = 0;
    double Wp = 0., Gp = 0.;                      // W(k-1), G(k-1)
    double Pk = __ldg(P + c + (size_t)sk);        // P(k) sliding window
    for (int k = 1; k <= nk; ++k) {
        const size_t a = c + (size_t)sk * k;
        const double Vk = __ldg(A.V + a);
        const int opk = __ldg(A.OP + a);
        const double Pkp1 = __ldg(P + a + sk);
        double D = 0., E = 1., F = 0., TI;
        double aTi = 0., aD = 0., aE = 0., aF = 0.;   // AdvectionTi/D/E/F (nudging)

        if (MODE == kPlainVertical) {
            TI = Pk;                              // the step restarts from the line solution
        } else {
        // VolumeVariation
        if (opk == 1) {
            TI = Pk * (__ldg(A.Vold + a) / Vk);
            if (k == nk) {
                double DT_V = DT / Vk;
                E = 1.0 + DT_V * __ldg(A.Qz + a + sk);
            }
        } else {
            TI = Pk;
        }
        // Discharges (AD:4025-4128): this row's terms, in the reference's order
        if (A.dStart) {
            const int q1 = __ldg(A.dStart + c + 1);
            for (int q = __ldg(A.dStart + c); q < q1; ++q) {
                const DischTerm T = A.dTerms[q];
                if (T.k != k) continue;
                const double DT_V = DT / Vk;
                double Flow = T.flow;
                if (T.flags & 1) {                   // uniform: by layer thickness
                    double WaterColumn = 0.0;
                    for (int kk = T.kmin; kk <= T.kmax; ++kk) WaterColumn = WaterColumn + __ldg(A.DWZ + c + (size_t)sk * kk);
                    Flow = T.flow * __ldg(A.DWZ + a) / WaterColumn;
                }
                if (opk == 1) {
                    if ((T.flags & 2) || Flow > 0.) TI = TI + Flow * DT_V * T.conc;
                    else E = E - Flow * DT_V * T.concMF;
                } else if (Flow > 0.) {
                    TI = Pk * __ldg(A.Vold + a) / Vk + Flow * DT_V * T.conc;
                }
            }
        }

        if (!A.vertical1D) {
            // HorizontalDiffusionXX: west face j, east face j+1 (loop runs j = JLB..JUB)
            if (__ldg(A.CFU + a) == 1) {
                size_t am = a - sj;
                double Kx = A.schmidtH * (__ldg(A.ViscH + a) * __ldg(A.DUX + c - sj) +
                                          __ldg(A.ViscH + am) * __ldg(A.DUX + c)) /
                            (__ldg(A.DUX + c) + __ldg(A.DUX + c - sj));
                if (A.nullDif && __ldg(A.Qx + a) == 0.) Kx = 0.;
                if (A.noDif && __ldg(A.NFU + a) == 1) Kx = 0.;              // AD:2496-2500
                double AuxJ = Kx * __ldg(A.AreaU + a) / __ldg(A.DZX + c - sj);
                TI = TI - AuxJ * DT / Vk * (Pk - __ldg(P + am));
                if (A.fDX) A.fDX[a] = 0.0 - AuxJ * (Pk - __ldg(P + am));       // AD:3784-3825
            }
            if (j + 1 <= nj && __ldg(A.CFU + a + sj) == 1) {
                size_t ap = a + sj;
                double Kx = A.schmidtH * (__ldg(A.ViscH + ap) * __ldg(A.DUX + c) +
                                          __ldg(A.ViscH + a) * __ldg(A.DUX + c + sj)) /
                            (__ldg(A.DUX + c + sj) + __ldg(A.DUX + c));
                if (A.nullDif && __ldg(A.Qx + ap) == 0.) Kx = 0.;
                if (A.noDif && __ldg(A.NFU + ap) == 1) Kx = 0.;
                double AuxJ = Kx * __ldg(A.AreaU + ap) / __ldg(A.DZX + c);
                TI = TI + AuxJ * DT / Vk * (__ldg(P + ap) - Pk);
            }
            // HorizontalDiffusionYY
            if (!A.xzflow) {
                if (__ldg(A.CFV + a) == 1) {
                    size_t am = a - 1;
                    double Ky = A.schmidtH * (__ldg(A.ViscH + a) * __ldg(A.DVY + c - 1) +
                                              __ldg(A.ViscH + am) * __ldg(A.DVY + c)) /
                                (__ldg(A.DVY + c) + __ldg(A.DVY + c - 1));
                    if (A.nullDif && __ldg(A.Qy + a) == 0.) Ky = 0.;
                    if (A.noDif && __ldg(A.NFV + a) == 1) Ky = 0.;          // AD:2527-2531
                    double AuxI = Ky * __ldg(A.AreaV + a) / __ldg(A.DZY + c - 1);
                    TI = TI - AuxI * DT / Vk * (Pk - __ldg(P + am));
                    if (A.fDY) A.fDY[a] = 0.0 - AuxI * (Pk - __ldg(P + am));   // AD:3871-3911
                }
                if (i + 1 <= ni && __ldg(A.CFV + a + 1) == 1) {
                    size_t ap = a + 1;
                    double Ky = A.schmidtH * (__ldg(A.ViscH + ap) * __ldg(A.DVY + c) +
                                              __ldg(A.ViscH + a) * __ldg(A.DVY + c + 1)) /
                                (__ldg(A.DVY + c + 1) + __ldg(A.DVY + c));
                    if (A.nullDif && __ldg(A.Qy + ap) == 0.) Ky = 0.;
                    if (A.noDif && __ldg(A.NFV + ap) == 1) Ky = 0.;
                    double AuxI = Ky * __ldg(A.AreaV + ap) / __ldg(A.DZY + c);
                    TI = TI + AuxI * DT / Vk * (__ldg(P + ap) - Pk);
                }
            }
            // HorizontalAdvectionXX: explicit (AD:4454-4488), or implicit
            // (AD:4490-4515: west face j into D, E; east face j+1 into E, F)
            const bool up2H = A.upwind2H != 0;
            const int* nfU = A.noAdv ? A.NFU : nullptr;
            const int* nfV = A.noAdv ? A.NFV : nullptr;
            auto duW = [&](int n) { return __ldg(A.DUX + c + (long long)(n - 2) * sj); };
            auto duE = [&](int n) { return __ldg(A.DUX + c + (long long)(n - 1) * sj); };
            if (__ldg(A.CFU + a) == 1) {
                if (!A.impXX) {
                    double Fx = adv_flux(A, a, sj, A.Qx, nfU, A.methodH, A.limiterH, up2H, duW);
                    if (nud) aTi = aTi + Fx * DT / Vk;
                    else TI = TI + Fx * DT / Vk;
                    if (A.fAX) A.fAX[a] = 0.0 + 1.0 * Fx;                       // AD:4531-4537
                } else {
                    double C[4];
                    adv_coef(A, a, sj, A.Qx, nfU, A.methodH, A.limiterH, up2H, duW, C);
                    double DT2 = DT / Vk;
                    D = D - C[1] * DT2;
                    E = E - C[2] * DT2;
                }
            }
            if (j + 1 <= nj && __ldg(A.CFU + a + sj) == 1) {
                if (!A.impXX) {
                    double Fx = adv_flux(A, a + sj, sj, A.Qx, nfU, A.methodH, A.limiterH, up2H, duE);
                    if (nud) aTi = aTi - Fx * DT / Vk;
                    else TI = TI - Fx * DT / Vk;
                } else {
                    double C[4];
                    adv_coef(A, a + sj, sj, A.Qx, nfU, A.methodH, A.limiterH, up2H, duE, C);
                    double DT1 = DT / Vk;
                    E = E + C[1] * DT1;
                    F = F + C[2] * DT1;
                }
            }
            // HorizontalAdvectionYY: explicit, or implicit (AD:4855-4880)
            if (!A.xzflow) {
                auto dvS = [&](int n) { return __ldg(A.DVY + c + (n - 2)); };
                auto dvN = [&](int n) { return __ldg(A.DVY + c + (n - 1)); };
                if (__ldg(A.CFV + a) == 1) {
                    if (!A.impYY) {
                        double Fy = adv_flux(A, a, 1, A.Qy, nfV, A.methodH, A.limiterH, up2H, dvS);
                        if (nud) aTi = aTi + Fy * DT / Vk;
                        else TI = TI + Fy * DT / Vk;
                        if (A.fAY) A.fAY[a] = 0.0 + 1.0 * Fy;                   // AD:4900-4906
                    } else {
                        double C[4];
                        adv_coef(A, a, 1, A.Qy, nfV, A.methodH, A.limiterH, up2H, dvS, C);
                        double DT2 = DT / Vk;
                        D = D - C[1] * DT2;
                        E = E - C[2] * DT2;
                    }
                }
                if (i + 1 <= ni && __ldg(A.CFV + a + 1) == 1) {
                    if (!A.impYY) {
                        double Fy = adv_flux(A, a + 1, 1, A.Qy, nfV, A.methodH, A.limiterH, up2H, dvN);
                        if (nud) aTi = aTi - Fy * DT / Vk;
                        else TI = TI - Fy * DT / Vk;
                    } else {
                        double C[4];
                        adv_coef(A, a + 1, 1, A.Qy, nfV, A.methodH, A.limiterH, up2H, dvN, C);
                        double DT1 = DT / Vk;
                        E = E + C[1] * DT1;
                        F = F + C[2] * DT1;
                    }
                }
            }
        }
        }

        if (MODE == kPlainHorizRows) {            // the horizontal system, solved by lines
            A.sD[a] = D; A.sE[a] = E; A.sF[a] = F; A.sTI[a] = TI;
            Pk = Pkp1;
            continue;
        }

        if (doVert) {
            // CellFluxes, explicit part of the diffusion through face k (the
            // reference records it at every W compute face, AD:2776-2777, 3668-3711)
            if (A.fDZ && ie < 1. && __ldg(A.CFW + a) == 1)
                A.fDZ[a] = 0.0 - (1. - ie) * Kz(a) * DUXc * DVYc / __ldg(A.DZZ + a - sk) *
                                     (Pk - __ldg(P + a - sk));
            // VerticalDiffusion: face k (below) then face k+1 (above)
            const bool fk = __ldg(A.CFW + a) == 1 && !sd;
            const bool fk1 = k + 1 <= nk && __ldg(A.CFW + a + sk) == 1 && !sd;
            if (fk) {
                double AuxK = Kz(a) * DUXc * DVYc / __ldg(A.DZZ + a - sk);
                if (A.noDif && __ldg(A.NFW + a) == 1) AuxK = 0.;            // AD:2741-2745
                double Aux2 = AuxK * DT / Vk;
                D = D - Aux2 * ie;
                E = E + Aux2 * ie;
                TI = TI - Aux2 * (Pk - __ldg(P + a - sk)) * (1. - ie);
            }
            if (fk1) {
                double AuxK = Kz(a + sk) * DUXc * DVYc / __ldg(A.DZZ + a);
                if (A.noDif && __ldg(A.NFW + a + sk) == 1) AuxK = 0.;
                double Aux1 = AuxK * DT / Vk;
                E = E + Aux1 * ie;
                F = F - Aux1 * ie;
                TI = TI + Aux1 * (Pkp1 - Pk) * (1. - ie);
            }
            if (doVAdv) {
                if (A.explicitV) {
                    if (__ldg(A.CFW + a) == 1) {
                        double C[4];
                        vcoef(k, C);
                        double Fz = C[0] * __ldg(P + a - 2 * sk) + C[1] * __ldg(P + a - sk) +
                                    C[2] * Pk + C[3] * Pkp1;
                        if (nud) aTi = aTi + Fz * DT / Vk;
                        else TI = TI + Fz * DT / Vk;
                        if (A.fAZ) A.fAZ[a] = 0.0 + 1.0 * Fz;                   // AD:3128-3135
                    }
                    if (k + 1 <= nk && __ldg(A.CFW + a + sk) == 1) {
                        double C[4];
                        vcoef(k + 1, C);
                        double Fz = C[0] * __ldg(P + a - sk) + C[1] * Pk + C[2] * Pkp1 +
                                    C[3] * __ldg(P + a + 2 * sk);
                        if (nud) aTi = aTi - Fz * DT / Vk;
                        else TI = TI - Fz * DT / Vk;
                    }
                } else if (nud) {                 // VerticalAdvection_Nudge AD:3302-3331: by layers
                    if (__ldg(A.CFW + a) == 1) {
                        double C[4];
                        vcoef(k, C);
                        double DT2 = DT / Vk;
                        aD = aD - C[1] * DT2;
                        aE = aE - C[2] * DT2;
                    }
                    if (k + 1 <= nk && __ldg(A.CFW + a + sk) == 1) {
                        double C[4];
                        vcoef(k + 1, C);
                        double DT1 = DT / Vk;
                        aE = aE + C[1] * DT1;
                        aF = aF + C[2] * DT1;
                    }
                } else {
                    bool gk, gk1;
                    if (A.docycle == 1) {
                        gk = colCFWTop && k >= kb + 1;
                        gk1 = colCFWTop && k + 1 <= nk && k + 1 >= kb + 1;
                    } else {
                        gk = __ldg(A.CFW + a) == 1;
                        gk1 = k + 1 <= nk && __ldg(A.CFW + a + sk) == 1;
                    }
                    if (gk) {
                        double C[4];
                        vcoef(k, C);
                        double DT2 = DT / Vk;
                        D = D - C[1] * DT2;
                        E = E - C[2] * DT2;
                    }
                    if (gk1) {
                        double C[4];
                        vcoef(k + 1, C);
                        double DT1 = DT / Vk;
                        E = E + C[1] * DT1;
                        F = F + C[2] * DT1;
                    }
                }
            }
        }

        // AdvectionNudging (AD:2051-2060): the advective terms, scaled, at open cells
        if (nud && opk == 1) {
            TI = TI + nudN * aTi;
            D = D + nudN * aD;
            E = E + nudN * aE;
            F = F + nudN * aF;
        }

        // OpenBoundaryCondition (boundary columns, open cells, k >= |KFloor|)
        if (bp && k >= kbp && opk == 1) {
            double DT_V = DT / Vk;
            const double Rf = __ldg(A.Ref + a);
            if (A.bc == 1 || A.bc == 6 || A.bc == 7) {   // MassConservation, Orlanski, MassConservNullGrad
                const double WF = obc_flux(A, a, Vk);
                if (A.bc != 7) {
                    double Ext;
                    if (A.bc == 1) {
                        Ext = Pk * (1.0 - A.tdecAux) + Rf * A.tdecAux;
                    } else {                      // the radiated value at the exterior point
                        int di, dj, ie, je;
                        bool en;
                        Ext = orl_normal(ni, nj, i, j, di, dj, en, ie, je)
                                  ? __ldg(A.Pobc + (size_t)ie + (size_t)sj * je + (size_t)sk * k) : 0.;
                    }
                    if (WF < 0.0) TI = TI - WF * Ext * DT_V;
                    else E = E + WF * DT_V;
                } else if (WF < 0.0) {            // inflow: interior mean of the old field
                    double g;
                    TI = null_grad(P, A.CFU, A.CFV, a, sj, g) ? g : Pk;
                    D = 0.0; E = 1.0; F = 0.0;
                } else {
                    E = E + WF * DT_V;
                }
            } else if (A.bc == 4 || A.bc == 8) {  // NullGradient / Cyclic: set after the solve
                TI = Pk; D = 0.0; E = 1.0; F = 0.0;
            } else {                              // ImposedValue / SubModel
                double A1 = (double)(__ldg(A.OP + a + 1) * (1 - __ldg(A.BP2D + c + 1)));
                double A2 = (double)(__ldg(A.OP + a - 1) * (1 - __ldg(A.BP2D + c - 1)));
                double A3 = (double)(__ldg(A.OP + a + sj) * (1 - __ldg(A.BP2D + c + sj)));
                double A4 = (double)(__ldg(A.OP + a - sj) * (1 - __ldg(A.BP2D + c - sj)));
                double P1 = __ldg(P + a + 1), P2 = __ldg(P + a - 1);
                double P3 = __ldg(P + a + sj), P4 = __ldg(P + a - sj);
                double At = A1 + A2 + A3 + A4;
                double Ext;
                if (At > 0) {
                    double In = (P1 * A1 + P2 * A2 + P3 * A3 + P4 * A4) / At;
                    Ext = In * (1.0 - A.tdecAux) + Rf * A.tdecAux;
                } else {
                    Ext = Rf;
                }
                TI = Ext; D = 0.0; E = 1.0; F = 0.0;
            }
        }

        if (__ldg(A.LP + a) == 1) TI = MOHID_NULL_REAL_D;

        if (MODE == kPlainRows2D) {               // one layer: solved by lines instead
            A.sD[a] = D; A.sE[a] = E; A.sF[a] = F; A.sTI[a] = TI;
            Pk = Pkp1;
            continue;
        }

        // THOMASZ forward sweep (row 1 has no pivot test, FN:4087-4088)
        double W, G;
        if (k == 1) {
            W = -F / E;
            G = TI / E;
        } else {
            double aux = E + D * Wp;
            if (fabs(aux) > 0) {
                W = -F / aux;
                G = (TI - D * Gp) / aux;
            } else {
                W = 0.; G = 0.; flags |= MOHID_DEV_ZERO_PIVOT;
            }
        }
        sW[(size_t)k * kThreads + tid] = W;
        Po[a] = G;
        Wp = W; Gp = G;
        Pk = Pkp1;
    }

    if (kRows) return;
    // row KUB+1: D = 0, E = 1, F = 0, TI = 0 (null_real if flagged land); after
    // a line solve TI there is the field's value (the matrix restarted from it)
    {
        const size_t a = c + (size_t)sk * (nk + 1);
        double TI = (__ldg(A.LP + a) == 1) ? MOHID_NULL_REAL_D : (MODE == kPlainVertical ? __ldg(P + a) : 0.);
        double D = 0., E = 1., F = 0.;
        double aux = E + D * Wp;
        double G;
        if (fabs(aux) > 0) { G = (TI - D * Gp) / aux; (void)F; }
        else { G = 0.; flags |= MOHID_DEV_ZERO_PIVOT; }
        Po[a] = G;
        double R = G;                             // RES(KUB+1) = G(KUB+1)
        for (int k = nk; k >= 1; --k) {
            const size_t b = c + (size_t)sk * k;
            R = sW[(size_t)k * kThreads + tid] * R + Po[b];
            Po[b] = R;
            if (!isfinite(R) && __ldg(A.LP + b) != 1) flags |= MOHID_DEV_NONFINITE;
        }
    }
    if (flags) atomicOr(A.status, flags);
}

// Stand-alone THOMASZ_NewType2 (FN:4026-4123), columns with WaterPoints(KUB)==1.
__global__ void thomasz_f64_kernel(int ni, int nj, int nk, const double* __restrict__ D,
                                   const double* __restrict__ E, const double* __restrict__ F,
                                   const double* __restrict__ TI, double* __restrict__ RES,
                                   const int* __restrict__ WP, unsigned int* status)
{
    extern __shared__ double sW[];
    const int tid = threadIdx.y * kBX + threadIdx.x;
    const int i = 1 + blockIdx.x * kBX + threadIdx.x;
    const int j = 1 + blockIdx.y * kBY + threadIdx.y;
    if (i > ni || j > nj) return;
    const size_t sj = (size_t)ni + 2, sk = sj * ((size_t)nj + 2);
    const size_t c = (size_t)i + sj * (size_t)j;
    if (__ldg(WP + c + sk * nk) != 1) return;
    unsigned int flags = 0;
    double Wp = -__ldg(F + c + sk) / __ldg(E + c + sk);
    double Gp = __ldg(TI + c + sk) / __ldg(E + c + sk);
    sW[kThreads + tid] = Wp;
    RES[c + sk] = Gp;
    for (int k = 2; k <= nk + 1; ++k) {
        const size_t a = c + sk * k;
        double d = __ldg(D + a);
        double aux = __ldg(E + a) + d * Wp;
        double W, G;
        if (fabs(aux) > 0) { W = -__ldg(F + a) / aux; G = (__ldg(TI + a) - d * Gp) / aux; }
        else { W = 0.; G = 0.; flags |= MOHID_DEV_ZERO_PIVOT; }
        sW[(size_t)k * kThreads + tid] = W;
        RES[a] = G;
        Wp = W; Gp = G;
    }
    double R = Gp;
    for (int k = nk; k >= 1; --k) {
        const size_t b = c + sk * k;
        R = sW[(size_t)k * kThreads + tid] * R + RES[b];
        RES[b] = R;
    }
    if (flags) atomicOr(status, flags);
}

// Lower-edge faces (U at j = 1, V at i = 1, W at k = 1) must be closed.
__global__ void check_faces_kernel(int ni, int nj, int nk, const int* __restrict__ CFU,
                                   const int* __restrict__ CFV, const int* __restrict__ CFW,
                                   unsigned int* status)
{
    const size_t sj = (size_t)ni + 2, sk = sj * ((size_t)nj + 2);
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    bool bad = false;
    if (t < (long long)ni * nk) {                         // U faces at j = 1
        int i = 1 + (int)(t % ni), k = 1 + (int)(t / ni);
        bad |= CFU[(size_t)i + sj + sk * k] == 1;
    }
    if (t < (long long)nj * nk) {                         // V faces at i = 1
        int j = 1 + (int)(t % nj), k = 1 + (int)(t / nj);
        bad |= CFV[1 + sj * j + sk * k] == 1;
    }
    if (t < (long long)ni * nj) {                         // W faces at k = 1
        int i = 1 + (int)(t % ni), j = 1 + (int)(t / ni);
        bad |= CFW[(size_t)i + sj * j + sk] == 1;
    }
    if (bad) atomicOr(status, MOHID_DEV_BAD_FACE);
}

// Vertical advection coefficients of face k of column c (AD:2986-3001), from
// A.P: columns with OpenPoints3D(KUB) == 1, faces between open cells.
__device__ void vcoef_at(const PlainArgs& A, size_t c, int k, double C[4])
{
    C[0] = C[1] = C[2] = C[3] = 0.;
    const long long sk = A.sk;
    if (__ldg(A.OP + c + (size_t)sk * A.nk) != 1) return;
    const size_t a = c + (size_t)sk * k;
    if (__ldg(A.OP + a - sk) == 1 && __ldg(A.OP + a) == 1) {
        const double QF = __ldg(A.Qz + a);
        const bool nb = (QF > 0) ? (__ldg(A.OP + a - 2 * sk) != 1) : (__ldg(A.OP + a + sk) != 1);
        double CF[4];
        face_coef(QF, A.DT, A.volumeRelMax, A.methodV, A.limiterV, nb, A.upwind2V != 0,
                  [&](int n) { return __ldg(A.P + a + (long long)(n - 2) * sk); },
                  [&](int n) { return __ldg(A.V + a + (long long)(n - 2) * sk); },
                  [&](int n) { return __ldg(A.DWZ + a + (long long)(n - 2) * sk); }, CF);
        for (int n = 0; n < 4; ++n) C[n] = QF * CF[n];
        if (A.noAdv && __ldg(A.NFW + a) == 1) C[0] = C[1] = C[2] = C[3] = 0.;
    }
}

// CellFluxes, the implicit parts (AD:1882-1916, with CalcVerticalAdvFlux
// AD:3356, CalcVerticalDifFlux AD:3668, CalcHorizontalAdvFluxXX/YY
// AD:3479/3571): the step's face coefficients applied to the new field Pn, at
// the compute faces of the work box, added to what the step recorded.  The
// horizontal coefficients come from H.P (the field the horizontal terms saw),
// the vertical ones from V.P; coefficients the step did not form
// (Vertical1D, XZFlow) are zero, as the reference's arrays.
__global__ void __launch_bounds__(kThreads)
cell_flux_kernel(const PlainArgs H, const PlainArgs Vv, const double* __restrict__ Pn, double impAdvV,
                 double impDifV)
{
    const int i = blockIdx.x * kBX + threadIdx.x, j = blockIdx.y * kBY + threadIdx.y;
    const int ni = H.ni, nj = H.nj, nk = H.nk;
    if (i < 1 || i > ni || j < 1 || j > nj) return;
    const long long sj = H.sj, sk = H.sk;
    const size_t c = (size_t)i + (size_t)sj * (size_t)j;
    const bool up2H = H.upwind2H != 0;
    for (int k = 1; k <= nk; ++k) {
        const size_t a = c + (size_t)sk * k;
        if (nk > 1 && __ldg(H.CFW + a) == 1) {
            if (impAdvV > 0.) {
                double C[4] = {0., 0., 0., 0.};
                if (!H.vertical1D) vcoef_at(Vv, c, k, C);
                H.fAZ[a] = H.fAZ[a] + impAdvV * (C[0] * Pn[a - 2 * sk] + C[1] * Pn[a - sk] + C[2] * Pn[a] +
                                                 C[3] * Pn[a + sk]);
            }
            if (impDifV > 0.) {
                double kz = H.schmidtCoefV * __ldg(H.DiffV + a) + H.schmidtBackV;
                if (H.nullDif && __ldg(H.Qz + a) == 0.) kz = 0.;
                H.fDZ[a] = H.fDZ[a] - impDifV * kz * __ldg(H.DUX + c) * __ldg(H.DVY + c) / __ldg(H.DZZ + a - sk) *
                                          (Pn[a] - Pn[a - sk]);
            }
        }
        if (H.impXX && __ldg(H.CFU + a) == 1) {
            double C[4] = {0., 0., 0., 0.};
            if (!H.vertical1D)
                adv_coef(H, a, sj, H.Qx, H.noAdv ? H.NFU : nullptr, H.methodH, H.limiterH, up2H, [&](int n) {
                    return __ldg(H.DUX + c + (long long)(n - 2) * sj); }, C);
            H.fAX[a] = H.fAX[a] + 1.0 * (C[0] * Pn[a - 2 * sj] + C[1] * Pn[a - sj] + C[2] * Pn[a] +
                                         C[3] * Pn[a + sj]);
        }
        if (H.impYY && __ldg(H.CFV + a) == 1) {
            double C[4] = {0., 0., 0., 0.};
            if (!H.vertical1D && !H.xzflow)
                adv_coef(H, a, 1, H.Qy, H.noAdv ? H.NFV : nullptr, H.methodH, H.limiterH, up2H, [&](int n) {
                    return __ldg(H.DVY + c + (n - 2)); }, C);
            H.fAY[a] = H.fAY[a] + 1.0 * (C[0] * Pn[a - 2] + C[1] * Pn[a - 1] + C[2] * Pn[a] + C[3] * Pn[a + 1]);
        }
    }
}

// THOMAS_3D_i0_j1_NewType / _i1_j0_NewType (FN:3760-3876): thread e solves
// line (l, k), l = 1 + e % m over i (lines along j) or j (lines along i), in
// the reference's arithmetic; W to the scratch, G parked in P, then the
// back-substitution.  A zero pivot, on which the reference stops, is reported.
__global__ void line_solve_kernel(int ni, int nj, int nk, bool alongJ, const double* __restrict__ D,
                                  const double* __restrict__ E, const double* __restrict__ F,
                                  const double* __restrict__ TI, const int* __restrict__ LP, bool landHalo,
                                  double* W, double* P, unsigned int* status)
{
    const int m = alongJ ? ni : nj, n = alongJ ? nj : ni;
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= (long long)m * nk) return;
    const int l = 1 + (int)(e % m), k = 1 + (int)(e / m);
    const long long sj = ni + 2, sk = (long long)(ni + 2) * (nj + 2);
    const long long st = alongJ ? sj : 1;
    const size_t base = (size_t)(alongJ ? l : sj * l) + (size_t)(sk * k);
    unsigned int flags = 0;
    size_t a = base + st;
    double Wp = -F[a] / E[a];
    double Gp = TI[a] / E[a];
    W[a] = Wp; P[a] = Gp;
    for (int x = 2; x <= n + 1; ++x) {
        a = base + (size_t)(st * x);
        double d, ee, f, ti;
        if (x <= n) { d = D[a]; ee = E[a]; f = F[a]; ti = TI[a]; }
        else { d = 0.; ee = 1.; f = 0.; ti = (landHalo && LP[a] == 1) ? MOHID_NULL_REAL_D : 0.; }
        double aux = ee + d * Wp;
        double w, g;
        if (fabs(aux) > 0) {
            w = -f / aux;
            g = (ti - d * Gp) / aux;
        } else {
            w = 0.; g = 0.; flags |= MOHID_DEV_ZERO_PIVOT;
        }
        W[a] = w; P[a] = g;
        Wp = w; Gp = g;
    }
    double R = Gp;                                 // ANSWER(n+1) = G(n+1)
    for (int x = n; x >= 1; --x) {
        a = base + (size_t)(st * x);
        R = W[a] * R + P[a];
        P[a] = R;
    }
    if (flags) atomicOr(status, flags);
}

// ImposeNullGradient (AD:1926-1987).  The reference sweeps the boundary
// columns in order and a cell reads the new values of the boundary cells
// swept before it, so each layer is one sequential sweep: thread k walks the
// column list at layer k (layers never mix).
__global__ void null_gradient_kernel(int nk, long long sj, long long sk, double* P, const int* __restrict__ CFU,
                                     const int* __restrict__ CFV, const int* __restrict__ KFloor,
                                     const int* __restrict__ cols, int ncols)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k > nk) return;
    for (int q = 0; q < ncols; ++q) {
        const size_t c = (size_t)cols[q];
        const int kf = KFloor[c];
        if (k < (kf < 0 ? -kf : kf)) continue;
        const size_t a = c + (size_t)sk * k;
        double g;
        if (null_grad(P, CFU, CFV, a, sj, g)) P[a] = g;
    }
}

// Prop_CyclicBoundary (AD:2121-2224), first part: boundary columns take the
// reference at k = 1..KUB (cell (q, k) of the column list per thread)
__global__ void cyclic_ref_kernel(int nk, long long sk, double* P, const double* __restrict__ Ref,
                                  const int* __restrict__ cols, int ncols)
{
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= (long long)ncols * nk) return;
    const size_t a = (size_t)cols[e / nk] + (size_t)sk * (size_t)(1 + e % nk);
    P[a] = Ref[a];
}

// second part: rows i (ends j = 1, nj) copy the interior next to the opposite
// end, then columns j (ends i = 1, ni); from KFloorZ as stored (a negative
// value starts at the box's lower layer), in the reference's order; thread k
// does layer k
__global__ void cyclic_copy_kernel(int ni, int nj, int nk, long long sj, long long sk, double* P,
                                   const int* __restrict__ KFloor, const int* __restrict__ rows, int nrows,
                                   int ncyc)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k > nk) return;
    auto from = [&](int i, int j) { const int kf = KFloor[(size_t)i + (size_t)sj * j]; return kf < 0 ? 0 : kf; };
    auto at = [&](int i, int j) { return (size_t)i + (size_t)sj * j + (size_t)sk * k; };
    for (int q = 0; q < nrows; ++q) {
        const int i = rows[q];
        if (k >= from(i, nj - 1)) P[at(i, 1)] = P[at(i, nj - 1)];
        if (k >= from(i, 2)) P[at(i, nj)] = P[at(i, 2)];
    }
    for (int q = nrows; q < nrows + ncyc; ++q) {
        const int j = rows[q];
        if (k >= from(ni - 1, j)) P[at(1, j)] = P[at(ni - 1, j)];
        if (k >= from(2, j)) P[at(ni, j)] = P[at(2, j)];
    }
}

// Orlanski radiation (OpenBoundaryCondition AD:5496-5569) at every open cell
// of the boundary columns: the new value at the cell's exterior point, into S
// (a copy of A.P).  The reference calls OrlanskiCelerity2D point by point (j
// outer, i inner, then k), each call reading NewField at three interior points
// and writing it at the exterior point.  Layers never mix.  On grids at least
// 4 cells wide in i and j every such read precedes (in the reference's order)
// any write to the same point, so each (column, layer) is one thread reading
// A.P (seq false); on narrower grids thread k walks layer k in order, reading
// and writing S (seq true).  OldField is the reference's PROPOld, a copy of
// PROP whose values the calls never change: A.P.  Points off the work box's
// edges, and reads outside the layer plane, set a status bit instead.
__global__ void orlanski_kernel(const PlainArgs A, double* S, const int* __restrict__ cols, int ncols, bool seq)
{
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const int ni = A.ni, nj = A.nj, nk = A.nk;
    int q0, q1, k;
    if (seq) {
        k = 1 + (int)e;
        if (k > nk) return;
        q0 = 0; q1 = ncols;
    } else {
        if (e >= (long long)ncols * nk) return;
        q0 = (int)(e / nk); q1 = q0 + 1;
        k = 1 + (int)(e % nk);
    }
    const long long sj = A.sj, sk = A.sk, plane = sj * (nj + 2), lay = sk * k;
    const double* NF = seq ? S : A.P;
    unsigned flags = 0;
    for (int q = q0; q < q1; ++q) {
        const size_t c = (size_t)cols[q];
        const int i = (int)(c % (size_t)sj), j = (int)(c / (size_t)sj);
        const int kf = __ldg(A.KFloor + c);
        if (k < (kf < 0 ? -kf : kf)) continue;
        const size_t a = c + (size_t)lay;
        if (__ldg(A.OP + a) != 1) continue;
        int di, dj, ie, je;
        bool en;
        if (!orl_normal(ni, nj, i, j, di, dj, en, ie, je)) { flags |= MOHID_DEV_OBC_EDGE; continue; }
        // the exterior point, the three interior points along the normal and
        // the two beside the first are read without a bounds test
        const int sgn = en ? -1 : 1;
        bool inside = true;
        const int px[6] = {ie, ie + sgn * di, ie + 2 * sgn * di, ie + 3 * sgn * di, ie + sgn * di + dj,
                           ie + sgn * di - dj};
        const int py[6] = {je, je + sgn * dj, je + 2 * sgn * dj, je + 3 * sgn * dj, je + sgn * dj + di,
                           je + sgn * dj - di};
        for (int n = 0; n < 6; ++n) {
            const long long o = px[n] + sj * py[n];
            inside = inside && o >= 0 && o < plane;
        }
        if (!inside) { flags |= MOHID_DEV_OBC_READ; continue; }
        const double Vk = __ldg(A.V + a);
        const double DT_V = A.DT / Vk;
        const double VelBound = obc_flux(A, a, Vk) * DT_V;
        const double LimitMax = 10. * A.DT / (__ldg(A.DUX + c) + __ldg(A.DVY + c)) * 2;
        S[(size_t)(lay + ie + sj * je)] = orlanski_value(NF, A.P, A.Ref, A.OP, sj, lay, ni, nj, di, dj, ie, je,
                                                         en, LimitMax, A.DT, VelBound);
    }
    if (flags) atomicOr(A.status, flags);
}

}  // namespace

cudaError_t launch_orlanski(const PlainArgs& a, double* S, const int* cols, int ncols, cudaStream_t s)
{
    if (ncols <= 0 || a.nk <= 0) return cudaSuccess;
    const bool seq = a.ni < 4 || a.nj < 4;
    const long long n = seq ? a.nk : (long long)ncols * a.nk;
    orlanski_kernel<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(a, S, cols, ncols, seq);
    return cudaGetLastError();
}

cudaError_t launch_null_gradient(int ni, int nj, int nk, double* P, const int* CFU, const int* CFV,
                                 const int* KFloor, const int* cols, int ncols, cudaStream_t s)
{
    if (ncols <= 0) return cudaSuccess;
    const long long sj = ni + 2, sk = (long long)(ni + 2) * (nj + 2);
    null_gradient_kernel<<<(nk + 1 + 63) / 64, 64, 0, s>>>(nk, sj, sk, P, CFU, CFV, KFloor, cols, ncols);
    return cudaGetLastError();
}

cudaError_t launch_cyclic(int ni, int nj, int nk, double* P, const double* Ref, const int* KFloor,
                          const int* cols, int ncols, const int* rows, int nrows, int ncyc, cudaStream_t s)
{
    const long long sj = ni + 2, sk = (long long)(ni + 2) * (nj + 2);
    if (ncols > 0) {
        const long long n = (long long)ncols * nk;
        cyclic_ref_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(nk, sk, P, Ref, cols, ncols);
    }
    if (nrows + ncyc > 0)
        cyclic_copy_kernel<<<(nk + 1 + 63) / 64, 64, 0, s>>>(ni, nj, nk, sj, sk, P, KFloor, rows, nrows, ncyc);
    return cudaGetLastError();
}

template <int MODE>
cudaError_t launch_plain_mode(const PlainArgs& a, cudaStream_t s)
{
    dim3 blk(kBX, kBY);
    dim3 grd((unsigned)((a.ni + 2 + kBX - 1) / kBX), (unsigned)((a.nj + 2 + kBY - 1) / kBY));
    const bool rows = MODE == kPlainHorizRows || MODE == kPlainRows2D;
    size_t smem = rows ? 0 : sizeof(double) * (size_t)(a.nk + 2) * kThreads;
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(plain_f64_kernel<MODE>,
                                              cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    plain_f64_kernel<MODE><<<grd, blk, smem, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_plain_f64(const PlainArgs& a, cudaStream_t s, int mode)
{
    switch (mode) {
    case kPlainFull: return launch_plain_mode<kPlainFull>(a, s);
    case kPlainHorizRows:
    case kPlainRows2D:
        if (!a.sD || !a.sE || !a.sF || !a.sTI) return cudaErrorInvalidValue;
        return mode == kPlainHorizRows ? launch_plain_mode<kPlainHorizRows>(a, s)
                                       : launch_plain_mode<kPlainRows2D>(a, s);
    case kPlainVertical: return launch_plain_mode<kPlainVertical>(a, s);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_cell_fluxes(const PlainArgs& h, const PlainArgs& v, const double* Pnew, double impAdvV,
                               double impDifV, cudaStream_t s)
{
    if (!h.fAX || !h.fAY || !h.fAZ || !h.fDX || !h.fDY || !h.fDZ) return cudaErrorInvalidValue;
    dim3 blk(kBX, kBY);
    dim3 grd((unsigned)((h.ni + 2 + kBX - 1) / kBX), (unsigned)((h.nj + 2 + kBY - 1) / kBY));
    cell_flux_kernel<<<grd, blk, 0, s>>>(h, v, Pnew, impAdvV, impDifV);
    return cudaGetLastError();
}

cudaError_t launch_line_solve(int ni, int nj, int nk, bool alongJ, const double* D, const double* E,
                              const double* F, const double* TI, const int* LP, bool landHalo, double* W,
                              double* P, unsigned int* status, cudaStream_t s)
{
    const int m = alongJ ? ni : nj;
    const long long lines = (long long)m * nk;
    if (lines <= 0) return cudaSuccess;
    line_solve_kernel<<<(unsigned)((lines + 127) / 128), 128, 0, s>>>(ni, nj, nk, alongJ, D, E, F, TI, LP,
                                                                      landHalo, W, P, status);
    return cudaGetLastError();
}

cudaError_t launch_thomasz_f64(int ni, int nj, int nk, const double* D, const double* E,
                               const double* F, const double* TI, double* RES, const int* WP,
                               unsigned int* status, cudaStream_t s)
{
    dim3 blk(kBX, kBY);
    dim3 grd((unsigned)((ni + kBX - 1) / kBX), (unsigned)((nj + kBY - 1) / kBY));
    size_t smem = sizeof(double) * (size_t)(nk + 2) * kThreads;
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(thomasz_f64_kernel,
                                              cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    thomasz_f64_kernel<<<grd, blk, smem, s>>>(ni, nj, nk, D, E, F, TI, RES, WP, status);
    return cudaGetLastError();
}

cudaError_t launch_check_faces(int ni, int nj, int nk, const int* CFU, const int* CFV,
                               const int* CFW, unsigned int* status, cudaStream_t s)
{
    long long n = (long long)ni * nk;
    if ((long long)nj * nk > n) n = (long long)nj * nk;
    if ((long long)ni * nj > n) n = (long long)ni * nj;
    unsigned blocks = (unsigned)((n + 255) / 256);
    check_faces_kernel<<<blocks, 256, 0, s>>>(ni, nj, nk, CFU, CFV, CFW, status);
    return cudaGetLastError();
}

}  // namespace mohid
