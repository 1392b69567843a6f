/*
 * ad_oracle.c -- TEST INFRASTRUCTURE ONLY (checker and CPU baseline).
 *
 * FP64 restatement of one call of ModuleAdvectionDiffusion::AdvectionDiffusion
 * (Software/MOHIDBase2/ModuleAdvectionDiffusion.F90, "AD" below) on the
 * non-Optimize path, with its numerics from ModuleFunctions
 * (Software/MOHIDBase1/ModuleFunctions.F90, "FN").  Every pass is a full-array
 * sweep in the reference's order (k outer, j, i inner) with the reference's
 * OpenMP work split, so that each floating-point accumulation happens in the
 * same order as in the Fortran.  Compile with -ffp-contract=off: the Fortran
 * evaluates a*b+c as two rounded operations.
 *
 * Deviations (documented, not reachable with consistent MOHID masks):
 *  - THOMASZ with a zero pivot: the reference keeps W/G from whatever column
 *    its OpenMP thread solved before (FN:4090-4099); here W = G = 0 for that
 *    row and MOHID_AD_ERR_ZERO_PIVOT is returned.
 *  - faces on the WorkSize lower edge (j = JLB for U, i = ILB for V, k = KLB
 *    for W) must not be compute faces: the reference would read outside the
 *    Size box there.  Such input returns MOHID_AD_ERR_BOUNDS.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "oracle.h"

#define MINVALUE 1.e-16            /* MinValue, ModuleGlobalData.F90:1812 */
#define NULL_REAL (-9.9e15)        /* null_real, ModuleGlobalData.F90:143 */

typedef struct {
    int NI, NJ, NK;                /* Size extents */
    size_t n3, n2;
} ora_ext;

#define I3(i, j, k) ((size_t)(i) + (size_t)X.NI * ((size_t)(j) + (size_t)X.NJ * (size_t)(k)))
#define I2(i, j) ((size_t)(i) + (size_t)X.NI * (size_t)(j))

static inline double dmin2(double a, double b) { return (b < a) ? b : a; }
static inline double dmax2(double a, double b) { return (b > a) ? b : a; }

/* FaceConcUpFirstOrder, FN:11127-11140 */
static void face_up1(double c[4], double Q)
{
    c[0] = c[1] = c[2] = c[3] = 0.;
    if (Q > 0.) c[1] = 1.; else c[2] = 1.;
}

/* FaceConcUpSecondOrder, FN:11055-11084 */
static void face_up2(double c[4], double Q)
{
    c[0] = c[1] = c[2] = c[3] = 0.;
    if (Q > 0) { c[0] = -1. / 8.; c[1] = 6. / 8.; c[2] = 3. / 8.; }
    else if (Q < 0) { c[3] = -1. / 8.; c[2] = 6. / 8.; c[1] = 3. / 8.; }
    else face_up1(c, Q);
}

/* FaceConcUpThirdOrder, FN:11086-11125 */
static void face_up3(double c[4], double Q, double Cr)
{
    double cc = (1 - 2. * fabs(Cr)) / 6.;
    double a = 0.5 + cc, b = 0.5 - cc, d = (1 - fabs(Cr)) / 2.;
    if (Q > 0) { c[0] = -d * b; c[1] = 1 + d * (b - a); c[2] = d * a; c[3] = 0.; }
    else if (Q < 0) { c[3] = -d * b; c[2] = 1 + d * (b - a); c[1] = d * a; c[0] = 0.; }
    else face_up1(c, Q);
}

/* ComputeAdvectionFace, FN:10702-10894 (Courant, FN:11045-11052). */
int ora_advection_face(const double P[4], const double V[4], const double du[4], double dt,
                       double Q, double VolumeRelMax, int method, int limiter,
                       int nearBoundary, int upwind2, double CFace[4])
{
    double Cup1[4], CupH[4];
    double Cr = 0., Theta = 0., VolumeRel = 0.;
    face_up1(Cup1, Q);
    if (!nearBoundary) {
        double Aux;
        if (Q > 0) {
            Cr = Q * dt / V[1];
            Aux = dmin2(dmin2(V[0], V[1]), V[2]);
            VolumeRel = dmax2(dmax2(V[0], V[1]), V[2]) / Aux;
        } else {
            Cr = Q * dt / V[2];
            Aux = dmin2(dmin2(V[1], V[2]), V[3]);
            VolumeRel = dmax2(dmax2(V[1], V[2]), V[3]) / Aux;
        }
    }
    if (method == MOHID_UPWIND_ORDER1 || (nearBoundary && upwind2)) {
        memcpy(CupH, Cup1, sizeof CupH);
        Theta = 0.;
    } else if (method == MOHID_UPWIND_ORDER2 && !nearBoundary) {
        face_up2(CupH, Q);
        Theta = (VolumeRel > VolumeRelMax) ? 0. : 1.;
    } else if (method == MOHID_UPWIND_ORDER3 && !nearBoundary) {
        face_up3(CupH, Q, Cr);
        Theta = (VolumeRel > VolumeRelMax) ? 0. : 1.;
    } else if (method == MOHID_CENTRAL_DIF || method == MOHID_LEAP_FROG) {
        double AuxLeft = du[2] / (du[1] + du[2]);
        double AuxRight = du[1] / (du[1] + du[2]);
        CupH[0] = 0.; CupH[1] = AuxLeft; CupH[2] = AuxRight; CupH[3] = 0.;
        Theta = 1.;
    } else if (method == MOHID_P2_TVD && !nearBoundary) {
        double dC, r;
        CupH[0] = CupH[1] = CupH[2] = CupH[3] = 0.;
        if (Q > 0.) {
            CupH[2] = 1.;
            dC = (P[2] - P[1]) / (du[2] + du[1]);
            if (fabs(dC) < MINVALUE) dC = (dC >= 0) ? MINVALUE : -MINVALUE;
            r = (P[1] - P[0]) / (du[1] + du[0]) / dC;
        } else {
            CupH[1] = 1.;
            dC = (P[1] - P[2]) / (du[2] + du[1]);
            if (fabs(dC) < MINVALUE) dC = (dC >= 0) ? MINVALUE : -MINVALUE;
            r = (P[2] - P[3]) / (du[2] + du[3]) / dC;
        }
        if (limiter == MOHID_TVD_MINMOD) {
            Theta = dmax2(0., dmin2(1., r));
        } else if (limiter == MOHID_TVD_VANLEER) {
            Theta = (r < 0) ? 0. : 2. * r / (1 + r);
        } else if (limiter == MOHID_TVD_MUSCL) {
            Theta = dmax2(0., dmin2(dmin2(2., 2. * r), (1 + r) / 2.));
        } else if (limiter == MOHID_TVD_SUPERBEE) {
            Theta = dmax2(dmax2(0., dmin2(1., 2. * r)), dmin2(r, 2.));
        } else if (limiter == MOHID_TVD_PDM) {
            double a = 0.5 + (1 - 2. * fabs(Cr)) / 6.;
            double b = 0.5 - (1 - 2. * fabs(Cr)) / 6.;
            double Aux = a + b * r;
            if (fabs(Cr) < MINVALUE) Cr = MINVALUE;
            Theta = dmax2(0., dmin2(dmin2(Aux, 2. / (1. - Cr)), 2. * r / Cr));
        } else {
            return MOHID_AD_ERR_OPTION;
        }
        Theta = 0.5 * Theta * (1. - Cr);
    } else {
        return MOHID_AD_ERR_OPTION;
    }
    for (int n = 0; n < 4; ++n) CFace[n] = (1. - Theta) * Cup1[n] + Theta * CupH[n];
    return 0;
}

/* ComputeAdvection1D_V2, FN:10534-10591, for one line.  The Fortran dummy
 * arrays are assumed-shape (lower bound 1), so dummy face index ilb..iub of a
 * line passed over the Size box 0..N+1 lands on actual faces ilb-1..iub-1;
 * the caller passes actual face bounds [flo, fhi].  `at(n)` addresses element
 * n (actual index, 0..N+1) of the line with stride `s` from base `o`. */
static int advection_line(int flo, int fhi, double dt, const double* du, size_t sdu,
                          const double* P, const double* Q, const double* V,
                          const int* CP, size_t o, size_t s,
                          double* Cf, double* Df, double* Ef, double* Ff,
                          int method, int limiter, double VolumeRelMax, int upwind2)
{
    for (int f = flo; f <= fhi; ++f) {
        size_t a = o + (size_t)f * s;
        if (CP[a - s] == 1 && CP[a] == 1) {
            double QF = Q[a];
            int nb = 0;
            if (QF > 0) { if (CP[a - 2 * s] != 1) nb = 1; }
            else { if (CP[a + s] != 1) nb = 1; }
            double P4[4], V4[4], du4[4], CF[4];
            for (int n = 0; n < 4; ++n) {
                size_t an = a + ((size_t)n - 2) * s;     /* f-2 .. f+1 */
                P4[n] = P[an];
                V4[n] = V[an];
                du4[n] = du[(size_t)(f + n - 2) * sdu];
            }
            int e = ora_advection_face(P4, V4, du4, dt, QF, VolumeRelMax, method, limiter,
                                       nb, upwind2, CF);
            if (e) return e;
            Cf[a] = QF * CF[0];
            Df[a] = QF * CF[1];
            Ef[a] = QF * CF[2];
            Ff[a] = QF * CF[3];
        }
    }
    return 0;
}

static int disch_valid(const ora_domain* d);

/* Orlanski boundaries (OpenBoundaryCondition AD:5496-5569): the normal of a
 * boundary point and the exterior point OrlanskiCelerity2D works on.  di = 1
 * on the i = ILB / IUB edges, else dj = 1 on the j = JLB / JUB edges, else the
 * reference stops ('Orlanski Advection 2'); the exterior point lies at -(di,
 * dj) when i = ILB or j = JLB, else at +(di, dj).  Returns 0, or 1 where the
 * reference stops. */
static int orlanski_normal(int ni, int nj, int i, int j, int* di, int* dj, int* en, int* iext, int* jext)
{
    if (i == 1 || i == ni) { *di = 1; *dj = 0; }
    else if (j == 1 || j == nj) { *di = 0; *dj = 1; }
    else return 1;
    if (i == 1 || j == 1) { *en = 0; *iext = i - *di; *jext = j - *dj; }
    else { *en = 1; *iext = i + *di; *jext = j + *dj; }
    return 0;
}

/* Every boundary point with an open cell must have a normal (else the
 * reference stops: MOHID_AD_ERR_OPTION).  The corner i = IUB, j = JLB takes
 * the interior point (IUB-1, JLB) as its exterior point and reads two cells
 * along i past it, (IUB+2, JLB): in the Size-box array, column-major, that
 * element is (ILB-1, JLB+1), which the reference reads (it does not check
 * bounds) and this restatement, indexing the same contiguous array, reads
 * too.  Reads whose element lies outside the whole layer plane are rejected
 * (MOHID_AD_ERR_BOUNDS): they only occur on grids under three cells wide. */
static int orlanski_geometry_ok(const ora_domain* d)
{
    const int ni = d->ni, nj = d->nj, nk = d->nk;
    ora_ext X = {ni + 2, nj + 2, nk + 2, 0, 0};
    const long long n2 = (long long)X.NI * X.NJ;
    for (int j = 1; j <= nj; ++j)
        for (int i = 1; i <= ni; ++i) {
            if (d->BoundaryPoints2D[I2(i, j)] != 1) continue;
            int open = 0;
            for (int k = abs(d->KFloorZ[I2(i, j)]); k <= nk; ++k) open |= d->OpenPoints3D[I3(i, j, k)] == 1;
            if (!open) continue;
            int di = 0, dj = 0, en = 0, ie = 0, je = 0;
            if (orlanski_normal(ni, nj, i, j, &di, &dj, &en, &ie, &je)) return MOHID_AD_ERR_OPTION;
            const int s = en ? -1 : 1;               /* towards the interior */
            const int pts[6][2] = {{ie, je}, {ie + s * di, je + s * dj}, {ie + 2 * s * di, je + 2 * s * dj},
                                   {ie + 3 * s * di, je + 3 * s * dj},
                                   {ie + s * di + dj, je + s * dj + di}, {ie + s * di - dj, je + s * dj - di}};
            for (int q = 0; q < 6; ++q) {
                const long long lin = (long long)pts[q][0] + (long long)X.NI * pts[q][1];
                if (lin < 0 || lin >= n2) return MOHID_AD_ERR_BOUNDS;
            }
        }
    return 0;
}

/* OrlanskiCelerity2D (ModuleFunctions.F90:4129-4490) with the arguments
 * OpenBoundaryCondition passes (AD:5551-5567): NewField = PROP, OldField =
 * PROPOld, ComputePoints = OpenPoints3D, ReferenceField = ReferenceProp,
 * Imin..Jmax = the work box, FlowVelX = the boundary flux times DT/V, no
 * relaxation times (86400 * 300 s), the implicit, non-constant-celerity,
 * oblique form.  Writes OldField and NewField at the exterior point (i, j, k)
 * and returns the new value there. */
static double orlanski_celerity_2d(ora_ext X, double* NewF, double* OldF, const double* Ref, const int* CP,
                                   int Imin, int Imax, int Jmin, int Jmax, int di, int dj, int i, int j, int k,
                                   int en, double LimitMax, double DT, double FlowVelX)
{
#define NF(a, b) NewF[I3((a), (b), k)]
#define OF(a, b) OldF[I3((a), (b), k)]
#define CPT(a, b) CP[I3((a), (b), k)]
    int noSW = 0, noNE = 0;
    double I1N, I1O, I2N, I2O, I3N, I3O, I6O, I7O;
    double B3 = 0, B32 = 0, B33 = 0, B4 = 0, B42 = 0, B43 = 0, B5;
    if (en) {
        I1N = NF(i - di, j - dj); I1O = OF(i - di, j - dj);
        I2N = NF(i - 2 * di, j - 2 * dj); I3N = NF(i - 3 * di, j - 3 * dj);
        I2O = OF(i - 2 * di, j - 2 * dj); I3O = OF(i - 3 * di, j - 3 * dj);
        I6O = OF(i - di + dj, j - dj + di); I7O = OF(i - di - dj, j - dj - di);
        if ((i - di + 3 * dj) > Imax || (j - dj + 3 * di) > Jmax) noNE = 1;
        else if (CPT(i - di + dj, j - dj + di) * CPT(i - di + 2 * dj, j - dj + 2 * di) *
                 CPT(i - di + 3 * dj, j - dj + 3 * di) == 0) noNE = 1;
        if ((i - di - 3 * dj) < Imin || (j - dj - 3 * di) < Jmin) noSW = 1;
        else if (CPT(i - di - dj, j - dj - di) * CPT(i - di - 2 * dj, j - dj - 2 * di) *
                 CPT(i - di - 3 * dj, j - dj - 3 * di) == 0) noSW = 1;
    } else {
        I1N = NF(i + di, j + dj); I1O = OF(i + di, j + dj);
        I2N = NF(i + 2 * di, j + 2 * dj); I3N = NF(i + 3 * di, j + 3 * dj);
        I2O = OF(i + 2 * di, j + 2 * dj); I3O = OF(i + 3 * di, j + 3 * dj);
        I6O = OF(i + di + dj, j + dj + di); I7O = OF(i + di - dj, j + dj - di);
        if ((i + di + 3 * dj) > Imax || (j + dj + 3 * di) > Jmax) noNE = 1;
        else if (CPT(i + di + dj, j + dj + di) * CPT(i + di + 2 * dj, j + dj + 2 * di) *
                 CPT(i + di + 3 * dj, j + dj + 3 * di) == 0) noNE = 1;
        if ((i + di - 3 * dj) < Imin || (j + dj - 3 * di) < Jmin) noSW = 1;
        else if (CPT(i + di - dj, j + dj - di) * CPT(i + di - 2 * dj, j + dj - 2 * di) *
                 CPT(i + di - 3 * dj, j + dj - 3 * di) == 0) noSW = 1;
    }
    (void)I2O; (void)I3O;                    /* read by the explicit form only */
    if (!noNE) { B3 = OF(i + dj, j + di); B32 = OF(i + 2 * dj, j + 2 * di); B33 = OF(i + 3 * dj, j + 3 * di); }
    if (!noSW) { B4 = OF(i - dj, j - di); B42 = OF(i - 2 * dj, j - 2 * di); B43 = OF(i - 3 * dj, j - 3 * di); }
    B5 = OF(i, j);
    /* the scheme of Marchesiello et al. (2000), FN:4316-4354 */
    const double tv = I1N - I1O;
    const double svx = I1N - I2N;
    const double auxIntY = I6O - I7O;
    double svy;
    if (auxIntY * tv > 0) { svy = I1O - I7O; if (noSW) svy = 0.; }
    else { svy = I6O - I1O; if (noNE) svy = 0.; }
    const double ss = svx * svx + svy * svy;
    double wcx, wcy;
    if (ss > 0.) {
        wcx = -((tv * svx) / ss);
        wcy = -((tv * svy) / ss);
        if (fabs(wcx) > LimitMax) wcx = LimitMax * wcx / fabs(wcx);
        if (fabs(wcy) > LimitMax) wcy = LimitMax * wcy / fabs(wcy);
    } else {
        wcx = 0.; wcy = 0.;
    }
    const double refv = Ref[I3(i, j, k)];
    const double trelax_out = 86400 * 300, trelax_in = 86400 * 300;
    wcx = wcx + FlowVelX;
    double adjx, trelax;
    if (wcx > 0) {
        wcx = 4 * wcx;
        adjx = 0.0546875 * I3N - 0.2578125 * I2N + 0.6015625 * I1N;
        trelax = trelax_out;
    } else {
        adjx = refv;
        wcx = 0.;
        wcy = 0.;
        trelax = trelax_in;
    }
    double auxInt = wcx * adjx;
    if (wcy >= 0 && !noSW) {
        const double adjy = 0.0546875 * B43 - 0.2578125 * B42 + 0.6015625 * B4 + 0.6015625 * B5;
        auxInt = auxInt - 4 * wcy * (B5 - adjy);
    } else if (wcy < 0 && !noNE) {
        const double adjy = 0.0546875 * B33 - 0.2578125 * B32 + 0.6015625 * B3 + 0.6015625 * B5;
        auxInt = auxInt - 4 * wcy * (adjy - B5);
    }
    OF(i, j) = NF(i, j);
    double auxBound = 1;
    auxBound = auxBound + wcx * (1 - 0.6015625) + DT / trelax;
    NF(i, j) = (OF(i, j) + auxInt + refv * DT / trelax) / auxBound;
    return NF(i, j);
#undef NF
#undef OF
#undef CPT
}

static int validate(const ora_domain* d, const double* PROP, const mohid_ad_params* p,
                    const double* ReferenceProp)
{
    if (!d || !PROP || !p) return MOHID_AD_ERR_NULLPTR;
    if (d->ni < 1 || d->nj < 1 || d->nk < 1) return MOHID_AD_ERR_BOUNDS;
    /* AD:1231-1239, AD:1340-1349 */
    if ((p->ImpExp_AdvXX == 1. || p->ImpExp_AdvYY == 1.) &&
        (p->AdvMethodH == MOHID_UPWIND_ORDER2 || p->AdvMethodH == MOHID_UPWIND_ORDER3))
        return MOHID_AD_ERR_OPTION;
    if (p->ImpExp_AdvV == 1. &&
        (p->AdvMethodV == MOHID_UPWIND_ORDER2 || p->AdvMethodV == MOHID_UPWIND_ORDER3))
        return MOHID_AD_ERR_OPTION;
    if (p->ImpExp_DifH != 0.) return MOHID_AD_ERR_OPTION;
    if (p->ImpExp_AdvXX == 1. && p->ImpExp_AdvYY == 1.) return MOHID_AD_ERR_OPTION;
    if (p->ImpExp_AdvV != 0. && p->ImpExp_AdvV != 1.) return MOHID_AD_ERR_OPTION;
    /* HorizontalAdvectionXX / YY ERR01: explicit (0) or implicit (1) only */
    if ((p->ImpExp_AdvXX != 0. && p->ImpExp_AdvXX != 1.) || (p->ImpExp_AdvYY != 0. && p->ImpExp_AdvYY != 1.))
        return MOHID_AD_ERR_OPTION;
    /* AdvectionNudging: HorizontalAdvectionXX/YY_Nudge add their implicit
     * coefficients (cells j-1, j or i-1, i) into the vertical system's D, E, F
     * (AD:4692-4696, 5076-5080), and with Vertical1D AdvectionNudging reads
     * AdvectionTi/D/E/F that nothing set in the call (AD:1704, 4151-4157);
     * neither is restated */
    if (p->AdvectionNudging && (p->ImpExp_AdvXX != 0. || p->ImpExp_AdvYY != 0. || p->Vertical1D))
        return MOHID_AD_ERR_UNSUPPORTED;
    if (!disch_valid(d)) return MOHID_AD_ERR_BOUNDS;
    /* the reference reads NoFluxU/V/W whenever NoAdvFlux or NoDifFlux is set */
    if ((p->NoAdvFlux || p->NoDifFlux) && (!d->NoFluxU || !d->NoFluxV || !d->NoFluxW)) return MOHID_AD_ERR_NULLPTR;
    if (p->Docycle_method != 1 && p->Docycle_method != 2) return MOHID_AD_ERR_OPTION;
    /* methods 2..4 reach `stop` at the first near-boundary face unless Upwind2 */
    int mH = p->AdvMethodH, mV = p->AdvMethodV;
    if (mH < 1 || mH > 6 || mV < 1 || mV > 6) return MOHID_AD_ERR_OPTION;
    if ((mH >= 2 && mH <= 4) && !p->Upwind2H) return MOHID_AD_ERR_OPTION;
    if ((mV >= 2 && mV <= 4) && !p->Upwind2V) return MOHID_AD_ERR_OPTION;
    if (mH == MOHID_P2_TVD && (p->TVDLimitationH < 1 || p->TVDLimitationH > 5)) return MOHID_AD_ERR_OPTION;
    if (mV == MOHID_P2_TVD && (p->TVDLimitationV < 1 || p->TVDLimitationV > 5)) return MOHID_AD_ERR_OPTION;
    {
        int bc = p->BoundaryCondition;
        if (ReferenceProp) {
            if (bc != 1 && bc != 2 && bc != 4 && bc != 5 && bc != 6 && bc != 7 && bc != 8)
                return MOHID_AD_ERR_OPTION;          /* Set_Internal_State ERR01, AD:5816-5830 */
            if (bc == MOHID_BC_ORLANSKI) {
                int e = orlanski_geometry_ok(d);
                if (e) return e;
            }
        } else if (bc == MOHID_BC_CYCLIC) {
            return MOHID_AD_ERR_OPTION;              /* Prop_CyclicBoundary reads ReferenceProp, AD:2150 */
        }
    }
    /* lower-edge faces must be closed (see header) */
    ora_ext X = {d->ni + 2, d->nj + 2, d->nk + 2, 0, 0};
    for (int k = 1; k <= d->nk; ++k) {
        for (int i = 1; i <= d->ni; ++i)
            if (d->ComputeFacesU3D[I3(i, 1, k)] == 1) return MOHID_AD_ERR_BOUNDS;
        for (int j = 1; j <= d->nj; ++j)
            if (d->ComputeFacesV3D[I3(1, j, k)] == 1) return MOHID_AD_ERR_BOUNDS;
    }
    for (int j = 1; j <= d->nj; ++j)
        for (int i = 1; i <= d->ni; ++i)
            if (d->ComputeFacesW3D[I3(i, j, 1)] == 1) return MOHID_AD_ERR_BOUNDS;
    return 0;
}

struct ora_work {
    int ni, nj, nk;
    double* pool;
    double *Kx, *Ky, *Kz;
    double *D, *E, *F, *TI;
    double *XC, *XD, *XE, *XF, *YC, *YD, *YE, *YF, *VC, *VD, *VE, *VF;
    double *WFOB;
    /* CellFluxes (allocated on first use): AdvFluxX/Y/Z, DifFluxX/Y/Z */
    double* fpool;
    double *FAX, *FAY, *FAZ, *FDX, *FDY, *FDZ;
    /* AdvectionNudging (allocated on first use): AdvectionTi/D/E/F */
    double* npool;
    double *ATi, *AD, *AE, *AF;
};

/* AllocateVariables, AD:537-684: work arrays live for the instance's life and
 * start at null_real (AD:640-675). */
ora_work* ora_work_new(int ni, int nj, int nk)
{
    size_t n3 = (size_t)(ni + 2) * (size_t)(nj + 2) * (size_t)(nk + 2);
    ora_work* w = (ora_work*)calloc(1, sizeof(ora_work));
    if (!w) return NULL;
    w->pool = (double*)malloc(sizeof(double) * n3 * 20);
    if (!w->pool) { free(w); return NULL; }
    w->ni = ni; w->nj = nj; w->nk = nk;
    double** slots[20] = {&w->Kx, &w->Ky, &w->Kz, &w->D, &w->E, &w->F, &w->TI, &w->XC, &w->XD,
                          &w->XE, &w->XF, &w->YC, &w->YD, &w->YE, &w->YF, &w->VC, &w->VD,
                          &w->VE, &w->VF, &w->WFOB};
    for (int s = 0; s < 20; ++s) *slots[s] = w->pool + (size_t)s * n3;
    #pragma omp parallel for schedule(static)
    for (size_t q = 0; q < n3 * 20; ++q) w->pool[q] = NULL_REAL;
    return w;
}

void ora_work_free(ora_work* w)
{
    if (w) { free(w->pool); free(w->fpool); free(w->npool); free(w); }
}

/* AllocateVariables AD:608-612 (AdvectionTi/D/E/F) */
static int ora_work_nudge(ora_work* w)
{
    if (w->npool) return 1;
    size_t n3 = (size_t)(w->ni + 2) * (size_t)(w->nj + 2) * (size_t)(w->nk + 2);
    w->npool = (double*)malloc(sizeof(double) * n3 * 4);
    if (!w->npool) return 0;
    double** slots[4] = {&w->ATi, &w->AD, &w->AE, &w->AF};
    for (int s = 0; s < 4; ++s) *slots[s] = w->npool + (size_t)s * n3;
    return 1;
}

/* AllocateVariables AD:567-573 (the cell-flux arrays) */
static int ora_work_fluxes(ora_work* w)
{
    if (w->fpool) return 1;
    size_t n3 = (size_t)(w->ni + 2) * (size_t)(w->nj + 2) * (size_t)(w->nk + 2);
    w->fpool = (double*)malloc(sizeof(double) * n3 * 6);
    if (!w->fpool) return 0;
    double** slots[6] = {&w->FAX, &w->FAY, &w->FAZ, &w->FDX, &w->FDY, &w->FDZ};
    for (int s = 0; s < 6; ++s) *slots[s] = w->fpool + (size_t)s * n3;
    return 1;
}

/* GetAdvFlux / GetDifFlux, AD:697-860: the fluxes of the last step made with
 * CellFluxes (which = 0..5: AdvFluxX, AdvFluxY, AdvFluxZ, DifFluxX, DifFluxY,
 * DifFluxZ), or NULL */
const double* ora_cell_flux(const ora_work* w, int which)
{
    if (!w || !w->fpool || which < 0 || which > 5) return NULL;
    const double* f[6] = {w->FAX, w->FAY, w->FAZ, w->FDX, w->FDY, w->FDZ};
    return f[which];
}

/* SetMatrixValue over the Size box (FN:1599-1645: OpenMP over k, static). */
static void fill3(ora_ext X, double* a, double v)
{
    #pragma omp parallel for schedule(static)
    for (int k = 0; k < X.NK; ++k) {
        double* s = a + (size_t)k * X.n2;
        for (size_t q = 0; q < X.n2; ++q) s[q] = v;
    }
}

/* THOMAS_3D_i0_j1_NewType / THOMAS_3D_i1_j0_NewType, FN:3760-3876: one
 * tridiagonal system per line of the work box along j (alongJ) or i, from the
 * first work cell to the halo cell past the last (the row there is whatever
 * the matrix holds: D = 0, E = 1, F = 0, TI = 0 unless assembled), every
 * layer k = 1..KUB.  The first row is divided by E without a test; a zero
 * pivot later stops the reference (ERR10), here it is reported.  The answer
 * goes to P. */
static int thomas_3d(const ora_domain* d, int alongJ, const double* D, const double* E, const double* F,
                     const double* TI, double* P)
{
    ora_ext X = {d->ni + 2, d->nj + 2, d->nk + 2, 0, 0};
    const int n = alongJ ? d->nj : d->ni, m = alongJ ? d->ni : d->nj, nk = d->nk;
    int zero = 0;
    #pragma omp parallel reduction(|:zero)
    {
        double* W = (double*)malloc(sizeof(double) * (size_t)(n + 2));
        double* G = (double*)malloc(sizeof(double) * (size_t)(n + 2));
        #pragma omp for schedule(dynamic, 1) collapse(2)
        for (int k = 1; k <= nk; ++k)
            for (int l = 1; l <= m; ++l) {
                #define CELL(x) (alongJ ? I3(l, (x), k) : I3((x), l, k))
                size_t a1 = CELL(1);
                W[1] = -F[a1] / E[a1];
                G[1] = TI[a1] / E[a1];
                for (int x = 2; x <= n + 1; ++x) {
                    size_t a = CELL(x);
                    double aux = E[a] + D[a] * W[x - 1];
                    if (fabs(aux) > 0) {
                        W[x] = -F[a] / aux;
                        G[x] = (TI[a] - D[a] * G[x - 1]) / aux;
                    } else {
                        W[x] = 0.; G[x] = 0.; zero = 1;
                    }
                }
                P[CELL(n + 1)] = G[n + 1];
                for (int x = n; x >= 1; --x) P[CELL(x)] = W[x] * P[CELL(x + 1)] + G[x];
                #undef CELL
            }
        free(W); free(G);
    }
    return zero;
}

/* NullGradProp, AD:2071-2110: the mean of the four neighbours across compute
 * faces (V faces i, i+1; U faces j, j+1); 0 when the cell has none. */
static int null_grad_prop(const ora_domain* d, const double* P, int i, int j, int k, double* out)
{
    ora_ext X = {d->ni + 2, d->nj + 2, d->nk + 2, 0, 0};
    const int *CFU = d->ComputeFacesU3D, *CFV = d->ComputeFacesV3D;
    int Aux = CFV[I3(i + 1, j, k)] + CFV[I3(i, j, k)] + CFU[I3(i, j + 1, k)] + CFU[I3(i, j, k)];
    if (Aux <= 0) return 0;
    *out = (P[I3(i + 1, j, k)] * (double)CFV[I3(i + 1, j, k)] + P[I3(i - 1, j, k)] * (double)CFV[I3(i, j, k)] +
            P[I3(i, j + 1, k)] * (double)CFU[I3(i, j + 1, k)] + P[I3(i, j - 1, k)] * (double)CFU[I3(i, j, k)]) /
           (double)Aux;
    return 1;
}

/* ImposeNullGradient, AD:1926-1987: in place after the solve, boundary
 * columns in the reference's order (j, i, k from |KFloorZ| to KUB), so a cell
 * reads the new values of boundary neighbours set before it. */
static void impose_null_gradient(const ora_domain* d, double* P)
{
    ora_ext X = {d->ni + 2, d->nj + 2, d->nk + 2, 0, 0};
    for (int j = 1; j <= d->nj; ++j)
        for (int i = 1; i <= d->ni; ++i) {
            if (d->BoundaryPoints2D[I2(i, j)] != 1) continue;
            for (int k = abs(d->KFloorZ[I2(i, j)]); k <= d->nk; ++k) {
                double v;
                if (null_grad_prop(d, P, i, j, k, &v)) P[I3(i, j, k)] = v;
            }
        }
}

/* Prop_CyclicBoundary, AD:2121-2224: boundary columns take the reference
 * (k = 1..KUB), then a row (column) whose two ends are boundary points copies
 * the interior values next to the opposite end, from that column's KFloorZ. */
/* the reference loops from KFloorZ as stored; a negative KFloorZ would index
 * below the Size box there, here the loop starts at the box's lower layer */
static inline int kfloor_clamp(int kf) { return kf < 0 ? 0 : kf; }

static void cyclic_boundary(const ora_domain* d, double* P, const double* Ref)
{
    ora_ext X = {d->ni + 2, d->nj + 2, d->nk + 2, 0, 0};
    const int ni = d->ni, nj = d->nj, nk = d->nk;
    const int* BP = d->BoundaryPoints2D;
    for (int j = 1; j <= nj; ++j)
        for (int i = 1; i <= ni; ++i)
            if (BP[I2(i, j)] == 1)
                for (int k = 1; k <= nk; ++k) P[I3(i, j, k)] = Ref[I3(i, j, k)];
    for (int i = 2; i <= ni - 1; ++i) {
        if (BP[I2(i, 1)] != 1 || BP[I2(i, nj)] != 1) continue;
        for (int k = kfloor_clamp(d->KFloorZ[I2(i, nj - 1)]); k <= nk; ++k) P[I3(i, 1, k)] = P[I3(i, nj - 1, k)];
        for (int k = kfloor_clamp(d->KFloorZ[I2(i, 2)]); k <= nk; ++k) P[I3(i, nj, k)] = P[I3(i, 2, k)];
    }
    for (int j = 2; j <= nj - 1; ++j) {
        if (BP[I2(1, j)] != 1 || BP[I2(ni, j)] != 1) continue;
        for (int k = kfloor_clamp(d->KFloorZ[I2(ni - 1, j)]); k <= nk; ++k) P[I3(1, j, k)] = P[I3(ni - 1, j, k)];
        for (int k = kfloor_clamp(d->KFloorZ[I2(2, j)]); k <= nk; ++k) P[I3(ni, j, k)] = P[I3(2, j, k)];
    }
}

/* CalcHorizontalAdvFluxXX / YY, AD:3479-3526, AD:3571-3619: over the work
 * box, at compute faces, Flux += Weigth * (C P(-2) + D P(-1) + E P(0) + F P(+1))
 * along the face's direction (s: the stride) */
static void cell_adv_flux(const ora_domain* d, const int* CF, long long s, double wgt, const double* Cc,
                          const double* Cd, const double* Ce, const double* Cf, const double* P, double* Flux)
{
    ora_ext X = {d->ni + 2, d->nj + 2, d->nk + 2, 0, 0};
    for (int k = 1; k <= d->nk; ++k)
        for (int j = 1; j <= d->nj; ++j)
            for (int i = 1; i <= d->ni; ++i) {
                size_t a = I3(i, j, k);
                if (CF[a] == 1)
                    Flux[a] = Flux[a] + wgt * (Cc[a] * P[a - 2 * s] + Cd[a] * P[a - s] + Ce[a] * P[a] +
                                               Cf[a] * P[a + s]);
            }
}

/* CalcVerticalDifFlux, AD:3668-3711 */
static void cell_dif_flux_z(const ora_domain* d, double wgt, const double* Kz, const double* P, double* Flux)
{
    ora_ext X = {d->ni + 2, d->nj + 2, d->nk + 2, 0, 0};
    for (int k = 1; k <= d->nk; ++k)
        for (int j = 1; j <= d->nj; ++j)
            for (int i = 1; i <= d->ni; ++i) {
                size_t a = I3(i, j, k), am = I3(i, j, k - 1);
                if (d->ComputeFacesW3D[a] == 1)
                    Flux[a] = Flux[a] - wgt * Kz[a] * d->DUX[I2(i, j)] * d->DVY[I2(i, j)] / d->DZZ[am] *
                                            (P[a] - P[am]);
            }
}

#define ORA_FILL_INT (-9999999)   /* FillValueInt, ModuleGlobalData.F90:131 */
#define ORA_DISCH_UNIFORM 5       /* DischUniform_, ModuleGlobalData.F90:1006 */

/* the discharge cells' layer range: the given layer, or for a uniform
 * vertical distribution Kmin..Kmax with "not given" read as KFloorZ and KUB */
static void disch_layers(const ora_domain* d, int dis, int n, int* kmin, int* kmax)
{
    const ora_discharges* q = d->Disch;
    ora_ext X = {d->ni + 2, d->nj + 2, d->nk + 2, 0, 0};
    if (q->vert[dis] == ORA_DISCH_UNIFORM) {
        *kmin = q->Kmin[n] == ORA_FILL_INT ? d->KFloorZ[I2(q->I[n], q->J[n])] : q->Kmin[n];
        *kmax = q->Kmax[n] == ORA_FILL_INT ? d->nk : q->Kmax[n];
    } else {
        *kmin = *kmax = q->K[n];
    }
}

/* cells of the work box, layers 1..KUB (the reference does not check) */
static int disch_valid(const ora_domain* d)
{
    const ora_discharges* q = d->Disch;
    if (!q) return 1;
    if (q->number < 0 || (q->number > 0 && (!q->nCells || !q->ignore || !q->bypass || !q->vert))) return 0;
    int n = 0;
    for (int dis = 0; dis < q->number; ++dis) {
        if (q->ignore[dis]) continue;
        for (int nc = 0; nc < q->nCells[dis]; ++nc, ++n) {
            if (q->I[n] < 1 || q->I[n] > d->ni || q->J[n] < 1 || q->J[n] > d->nj) return 0;
            int kmin, kmax;
            disch_layers(d, dis, n, &kmin, &kmax);
            if (kmin < 1 || kmax > d->nk) return 0;
        }
    }
    return 1;
}

/* Discharges, AD:4025-4128: after VolumeVariation, each discharge cell adds
 * its inflow to TI, or a withdrawal to E (times DischConcMF); a uniform
 * discharge spreads its flow over Kmin..Kmax by layer thickness.  A closed
 * cell takes the inflow over the old mass.  In the reference's order. */
static void discharges(const ora_domain* d, const double* P, double* TI, double* E, double DT)
{
    const ora_discharges* q = d->Disch;
    ora_ext X = {d->ni + 2, d->nj + 2, d->nk + 2, 0, 0};
    int n = 0;
    for (int dis = 0; dis < q->number; ++dis) {
        if (q->ignore[dis]) continue;
        const int uniform = q->vert[dis] == ORA_DISCH_UNIFORM;
        for (int nc = 0; nc < q->nCells[dis]; ++nc, ++n) {
            const int i = q->I[n], j = q->J[n];
            int kmin, kmax;
            disch_layers(d, dis, n, &kmin, &kmax);
            double WaterColumn = 0.0;
            for (int k = kmin; k <= kmax; ++k) WaterColumn = WaterColumn + d->DWZ[I3(i, j, k)];
            for (int k = kmin; k <= kmax; ++k) {
                const size_t a = I3(i, j, k);
                const double DT_V = DT / d->VolumeZ[a];
                const double Flow = uniform ? q->Flow[n] * d->DWZ[a] / WaterColumn : q->Flow[n];
                if (d->OpenPoints3D[a] == 1) {
                    if (q->bypass[dis]) TI[a] = TI[a] + Flow * DT_V * q->Conc[n];
                    else if (Flow > 0.) TI[a] = TI[a] + Flow * DT_V * q->Conc[n];
                    else E[a] = E[a] - Flow * DT_V * q->ConcMF[n];
                } else if (Flow > 0.) {
                    TI[a] = P[a] * d->VolumeZOld[a] / d->VolumeZ[a] + Flow * DT_V * q->Conc[n];
                }
            }
        }
    }
}

/* NoAdvFlux: the face coefficients of the masked faces of the work box are
 * zeroed after their lines are formed (AD:4434-4443, AD:4804-4813); from
 * KFloorZ for the vertical ones, on columns open at KUB (AD:3004-3013) */
static void noflux_zero(const ora_domain* d, const int* NF, int vertical, double* C, double* D, double* E,
                        double* F)
{
    ora_ext X = {d->ni + 2, d->nj + 2, d->nk + 2, 0, 0};
    for (int j = 1; j <= d->nj; ++j)
        for (int i = 1; i <= d->ni; ++i) {
            int k0 = 1;
            if (vertical) {
                if (d->OpenPoints3D[I3(i, j, d->nk)] != 1) continue;
                k0 = d->KFloorZ[I2(i, j)] < 0 ? 0 : d->KFloorZ[I2(i, j)];
            }
            for (int k = k0; k <= d->nk; ++k) {
                size_t a = I3(i, j, k);
                if (NF[a] == 1) C[a] = D[a] = E[a] = F[a] = 0.;
            }
        }
}

int ora_step_f64(const ora_domain* d, double* PROP, const double* ReferenceProp,
                 const mohid_ad_params* p, ora_work* work, int nthreads)
{
    int st = validate(d, PROP, p, ReferenceProp);
    if (st) return st;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    const int ni = d->ni, nj = d->nj, nk = d->nk;
    ora_ext X = {ni + 2, nj + 2, nk + 2, 0, 0};
    X.n3 = (size_t)X.NI * X.NJ * X.NK;
    X.n2 = (size_t)X.NI * X.NJ;
    const double DT = p->DTProp;
    const int *CFU = d->ComputeFacesU3D, *CFV = d->ComputeFacesV3D, *CFW = d->ComputeFacesW3D;
    const int *OP = d->OpenPoints3D;
    const double *V = d->VolumeZ, *P = PROP;

    ora_work* own = NULL;
    if (!work) { own = work = ora_work_new(ni, nj, nk); if (!work) return MOHID_AD_ERR_ALLOC; }
    if (work->ni != ni || work->nj != nj || work->nk != nk) return MOHID_AD_ERR_BOUNDS;
    const int cflux = p->CellFluxes != 0;
    if (cflux && !ora_work_fluxes(work)) { ora_work_free(own); return MOHID_AD_ERR_ALLOC; }
    /* AdvectionNudging: the advective terms go to AdvectionTi/D/E/F first */
    const int nudge = p->AdvectionNudging != 0;
    if (nudge && !ora_work_nudge(work)) { ora_work_free(own); return MOHID_AD_ERR_ALLOC; }
    ora_work w = *work;
    /* the Nudge routines ignore the NoAdvFlux masks (AD:4586-4733, 4957-5118, 3211-3350) */
    const int noAdv = p->NoAdvFlux && !nudge;
    int err = 0, zeroH = 0;

    /* Convert_Dif_Vertical, AD:2364-2443: do k = KLB+1,KUB / OMP DO j / do i */
    #pragma omp parallel
    for (int k = 2; k <= nk; ++k) {
        #pragma omp for schedule(dynamic, 1)
        for (int j = 1; j <= nj; ++j)
            for (int i = 1; i <= ni; ++i) {
                size_t a = I3(i, j, k);
                if (CFW[a] == 1) w.Kz[a] = p->SchmidtCoef_V * d->Diff_V[a] + p->SchmidtBackground_V;
            }
    }
    if (p->NullDif) {
        #pragma omp parallel
        for (int k = 2; k <= nk; ++k) {
            #pragma omp for schedule(dynamic, 1)
            for (int j = 1; j <= nj; ++j)
                for (int i = 1; i <= ni; ++i) {
                    size_t a = I3(i, j, k);
                    if (CFW[a] == 1 && d->Wflux_Z[a] == 0.) w.Kz[a] = 0.;
                }
        }
    }
    /* Convert_Visc_Dif_Horizontal, AD:2453-2595 */
    #pragma omp parallel
    {
        for (int k = 1; k <= nk; ++k) {
            #pragma omp for schedule(dynamic, 1) nowait
            for (int j = 1; j <= nj; ++j)
                for (int i = 1; i <= ni; ++i) {
                    size_t a = I3(i, j, k);
                    if (CFU[a] == 1)
                        w.Kx[a] = p->schmidt_H * (d->Visc_H[a] * d->DUX[I2(i, j - 1)] +
                                                  d->Visc_H[I3(i, j - 1, k)] * d->DUX[I2(i, j)]) /
                                  (d->DUX[I2(i, j)] + d->DUX[I2(i, j - 1)]);
                }
        }
        for (int k = 1; k <= nk; ++k) {
            #pragma omp for schedule(dynamic, 1)
            for (int j = 1; j <= nj; ++j)
                for (int i = 1; i <= ni; ++i) {
                    size_t a = I3(i, j, k);
                    if (CFV[a] == 1)
                        w.Ky[a] = p->schmidt_H * (d->Visc_H[a] * d->DVY[I2(i - 1, j)] +
                                                  d->Visc_H[I3(i - 1, j, k)] * d->DVY[I2(i, j)]) /
                                  (d->DVY[I2(i, j)] + d->DVY[I2(i - 1, j)]);
                }
        }
        if (p->NoDifFlux) {                      /* AD:2496-2500, AD:2527-2531 */
            for (int k = 1; k <= nk; ++k) {
                #pragma omp for schedule(dynamic, 1)
                for (int j = 1; j <= nj; ++j)
                    for (int i = 1; i <= ni; ++i) {
                        size_t a = I3(i, j, k);
                        if (CFU[a] == 1 && d->NoFluxU[a] == 1) w.Kx[a] = 0.;
                        if (CFV[a] == 1 && d->NoFluxV[a] == 1) w.Ky[a] = 0.;
                    }
            }
        }
        if (p->NullDif) {
            for (int k = 1; k <= nk; ++k) {
                #pragma omp for schedule(dynamic, 1)
                for (int j = 1; j <= nj; ++j)
                    for (int i = 1; i <= ni; ++i) {
                        size_t a = I3(i, j, k);
                        if (CFU[a] == 1 && d->Wflux_X[a] == 0.) w.Kx[a] = 0.;
                        if (CFV[a] == 1 && d->Wflux_Y[a] == 0.) w.Ky[a] = 0.;
                    }
            }
        }
    }

    /* AdvectionDiffusion cd8 (AD:1439-1456) and AdvectionDiffusionIteration
     * init (AD:1660-1697): D=0, E=1, F=0, TI=0 and the flux-coefficient
     * arrays zero over the Size box. */
    fill3(X, w.D, 0.); fill3(X, w.E, 1.); fill3(X, w.F, 0.); fill3(X, w.TI, 0.);
    {
        double* c12[12] = {w.XC, w.XD, w.XE, w.XF, w.YC, w.YD, w.YE, w.YF, w.VC, w.VD, w.VE, w.VF};
        for (int s = 0; s < 12; ++s) fill3(X, c12[s], 0.);
    }
    if (cflux) {                                 /* AD:1458-1468 */
        double* f6[6] = {w.FAX, w.FAY, w.FAZ, w.FDX, w.FDY, w.FDZ};
        for (int s = 0; s < 6; ++s) fill3(X, f6[s], 0.);
    }

    /* VolumeVariation, AD:3966-4021: do k / OMP DO j / do i */
    #pragma omp parallel
    for (int k = 1; k <= nk; ++k) {
        #pragma omp for schedule(dynamic, 1)
        for (int j = 1; j <= nj; ++j)
            for (int i = 1; i <= ni; ++i) {
                size_t a = I3(i, j, k);
                if (OP[a] == 1) {
                    w.TI[a] = P[a] * (d->VolumeZOld[a] / V[a]);
                    if (k == nk) {
                        double DT_V = DT / V[a];
                        w.E[a] = 1.0 + DT_V * d->Wflux_Z[I3(i, j, k + 1)];
                    }
                } else {
                    w.TI[a] = P[a];
                }
            }
    }
    if (d->Disch) discharges(d, P, w.TI, w.E, DT);   /* AD:1702 */

    if (!p->Vertical1D) {
        /* HorizontalDiffusionXX, AD:5156-5214: OMP DO k / do j / do i */
        #pragma omp parallel for schedule(dynamic, 1)
        for (int k = 1; k <= nk; ++k)
            for (int j = 1; j <= nj; ++j)
                for (int i = 1; i <= ni; ++i) {
                    size_t a = I3(i, j, k), am = I3(i, j - 1, k);
                    if (CFU[a] == 1) {
                        double AuxJ = w.Kx[a] * d->AreaU[a] / d->DZX[I2(i, j - 1)];
                        w.TI[am] = w.TI[am] + AuxJ * DT / V[am] * (P[a] - P[am]);
                        w.TI[a] = w.TI[a] - AuxJ * DT / V[a] * (P[a] - P[am]);
                    }
                }
        if (cflux)                               /* CalcHorizontalDifFluxXX, AD:3784-3825 */
            for (int k = 1; k <= nk; ++k)
                for (int j = 1; j <= nj; ++j)
                    for (int i = 1; i <= ni; ++i) {
                        size_t a = I3(i, j, k), am = I3(i, j - 1, k);
                        if (CFU[a] == 1)
                            w.FDX[a] = w.FDX[a] - w.Kx[a] * d->AreaU[a] / d->DZX[I2(i, j - 1)] * (P[a] - P[am]);
                    }
        /* HorizontalDiffusionYY, AD:5313-5365: do k / OMP DO j / do i */
        if (!p->XZFlow) {
            #pragma omp parallel
            for (int k = 1; k <= nk; ++k) {
                #pragma omp for schedule(dynamic, 1)
                for (int j = 1; j <= nj; ++j)
                    for (int i = 1; i <= ni; ++i) {
                        size_t a = I3(i, j, k), am = I3(i - 1, j, k);
                        if (CFV[a] == 1) {
                            double AuxI = w.Ky[a] * d->AreaV[a] / d->DZY[I2(i - 1, j)];
                            w.TI[am] = w.TI[am] + AuxI * DT / V[am] * (P[a] - P[am]);
                            w.TI[a] = w.TI[a] - AuxI * DT / V[a] * (P[a] - P[am]);
                        }
                    }
            }
            if (cflux)                           /* CalcHorizontalDifFluxYY, AD:3871-3911 */
                for (int k = 1; k <= nk; ++k)
                    for (int j = 1; j <= nj; ++j)
                        for (int i = 1; i <= ni; ++i) {
                            size_t a = I3(i, j, k), am = I3(i - 1, j, k);
                            if (CFV[a] == 1)
                                w.FDY[a] = w.FDY[a] - w.Ky[a] * d->AreaV[a] / d->DZY[I2(i - 1, j)] * (P[a] - P[am]);
                        }
        }

        /* HorizontalAdvection AD:4151-4165: with AdvectionNudging the
         * explicit updates go to AdvectionTi, zeroed first (the _Nudge
         * variants of XX and YY, AD:4586-4733 and AD:4957-5118) */
        double* TIa = nudge ? w.ATi : w.TI;
        if (nudge) { fill3(X, w.ATi, 0.); fill3(X, w.AD, 0.); fill3(X, w.AE, 0.); fill3(X, w.AF, 0.); }
        /* HorizontalAdvectionXX, AD:4368-4540: coefficients per line (i,:,k)
         * (do k / OMP DO i), faces j = JLB..JUB after the dummy-index shift;
         * explicit update OMP DO k / do j / do i. */
        #pragma omp parallel reduction(|:err)
        for (int k = 1; k <= nk; ++k) {
            #pragma omp for schedule(dynamic, 1)
            for (int i = 1; i <= ni; ++i)
                err |= advection_line(1, nj, DT, d->DUX + I2(i, 0), (size_t)X.NI, P, d->Wflux_X, V,
                                      OP, I3(i, 0, k), (size_t)X.NI, w.XC, w.XD, w.XE, w.XF,
                                      p->AdvMethodH, p->TVDLimitationH, p->VolumeRelMax,
                                      p->Upwind2H);
        }
        if (err) goto fail;
        if (noAdv) noflux_zero(d, d->NoFluxU, 0, w.XC, w.XD, w.XE, w.XF);
        if (p->ImpExp_AdvXX == 0.) {
        #pragma omp parallel for schedule(dynamic, 1)
        for (int k = 1; k <= nk; ++k)
            for (int j = 1; j <= nj; ++j)
                for (int i = 1; i <= ni; ++i) {
                    size_t a = I3(i, j, k);
                    if (CFU[a] == 1) {
                        size_t am = I3(i, j - 1, k);
                        double Fx = w.XC[a] * P[I3(i, j - 2, k)] + w.XD[a] * P[am] +
                                    w.XE[a] * P[a] + w.XF[a] * P[I3(i, j + 1, k)];
                        TIa[a] = TIa[a] + Fx * DT / V[a];
                        TIa[am] = TIa[am] - Fx * DT / V[am];
                    }
                }
        if (cflux)                               /* AD:4531-4537 */
            cell_adv_flux(d, CFU, X.NI, 1. - p->ImpExp_AdvXX, w.XC, w.XD, w.XE, w.XF, P, w.FAX);
        } else {
            /* implicit, AD:4490-4515: OMP DO k / do j / do i */
            #pragma omp parallel for schedule(dynamic, 1)
            for (int k = 1; k <= nk; ++k)
                for (int j = 1; j <= nj; ++j)
                    for (int i = 1; i <= ni; ++i) {
                        size_t a = I3(i, j, k);
                        if (CFU[a] == 1) {
                            size_t am = I3(i, j - 1, k);
                            double DT2 = DT / V[a], DT1 = DT / V[am];
                            w.D[a] = w.D[a] - w.XD[a] * DT2;
                            w.E[a] = w.E[a] - w.XE[a] * DT2;
                            w.E[am] = w.E[am] + w.XD[a] * DT1;
                            w.F[am] = w.F[am] + w.XE[a] * DT1;
                        }
                    }
        }
        /* HorizontalAdvectionYY, AD:4739-4910: do k / OMP DO j for both parts */
        if (!p->XZFlow) {
            #pragma omp parallel reduction(|:err)
            for (int k = 1; k <= nk; ++k) {
                #pragma omp for schedule(dynamic, 1)
                for (int j = 1; j <= nj; ++j)
                    err |= advection_line(1, ni, DT, d->DVY + I2(0, j), 1, P, d->Wflux_Y, V, OP,
                                          I3(0, j, k), 1, w.YC, w.YD, w.YE, w.YF,
                                          p->AdvMethodH, p->TVDLimitationH, p->VolumeRelMax,
                                          p->Upwind2H);
            }
            if (err) goto fail;
            if (noAdv) noflux_zero(d, d->NoFluxV, 0, w.YC, w.YD, w.YE, w.YF);
            if (p->ImpExp_AdvYY == 0.) {
            #pragma omp parallel
            for (int k = 1; k <= nk; ++k) {
                #pragma omp for schedule(dynamic, 1)
                for (int j = 1; j <= nj; ++j)
                    for (int i = 1; i <= ni; ++i) {
                        size_t a = I3(i, j, k);
                        if (CFV[a] == 1) {
                            size_t am = I3(i - 1, j, k);
                            double Fy = w.YC[a] * P[I3(i - 2, j, k)] + w.YD[a] * P[am] +
                                        w.YE[a] * P[a] + w.YF[a] * P[I3(i + 1, j, k)];
                            TIa[a] = TIa[a] + Fy * DT / V[a];
                            TIa[am] = TIa[am] - Fy * DT / V[am];
                        }
                    }
            }
            if (cflux)                           /* AD:4900-4906 */
                cell_adv_flux(d, CFV, 1, 1. - p->ImpExp_AdvYY, w.YC, w.YD, w.YE, w.YF, P, w.FAY);
            } else {
                /* implicit, AD:4855-4880: do k / do j / do i */
                for (int k = 1; k <= nk; ++k)
                    for (int j = 1; j <= nj; ++j)
                        for (int i = 1; i <= ni; ++i) {
                            size_t a = I3(i, j, k);
                            if (CFV[a] == 1) {
                                size_t am = I3(i - 1, j, k);
                                double DT2 = DT / V[a], DT1 = DT / V[am];
                                w.D[a] = w.D[a] - w.YD[a] * DT2;
                                w.E[a] = w.E[a] - w.YE[a] * DT2;
                                w.E[am] = w.E[am] + w.YD[a] * DT1;
                                w.F[am] = w.F[am] + w.YE[a] * DT1;
                            }
                        }
            }
        }
        /* HorizontalAdvection AD:4167-4254: in 3-D the implicit direction is
         * solved now (THOMAS_3D into PROP), and the vertical step starts again
         * from D = 0, E = 1, F = 0, TI = PROP over the Size box */
        if ((p->ImpExp_AdvXX == 1. || p->ImpExp_AdvYY == 1.) && nk > 1) {
            zeroH |= thomas_3d(d, p->ImpExp_AdvXX == 1., w.D, w.E, w.F, w.TI, PROP);
            fill3(X, w.D, 0.); fill3(X, w.E, 1.); fill3(X, w.F, 0.);
            #pragma omp parallel for schedule(static)
            for (int k = 0; k < X.NK; ++k)
                for (size_t q = (size_t)k * X.n2; q < (size_t)(k + 1) * X.n2; ++q) w.TI[q] = PROP[q];
        }
    }

    if (nk > 1) {
        /* VerticalDiffusion, AD:2708-2784: do k / OMP DO j / do i */
        const double ie = p->ImpExp_DifV;
        #pragma omp parallel
        for (int k = 1; k <= nk; ++k) {
            #pragma omp for schedule(dynamic, 1)
            for (int j = 1; j <= nj; ++j)
                for (int i = 1; i <= ni; ++i) {
                    size_t a = I3(i, j, k), am = I3(i, j, k - 1);
                    int sd = d->SmallDepths ? d->SmallDepths[I2(i, j)] : 0;
                    if (CFW[a] == 1 && !sd) {
                        double AuxK = w.Kz[a] * d->DUX[I2(i, j)] * d->DVY[I2(i, j)] / d->DZZ[am];
                        if (p->NoDifFlux && d->NoFluxW[a] == 1) AuxK = 0.;   /* AD:2741-2745 */
                        double Aux1 = AuxK * DT / V[am];
                        double Aux2 = AuxK * DT / V[a];
                        w.E[am] = w.E[am] + Aux1 * ie;
                        w.F[am] = w.F[am] - Aux1 * ie;
                        w.TI[am] = w.TI[am] + Aux1 * (P[a] - P[am]) * (1. - ie);
                        w.D[a] = w.D[a] - Aux2 * ie;
                        w.E[a] = w.E[a] + Aux2 * ie;
                        w.TI[a] = w.TI[a] - Aux2 * (P[a] - P[am]) * (1. - ie);
                    }
                }
        }
        if (cflux && ie < 1.) cell_dif_flux_z(d, 1. - ie, w.Kz, P, w.FDZ);   /* AD:2776-2777 */

        if (!p->Vertical1D) {
            /* VerticalAdvection, AD:2941-3140: coefficients per column with
             * OpenPoints3D(i,j,KUB) == 1 (OMP DO j / do i), faces k = KLB..KUB
             * after the dummy-index shift. */
            #pragma omp parallel for schedule(dynamic, 1) reduction(|:err)
            for (int j = 1; j <= nj; ++j)
                for (int i = 1; i <= ni; ++i)
                    if (OP[I3(i, j, nk)] == 1)
                        err |= advection_line(1, nk, DT, d->DWZ + I3(i, j, 0), X.n2, P,
                                              d->Wflux_Z, V, OP, I3(i, j, 0), X.n2,
                                              w.VC, w.VD, w.VE, w.VF, p->AdvMethodV,
                                              p->TVDLimitationV, p->VolumeRelMax, p->Upwind2V);
            if (err) goto fail;
            if (noAdv) noflux_zero(d, d->NoFluxW, 1, w.VC, w.VD, w.VE, w.VF);
            /* VerticalAdvection_Nudge (AD:3211-3350): explicit to AdvectionTi,
             * implicit to AdvectionD/E/F by layers whatever Docycle_method */
            double* TIv = nudge ? w.ATi : w.TI;

            if (p->ImpExp_AdvV == 0.) {
                /* explicit, AD:3036-3063: do k / OMP DO j / do i */
                #pragma omp parallel
                for (int k = 1; k <= nk; ++k) {
                    #pragma omp for schedule(dynamic, 1)
                    for (int j = 1; j <= nj; ++j)
                        for (int i = 1; i <= ni; ++i) {
                            size_t a = I3(i, j, k), am = I3(i, j, k - 1);
                            if (CFW[a] == 1) {
                                double Fz = w.VC[a] * P[I3(i, j, k - 2)] + w.VD[a] * P[am] +
                                            w.VE[a] * P[a] + w.VF[a] * P[I3(i, j, k + 1)];
                                TIv[am] = TIv[am] - Fz * DT / V[am];
                                TIv[a] = TIv[a] + Fz * DT / V[a];
                            }
                        }
                }
            } else if (nudge) {
                /* implicit, AD:3302-3331: do k / OMP DO j / do i */
                for (int k = 1; k <= nk; ++k)
                    for (int j = 1; j <= nj; ++j)
                        for (int i = 1; i <= ni; ++i) {
                            size_t a = I3(i, j, k), am = I3(i, j, k - 1);
                            if (CFW[a] == 1) {
                                double DT1 = DT / V[am];
                                double DT2 = DT / V[a];
                                w.AD[a] = w.AD[a] - w.VD[a] * DT2;
                                w.AE[a] = w.AE[a] - w.VE[a] * DT2;
                                w.AE[am] = w.AE[am] + w.VD[a] * DT1;
                                w.AF[am] = w.AF[am] + w.VE[a] * DT1;
                            }
                        }
            } else if (p->Docycle_method == 1) {
                /* implicit, column cycle, AD:3070-3093: OMP DO j / do i / do k */
                #pragma omp parallel for schedule(dynamic, 1)
                for (int j = 1; j <= nj; ++j)
                    for (int i = 1; i <= ni; ++i)
                        if (CFW[I3(i, j, nk)] == 1) {
                            int kb = d->KFloorZ[I2(i, j)];
                            double Vb = V[I3(i, j, kb)];
                            for (int k = kb + 1; k <= nk; ++k) {
                                size_t a = I3(i, j, k), am = I3(i, j, k - 1);
                                double DT1 = DT / Vb;
                                double DT2 = DT / V[a];
                                Vb = V[a];
                                w.D[a] = w.D[a] - w.VD[a] * DT2;
                                w.E[a] = w.E[a] - w.VE[a] * DT2;
                                w.E[am] = w.E[am] + w.VD[a] * DT1;
                                w.F[am] = w.F[am] + w.VE[a] * DT1;
                            }
                        }
            } else {
                /* implicit, layer cycle, AD:3094-3117: do k / OMP DO j / do i */
                #pragma omp parallel
                for (int k = 1; k <= nk; ++k) {
                    #pragma omp for schedule(dynamic, 1)
                    for (int j = 1; j <= nj; ++j)
                        for (int i = 1; i <= ni; ++i) {
                            size_t a = I3(i, j, k), am = I3(i, j, k - 1);
                            if (CFW[a] == 1) {
                                double DT1 = DT / V[am];
                                double DT2 = DT / V[a];
                                w.D[a] = w.D[a] - w.VD[a] * DT2;
                                w.E[a] = w.E[a] - w.VE[a] * DT2;
                                w.E[am] = w.E[am] + w.VD[a] * DT1;
                                w.F[am] = w.F[am] + w.VE[a] * DT1;
                            }
                        }
                }
            }
            if (cflux && p->ImpExp_AdvV < 1.)    /* AD:3128-3135 */
                cell_adv_flux(d, CFW, (long long)X.n2, 1. - p->ImpExp_AdvV, w.VC, w.VD, w.VE, w.VF, P, w.FAZ);
        }
    }

    if (nudge) {
        /* AdvectionNudging, AD:1989-2068: the advective terms enter scaled
         * by n = min(in, jn) / nCells near the edges, in / jn the distance in
         * cells to the nearer i / j edge.  A cell near only one pair of edges
         * reads the other distance from the last cell that set it: the
         * reference keeps in / jn as OpenMP-private variables across the loop,
         * so its result there depends on which cells a thread ran before.
         * This restatement runs the loop in order on one thread, where that
         * value is always nCells. */
        const int nc = p->AdvectionNudgingCells;
        int in_ = 0, jn_ = 0;                    /* max(0, i - ILB + 1) etc., ILB = JLB = 1 */
        for (int j = 1; j <= nj; ++j)
            for (int i = 1; i <= ni; ++i) {
                int cell = 0;
                if (i < nc + 1) { cell = 1; in_ = i > 0 ? i : 0; }
                else if (i > ni - nc) { cell = 1; in_ = ni - i + 1 > 0 ? ni - i + 1 : 0; }
                if (j < nc + 1) { cell = 1; jn_ = j > 0 ? j : 0; }
                else if (j > nj - nc) { cell = 1; jn_ = nj - j + 1 > 0 ? nj - j + 1 : 0; }
                double n;
                if (cell) { n = (double)(in_ < jn_ ? in_ : jn_); n = n / nc; }
                else n = 1.0;
                for (int k = 1; k <= nk; ++k) {
                    size_t a = I3(i, j, k);
                    if (OP[a] == 1) {
                        w.TI[a] = w.TI[a] + n * w.ATi[a];
                        w.D[a] = w.D[a] + n * w.AD[a];
                        w.E[a] = w.E[a] + n * w.AE[a];
                        w.F[a] = w.F[a] + n * w.AF[a];
                    }
                }
            }
    }

    if (ReferenceProp) {
        /* OpenBoundaryCondition, AD:5369-5672 (serial); FluxAtOpenBoundary,
         * AD:5680-5742 (OMP DO j / do i / do k). */
        const int bc = p->BoundaryCondition;
        const double TdecAux = 1.0 / (1.0 + p->DecayTime / DT);
        if (bc == MOHID_BC_MASS_CONSERVATION || bc == MOHID_BC_MASS_CONSERV_NULLGRAD || bc == MOHID_BC_ORLANSKI) {
            #pragma omp parallel for schedule(dynamic, 1)
            for (int j = 1; j <= nj; ++j)
                for (int i = 1; i <= ni; ++i)
                    if (d->BoundaryPoints2D[I2(i, j)] == 1) {
                        int kl = abs(d->KFloorZ[I2(i, j)]);
                        for (int k = kl; k <= nk; ++k) {
                            size_t a = I3(i, j, k);
                            w.WFOB[a] = d->Wflux_X[a] * CFU[a] -
                                        d->Wflux_X[I3(i, j + 1, k)] * CFU[I3(i, j + 1, k)] +
                                        d->Wflux_Y[a] * CFV[a] -
                                        d->Wflux_Y[I3(i + 1, j, k)] * CFV[I3(i + 1, j, k)] +
                                        d->Wflux_Z[a] * CFW[a] -
                                        d->Wflux_Z[I3(i, j, k + 1)] * CFW[I3(i, j, k + 1)] -
                                        (V[a] - d->VolumeZOld[a]) / DT;
                        }
                    }
        }
        /* Orlanski: PROPOld(:,:,:) = PROP(:,:,:) (AD:5428-5429); the field
         * itself is updated in place at the exterior points */
        double* PROPOld = NULL;
        double* ownOld = NULL;
        if (bc == MOHID_BC_ORLANSKI) {
            PROPOld = d->PROPOld;
            if (!PROPOld) PROPOld = ownOld = (double*)malloc(sizeof(double) * X.n3);
            if (!PROPOld) { ora_work_free(own); return MOHID_AD_ERR_ALLOC; }
            memcpy(PROPOld, PROP, sizeof(double) * X.n3);
        }
        for (int j = 1; j <= nj; ++j)
            for (int i = 1; i <= ni; ++i) {
                if (d->BoundaryPoints2D[I2(i, j)] != 1) continue;
                int kl = abs(d->KFloorZ[I2(i, j)]);
                for (int k = kl; k <= nk; ++k) {
                    size_t a = I3(i, j, k);
                    if (OP[a] != 1) continue;
                    double DT_V = DT / V[a];
                    double Ext;
                    if (bc == MOHID_BC_ORLANSKI) {
                        /* AD:5504-5567, then the inflow / outflow terms of MassConservation */
                        const double VelBound = w.WFOB[a] * DT_V;
                        int di = 0, dj = 0, en = 0, ie = 0, je = 0;
                        orlanski_normal(ni, nj, i, j, &di, &dj, &en, &ie, &je);   /* checked in validate */
                        const double LimitMax = 10. * DT / (d->DUX[I2(i, j)] + d->DVY[I2(i, j)]) * 2;
                        Ext = orlanski_celerity_2d(X, PROP, PROPOld, ReferenceProp, OP, 1, ni, 1, nj, di, dj, ie, je,
                                                   k, en, LimitMax, DT, VelBound);
                        if (w.WFOB[a] < 0.0) w.TI[a] = w.TI[a] - w.WFOB[a] * Ext * DT_V;
                        else w.E[a] = w.E[a] + w.WFOB[a] * DT_V;
                        continue;
                    }
                    if (bc == MOHID_BC_IMPOSED_VALUE || bc == MOHID_BC_SUBMODEL) {
                        double A1 = OP[I3(i + 1, j, k)] * (1 - d->BoundaryPoints2D[I2(i + 1, j)]);
                        double A2 = OP[I3(i - 1, j, k)] * (1 - d->BoundaryPoints2D[I2(i - 1, j)]);
                        double A3 = OP[I3(i, j + 1, k)] * (1 - d->BoundaryPoints2D[I2(i, j + 1)]);
                        double A4 = OP[I3(i, j - 1, k)] * (1 - d->BoundaryPoints2D[I2(i, j - 1)]);
                        double P1 = P[I3(i + 1, j, k)], P2 = P[I3(i - 1, j, k)];
                        double P3 = P[I3(i, j + 1, k)], P4 = P[I3(i, j - 1, k)];
                        double At = A1 + A2 + A3 + A4;
                        if (At > 0) {
                            double Int = (P1 * A1 + P2 * A2 + P3 * A3 + P4 * A4) / At;
                            Ext = Int * (1.0 - TdecAux) + ReferenceProp[a] * TdecAux;
                        } else {
                            Ext = ReferenceProp[a];
                        }
                        w.TI[a] = Ext;
                        w.D[a] = 0.0; w.E[a] = 1.0; w.F[a] = 0.0;
                    } else if (bc == MOHID_BC_NULL_GRADIENT || bc == MOHID_BC_CYCLIC) {
                        /* AD:5645-5650: the row keeps the old value; the
                         * boundary is set after the solve */
                        w.TI[a] = P[a];
                        w.D[a] = 0.0; w.E[a] = 1.0; w.F[a] = 0.0;
                    } else if (bc == MOHID_BC_MASS_CONSERV_NULLGRAD) {
                        /* AD:5603-5631: inflow takes the interior mean across
                         * compute faces (old values), outflow leaves implicitly */
                        if (w.WFOB[a] < 0.0) {
                            double bprop;
                            w.TI[a] = null_grad_prop(d, P, i, j, k, &bprop) ? bprop : P[a];
                            w.E[a] = 1.0; w.D[a] = 0.0; w.F[a] = 0.0;
                        } else {
                            w.E[a] = w.E[a] + w.WFOB[a] * DT_V;
                        }
                    } else { /* MassConservation */
                        double Int = P[a];
                        Ext = Int * (1.0 - TdecAux) + ReferenceProp[a] * TdecAux;
                        if (w.WFOB[a] < 0.0) w.TI[a] = w.TI[a] - w.WFOB[a] * Ext * DT_V;
                        else w.E[a] = w.E[a] + w.WFOB[a] * DT_V;
                    }
                }
            }
        free(ownOld);
    }

    /* SetMatrixValue(TICOEF3, Size, Null_Real, LandPoints3D), AD:1753 */
    #pragma omp parallel for schedule(dynamic, 1)
    for (int k = 0; k < X.NK; ++k)
        for (size_t q = (size_t)k * X.n2; q < (size_t)(k + 1) * X.n2; ++q)
            if (d->LandPoints3D[q] == 1) w.TI[q] = NULL_REAL;

    /* AD:1758-1858: a one-layer domain solves the implicit direction instead of the columns */
    if (nk == 1 && p->ImpExp_AdvXX == 1.)
        st = thomas_3d(d, 1, w.D, w.E, w.F, w.TI, PROP) ? MOHID_AD_ERR_ZERO_PIVOT : 0;
    else if (nk == 1 && p->ImpExp_AdvYY == 1.)
        st = thomas_3d(d, 0, w.D, w.E, w.F, w.TI, PROP) ? MOHID_AD_ERR_ZERO_PIVOT : 0;
    else
        st = ora_thomasz(ni, nj, nk, w.D, w.E, w.F, w.TI, PROP, d->WaterPoints3D);
    if (zeroH && !st) st = MOHID_AD_ERR_ZERO_PIVOT;
    /* AD:1874-1880: whether or not a reference is given */
    if (p->BoundaryCondition == MOHID_BC_NULL_GRADIENT) impose_null_gradient(d, PROP);
    else if (p->BoundaryCondition == MOHID_BC_CYCLIC) cyclic_boundary(d, PROP, ReferenceProp);
    if (cflux) {
        /* implicit parts with the new field, AD:1882-1916 */
        if (p->ImpExp_AdvV > 0. && nk > 1)
            cell_adv_flux(d, CFW, (long long)X.n2, p->ImpExp_AdvV, w.VC, w.VD, w.VE, w.VF, PROP, w.FAZ);
        if (p->ImpExp_DifV > 0. && nk > 1) cell_dif_flux_z(d, p->ImpExp_DifV, w.Kz, PROP, w.FDZ);
        if (p->ImpExp_AdvXX == 1.)
            cell_adv_flux(d, CFU, X.NI, p->ImpExp_AdvXX, w.XC, w.XD, w.XE, w.XF, PROP, w.FAX);
        if (p->ImpExp_AdvYY == 1.)
            cell_adv_flux(d, CFV, 1, p->ImpExp_AdvYY, w.YC, w.YD, w.YE, w.YF, PROP, w.FAY);
    }
    ora_work_free(own);
    return st;
fail:
    ora_work_free(own);
    return MOHID_AD_ERR_OPTION;
}

/* THOMASZ_NewType2, FN:4026-4123, called with the WorkSize bounds (KLB = 1). */
int ora_thomasz(int ni, int nj, int nk, const double* D, const double* E, const double* F,
                const double* TI, double* RES, const int* WaterPoints)
{
    ora_ext X = {ni + 2, nj + 2, nk + 2, 0, 0};
    int zero = 0;
    #pragma omp parallel reduction(|:zero)
    {
        double* W = (double*)malloc(sizeof(double) * (size_t)(nk + 2));
        double* G = (double*)malloc(sizeof(double) * (size_t)(nk + 2));
        #pragma omp for schedule(dynamic, 4)
        for (int j = 1; j <= nj; ++j)
            for (int i = 1; i <= ni; ++i) {
                if (WaterPoints[I3(i, j, nk)] != 1) continue;
                size_t a1 = I3(i, j, 1);
                W[1] = -F[a1] / E[a1];
                G[1] = TI[a1] / E[a1];
                for (int k = 2; k <= nk + 1; ++k) {
                    size_t a = I3(i, j, k);
                    double aux = E[a] + D[a] * W[k - 1];
                    if (fabs(aux) > 0) {
                        W[k] = -F[a] / aux;
                        G[k] = (TI[a] - D[a] * G[k - 1]) / aux;
                    } else {
                        W[k] = 0.; G[k] = 0.; zero = 1;
                    }
                }
                RES[I3(i, j, nk + 1)] = G[nk + 1];
                for (int k = nk; k >= 1; --k)
                    RES[I3(i, j, k)] = W[k] * RES[I3(i, j, k + 1)] + G[k];
            }
        free(W); free(G);
    }
    return zero ? MOHID_AD_ERR_ZERO_PIVOT : 0;
}

/* Neumaier-compensated sum of V*P over water cells (budget diagnostic). */
static double mass_impl(const ora_domain* d, const double* P64, const float* P32)
{
    ora_ext X = {d->ni + 2, d->nj + 2, d->nk + 2, 0, 0};
    double s = 0., c = 0.;
    for (int k = 1; k <= d->nk; ++k)
        for (int j = 1; j <= d->nj; ++j)
            for (int i = 1; i <= d->ni; ++i) {
                size_t a = I3(i, j, k);
                if (d->WaterPoints3D[a] != 1) continue;
                double x = d->VolumeZ[a] * (P64 ? P64[a] : (double)P32[a]);
                double t = s + x;
                if (fabs(s) >= fabs(x)) c += (s - t) + x; else c += (x - t) + s;
                s = t;
            }
    return s + c;
}

double ora_mass(const ora_domain* d, const double* PROP) { return mass_impl(d, PROP, NULL); }
double ora_mass_f32(const ora_domain* d, const float* PROP) { return mass_impl(d, NULL, PROP); }
