/*
 * synth.c -- seeded synthetic inputs for the advection-diffusion step
 * (benchmarks, tests, examples; not on the transport path).
 *
 * No public dataset is involved; these generators restate the reference's
 * geometry, mask and continuity rules so that the inputs are ones MOHID itself
 * could produce:
 *  - sigma / z-level layer thicknesses DWZ, DZZ = (DWZ(k)+DWZ(k+1))/2
 *    (ModuleGeometry.F90:3798), VolumeZ = DWZ*DUX*DVY (ModuleGeometry.F90:4108),
 *    face areas from the minimum adjacent thickness (ModuleGeometry.F90:3867,4278);
 *  - WaterPoints3D = k >= KFloor on water columns, LandPoints3D = 1 - WaterPoints3D
 *    on the work box (ModuleMap.F90:1487-1535); compute faces U/V where both
 *    sides are water; W faces KFloor+1..KUB on columns with a horizontal
 *    compute face at the surface (ModuleMap.F90:1576-1629); OpenPoints3D = any
 *    adjacent compute face (ModuleMap.F90:1760-1790);
 *  - horizontal transports from a streamfunction (divergence free per column),
 *    vertical transport from continuity bottom-up with Wflux_Z(KFloor) = 0
 *    (ModuleHydrodynamic.F90:43270-43349).
 * Arrays are over the Size box (0:ni+1, 0:nj+1[, 0:nk+1]), i fastest.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "synth.h"

#define PI 3.14159265358979323846

typedef struct { int NI, NJ, NK; } ext_t;
#define G3(i, j, k) ((size_t)(i) + (size_t)E.NI * ((size_t)(j) + (size_t)E.NJ * (size_t)(k)))
#define G2(i, j) ((size_t)(i) + (size_t)E.NI * (size_t)(j))

static uint64_t sm64(uint64_t* s)
{
    uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static double urand(uint64_t* s) { return (double)(sm64(s) >> 11) * (1.0 / 9007199254740992.0); }
static double nrand(uint64_t* s)
{
    double u1 = urand(s), u2 = urand(s);
    if (u1 < 1e-300) u1 = 1e-300;
    return sqrt(-2.0 * log(u1)) * cos(2.0 * PI * u2);
}

/* Smooth random 2-D field on the work box (ni x nj, i fastest), normalised to
 * [0,1]: a sum of `nm` plane waves with integer wavenumbers |k| <= kmax and
 * amplitude |k|^-slope.  Evaluated separably: cos(A+B) = cosA cosB - sinA sinB. */
static void smooth2d(int ni, int nj, int nm, int kmax, double slope, uint64_t seed, double* out)
{
    uint64_t s = seed ^ 0x5DEECE66Dull;
    double* ca = (double*)malloc(sizeof(double) * (size_t)nj);
    double* sa = (double*)malloc(sizeof(double) * (size_t)nj);
    double* cb = (double*)malloc(sizeof(double) * (size_t)ni);
    double* sb = (double*)malloc(sizeof(double) * (size_t)ni);
    memset(out, 0, sizeof(double) * (size_t)ni * (size_t)nj);
    for (int m = 0; m < nm; ++m) {
        int kx, ky;
        do {
            kx = (int)(urand(&s) * (2 * kmax + 1)) - kmax;
            ky = (int)(urand(&s) * (2 * kmax + 1)) - kmax;
        } while (kx == 0 && ky == 0);
        double amp = pow(sqrt((double)(kx * kx + ky * ky)), -slope) * (0.5 + urand(&s));
        double ph = 2.0 * PI * urand(&s);
        for (int j = 0; j < nj; ++j) {
            double A = 2.0 * PI * kx * (j + 0.5) / nj + ph;
            ca[j] = cos(A); sa[j] = sin(A);
        }
        for (int i = 0; i < ni; ++i) {
            double B = 2.0 * PI * ky * (i + 0.5) / ni;
            cb[i] = cos(B); sb[i] = sin(B);
        }
        for (int j = 0; j < nj; ++j) {
            double* o = out + (size_t)j * ni;
            for (int i = 0; i < ni; ++i) o[i] += amp * (ca[j] * cb[i] - sa[j] * sb[i]);
        }
    }
    double lo = 1e300, hi = -1e300;
    size_t n = (size_t)ni * nj;
    for (size_t q = 0; q < n; ++q) { if (out[q] < lo) lo = out[q]; if (out[q] > hi) hi = out[q]; }
    double r = (hi > lo) ? 1.0 / (hi - lo) : 0.0;
    for (size_t q = 0; q < n; ++q) out[q] = (out[q] - lo) * r;
    free(ca); free(sa); free(cb); free(sb);
}

static int cmp_d(const void* a, const void* b)
{
    double x = *(const double*)a, y = *(const double*)b;
    return (x > y) - (x < y);
}

static double quantile(const double* f, size_t n, double q)
{
    double* c = (double*)malloc(sizeof(double) * n);
    memcpy(c, f, sizeof(double) * n);
    qsort(c, n, sizeof(double), cmp_d);
    size_t idx = (size_t)(q * (double)(n - 1));
    double v = c[idx];
    free(c);
    return v;
}

int mohid_synth_generate(const mohid_synth_params* gp, mohid_synth_out* o)
{
    const int ni = gp->ni, nj = gp->nj, nk = gp->nk;
    if (ni < 1 || nj < 1 || nk < 1) return -1;
    ext_t E = {ni + 2, nj + 2, nk + 2};
    const size_t n2 = (size_t)E.NI * E.NJ, n3 = n2 * (size_t)E.NK, nw = (size_t)ni * nj;
    uint64_t seed = gp->seed;

    /* zero everything (halo and land stay 0) */
    double* d2[] = {o->DUX, o->DVY, o->DZX, o->DZY, o->depth};
    for (int q = 0; q < 5; ++q) memset(d2[q], 0, sizeof(double) * n2);
    int* i2[] = {o->KFloorZ, o->BoundaryPoints2D, o->WaterPoints2D};
    for (int q = 0; q < 3; ++q) memset(i2[q], 0, sizeof(int) * n2);
    double* d3[] = {o->Wflux_X, o->Wflux_Y, o->Wflux_Z, o->VolumeZOld, o->VolumeZ, o->Visc_H,
                    o->Diff_V, o->AreaU, o->AreaV, o->DZZ, o->DWZ};
    for (int q = 0; q < 11; ++q) memset(d3[q], 0, sizeof(double) * n3);
    int* i3[] = {o->OpenPoints3D, o->LandPoints3D, o->WaterPoints3D, o->ComputeFacesU3D,
                 o->ComputeFacesV3D, o->ComputeFacesW3D};
    for (int q = 0; q < 6; ++q) memset(i3[q], 0, sizeof(int) * n3);

    /* horizontal metrics (uniform Cartesian grid), over the Size box */
    for (size_t q = 0; q < n2; ++q) {
        o->DUX[q] = gp->dx; o->DVY[q] = gp->dy; o->DZX[q] = gp->dx; o->DZY[q] = gp->dy;
    }

    /* land mask and bathymetry on the work box (wb: i fastest, ni x nj) */
    double* fland = (double*)malloc(sizeof(double) * nw);
    double* fbat = (double*)malloc(sizeof(double) * nw);
    int* wet = (int*)malloc(sizeof(int) * nw);
    if (gp->land_kind == 2 || gp->bathy_kind == 2)
        smooth2d(ni, nj, 48, 24, 1.2, seed * 7 + 1, fland);
    else
        smooth2d(ni, nj, 12, 3, 1.0, seed * 7 + 1, fland);
    for (size_t q = 0; q < nw; ++q) wet[q] = 1;
    double qland = 0.0;
    if (gp->land_frac > 0.0) {
        if (gp->land_kind == 0) {
            /* contiguous coastline block on the western edge (j small) */
            uint64_t s = seed * 13 + 5;
            double ph1 = 2 * PI * urand(&s), ph2 = 2 * PI * urand(&s);
            for (int i = 0; i < ni; ++i) {
                double wv = 1.0 + 0.45 * sin(2 * PI * i / ni + ph1) + 0.2 * sin(6 * PI * i / ni + ph2);
                int c = (int)floor(gp->land_frac * nj * wv + 0.5);
                for (int j = 0; j < nj && j < c; ++j) wet[(size_t)j * ni + i] = 0;
            }
        } else {
            qland = quantile(fland, nw, gp->land_frac);
            for (size_t q = 0; q < nw; ++q) wet[q] = fland[q] > qland;
        }
    }
    if (gp->bathy_kind == 0) {
        uint64_t s = seed * 17 + 3;
        double ic = ni * (0.35 + 0.3 * urand(&s)), jc = nj * (0.45 + 0.3 * urand(&s));
        double sg = 0.15 * (ni < nj ? ni : nj);
        for (int j = 0; j < nj; ++j)
            for (int i = 0; i < ni; ++i) {
                double ramp = (nj > 1) ? (double)j / (nj - 1) : 0.0;
                double bump = exp(-((i - ic) * (i - ic) + (j - jc) * (j - jc)) / (2 * sg * sg));
                double h = gp->hmin + (gp->hmax - gp->hmin) * (0.75 * ramp + 0.25 * bump);
                fbat[(size_t)j * ni + i] = h;
            }
    } else if (gp->bathy_kind == 1) {
        smooth2d(ni, nj, 10, 3, 1.0, seed * 19 + 11, fbat);
        for (size_t q = 0; q < nw; ++q) fbat[q] = gp->hmin + (gp->hmax - gp->hmin) * fbat[q];
    } else {
        /* deepening away from the fractal coast */
        double hi = -1e300;
        for (size_t q = 0; q < nw; ++q) if (fland[q] > hi) hi = fland[q];
        for (size_t q = 0; q < nw; ++q) {
            double t = (hi > qland) ? (fland[q] - qland) / (hi - qland) : 1.0;
            if (t < 0) t = 0;
            fbat[q] = gp->hmin + (gp->hmax - gp->hmin) * pow(t, 0.8);
        }
    }

    /* vertical geometry */
    const double dzz = gp->hmax / nk;
    for (int j = 1; j <= nj; ++j)
        for (int i = 1; i <= ni; ++i) {
            size_t w = (size_t)(j - 1) * ni + (i - 1);
            if (!wet[w]) { o->KFloorZ[G2(i, j)] = nk + 1; continue; }
            double H = fbat[w];
            o->WaterPoints2D[G2(i, j)] = 1;
            int kf = 1;
            if (gp->zlevel) {
                int na = (int)ceil(H / dzz - 1e-9);
                if (na < 1) na = 1;
                if (na > nk) na = nk;
                kf = nk - na + 1;
                double bot = H - (na - 1) * dzz;
                if (bot < 0.25 * dzz) bot = 0.25 * dzz;
                for (int k = kf; k <= nk; ++k) o->DWZ[G3(i, j, k)] = (k == kf) ? bot : dzz;
                H = bot + (na - 1) * dzz;
            } else {
                for (int k = 1; k <= nk; ++k) o->DWZ[G3(i, j, k)] = H / nk;
            }
            o->depth[G2(i, j)] = H;
            o->KFloorZ[G2(i, j)] = kf;
            for (int k = kf; k <= nk; ++k) o->WaterPoints3D[G3(i, j, k)] = 1;
        }
    for (int k = 0; k <= nk; ++k)
        for (int j = 0; j < E.NJ; ++j)
            for (int i = 0; i < E.NI; ++i)
                o->DZZ[G3(i, j, k)] = (o->DWZ[G3(i, j, k)] + o->DWZ[G3(i, j, k + 1)]) / 2;
    for (int k = 1; k <= nk; ++k)
        for (int j = 1; j <= nj; ++j)
            for (int i = 1; i <= ni; ++i) {
                size_t a = G3(i, j, k);
                o->LandPoints3D[a] = 1 - o->WaterPoints3D[a];
                o->VolumeZOld[a] = o->DWZ[a] * o->DUX[G2(i, j)] * o->DVY[G2(i, j)];
            }

    /* compute faces */
    for (int k = 1; k <= nk; ++k)
        for (int j = 1; j <= nj; ++j)
            for (int i = 1; i <= ni; ++i) {
                size_t a = G3(i, j, k);
                if (j >= 2 && o->WaterPoints3D[a] && o->WaterPoints3D[G3(i, j - 1, k)])
                    o->ComputeFacesU3D[a] = 1;
                if (i >= 2 && o->WaterPoints3D[a] && o->WaterPoints3D[G3(i - 1, j, k)])
                    o->ComputeFacesV3D[a] = 1;
                double duz = fmin(o->DWZ[a], o->DWZ[G3(i, j - 1, k)]);
                double dvz = fmin(o->DWZ[a], o->DWZ[G3(i - 1, j, k)]);
                o->AreaU[a] = duz * gp->dy;
                o->AreaV[a] = dvz * gp->dx;
            }
    /* east / north face planes j = nj+1, i = ni+1 (areas only; never compute faces) */
    for (int k = 1; k <= nk; ++k) {
        for (int i = 1; i <= ni; ++i)
            o->AreaU[G3(i, nj + 1, k)] = fmin(o->DWZ[G3(i, nj, k)], o->DWZ[G3(i, nj + 1, k)]) * gp->dy;
        for (int j = 1; j <= nj; ++j)
            o->AreaV[G3(ni + 1, j, k)] = fmin(o->DWZ[G3(ni, j, k)], o->DWZ[G3(ni + 1, j, k)]) * gp->dx;
    }
    for (int j = 1; j <= nj; ++j)
        for (int i = 1; i <= ni; ++i) {
            int s = o->ComputeFacesU3D[G3(i, j, nk)] + o->ComputeFacesU3D[G3(i, j + 1, nk)] +
                    o->ComputeFacesV3D[G3(i, j, nk)] + o->ComputeFacesV3D[G3(i + 1, j, nk)];
            if (s > 0)
                for (int k = o->KFloorZ[G2(i, j)] + 1; k <= nk; ++k) o->ComputeFacesW3D[G3(i, j, k)] = 1;
        }
    for (int k = 1; k <= nk; ++k)
        for (int j = 1; j <= nj; ++j)
            for (int i = 1; i <= ni; ++i) {
                int s = o->ComputeFacesU3D[G3(i, j, k)] + o->ComputeFacesU3D[G3(i, j + 1, k)] +
                        o->ComputeFacesV3D[G3(i, j, k)] + o->ComputeFacesV3D[G3(i + 1, j, k)] +
                        o->ComputeFacesW3D[G3(i, j, k)] + o->ComputeFacesW3D[G3(i, j, k + 1)];
                o->OpenPoints3D[G3(i, j, k)] = s > 0;
            }
    /* open-boundary columns */
    for (int j = 1; j <= nj; ++j)
        for (int i = 1; i <= ni; ++i) {
            if (!o->WaterPoints2D[G2(i, j)]) continue;
            int b = ((gp->open_sides & 1) && j == 1) || ((gp->open_sides & 2) && j == nj) ||
                    ((gp->open_sides & 4) && i == 1) || ((gp->open_sides & 8) && i == ni);
            o->BoundaryPoints2D[G2(i, j)] = b;
        }

    /* streamfunction at cell corners (I = 0..ni, J = 0..nj): corner (I,J) touches
     * cells (I,J), (I+1,J), (I,J+1), (I+1,J+1).  It is zero where any touching
     * cell is land or lies outside a closed side; exterior cells on open sides
     * count as water when their interior neighbour is water. */
    const int CI = ni + 1, CJ = nj + 1;
    double* psi = (double*)calloc((size_t)CI * CJ, sizeof(double));
    double* fps = (double*)malloc(sizeof(double) * nw);
    smooth2d(ni, nj, 16, 4, 1.3, seed * 23 + 7, fps);
    for (int J = 0; J <= nj; ++J)
        for (int I = 0; I <= ni; ++I) {
            int ok = 1;
            for (int di = 0; di <= 1 && ok; ++di)
                for (int dj = 0; dj <= 1 && ok; ++dj) {
                    int ci = I + di, cj = J + dj;
                    int inside = ci >= 1 && ci <= ni && cj >= 1 && cj <= nj;
                    if (inside) { ok = o->WaterPoints2D[G2(ci, cj)]; continue; }
                    int side_open = (cj < 1 && (gp->open_sides & 1)) || (cj > nj && (gp->open_sides & 2)) ||
                                    (ci < 1 && (gp->open_sides & 4)) || (ci > ni && (gp->open_sides & 8));
                    if ((ci < 1 || ci > ni) && (cj < 1 || cj > nj)) side_open = 0;  /* corner cell */
                    if (!side_open) { ok = 0; continue; }
                    int mi = ci < 1 ? 1 : (ci > ni ? ni : ci);
                    int mj = cj < 1 ? 1 : (cj > nj ? nj : cj);
                    ok = o->WaterPoints2D[G2(mi, mj)];
                }
            if (!ok) continue;
            int ii = I < 1 ? 1 : (I > ni ? ni : I), jj = J < 1 ? 1 : (J > nj ? nj : J);
            double eddy = 2.0 * fps[(size_t)(jj - 1) * ni + (ii - 1)] - 1.0;
            double thru = 0.0;
            if (gp->open_sides) thru = 1.5 * sin(PI * (double)I / ni) * sin(PI * (double)J / nj + 0.5);
            psi[(size_t)J * CI + I] = eddy + thru;
        }
    /* face transports (column totals): Ux at west face of (i,j), Vy at south face */
    double* fal = (double*)malloc(sizeof(double) * nw);
    smooth2d(ni, nj, 8, 2, 1.0, seed * 29 + 13, fal);
    double* prof = (double*)malloc(sizeof(double) * (size_t)(nk + 2));
    double umax_seen = 0.0;
    for (int pass = 0; pass < 2; ++pass) {
        double scale = (pass == 0) ? 1.0 : ((umax_seen > 0) ? gp->umax / umax_seen : 0.0);
        for (int dir = 0; dir < 2; ++dir)
            for (int j = 1; j <= nj + (dir == 0); ++j)
                for (int i = 1; i <= ni + (dir == 1); ++i) {
                    double U;
                    int ia, ja, ib, jb;              /* the two cells across the face */
                    if (dir == 0) { U = psi[(size_t)(j - 1) * CI + i] - psi[(size_t)(j - 1) * CI + (i - 1)]; ia = i; ja = j - 1; ib = i; jb = j; }
                    else { U = -(psi[(size_t)j * CI + (i - 1)] - psi[(size_t)(j - 1) * CI + (i - 1)]); ia = i - 1; ja = j; ib = i; jb = j; }
                    if (U == 0.0) continue;
                    int wa = (ia >= 1 && ia <= ni && ja >= 1 && ja <= nj) ? o->WaterPoints2D[G2(ia, ja)] : -1;
                    int wb = (ib >= 1 && ib <= ni && jb >= 1 && jb <= nj) ? o->WaterPoints2D[G2(ib, jb)] : -1;
                    int kfa = (wa == 1) ? o->KFloorZ[G2(ia, ja)] : 0;
                    int kfb = (wb == 1) ? o->KFloorZ[G2(ib, jb)] : 0;
                    if (wa == 0 || wb == 0) continue;
                    int kf = kfa > kfb ? kfa : kfb;
                    if (kf < 1) kf = 1;
                    int ic = (wa == 1) ? ia : ib, jc = (wa == 1) ? ja : jb;
                    int icl = ic < 1 ? 1 : (ic > ni ? ni : ic), jcl = jc < 1 ? 1 : (jc > nj ? nj : jc);
                    double alpha = 1.2 * (fal[(size_t)(jcl - 1) * ni + (icl - 1)] - 0.5);
                    double sum = 0.0;
                    for (int k = kf; k <= nk; ++k) {
                        double th;
                        if (wa == 1 && wb == 1) th = fmin(o->DWZ[G3(ia, ja, k)], o->DWZ[G3(ib, jb, k)]);
                        else th = o->DWZ[G3(ic, jc, k)];
                        double s = (nk > 1) ? 2.0 * (k - kf + 0.5) / (nk - kf + 1) - 1.0 : 0.0;
                        prof[k] = th * (1.0 + alpha * s);
                        sum += prof[k];
                    }
                    double len = (dir == 0) ? gp->dy : gp->dx;
                    for (int k = kf; k <= nk; ++k) {
                        double q = scale * U * prof[k] / sum;
                        double th;
                        if (wa == 1 && wb == 1) th = fmin(o->DWZ[G3(ia, ja, k)], o->DWZ[G3(ib, jb, k)]);
                        else th = o->DWZ[G3(ic, jc, k)];
                        if (pass == 0) {
                            double u = fabs(q) / (th * len);
                            if (u > umax_seen) umax_seen = u;
                        } else if (dir == 0) {
                            o->Wflux_X[G3(i, j, k)] = q;
                        } else {
                            o->Wflux_Y[G3(i, j, k)] = q;
                        }
                    }
                }
    }

    /* moving volumes: redistribute volume inside each column (zero net change) */
    double* fvv = (double*)malloc(sizeof(double) * nw);
    smooth2d(ni, nj, 8, 3, 1.0, seed * 31 + 17, fvv);
    for (int j = 1; j <= nj; ++j)
        for (int i = 1; i <= ni; ++i) {
            if (!o->WaterPoints2D[G2(i, j)]) continue;
            int kf = o->KFloorZ[G2(i, j)];
            double g = 2.0 * fvv[(size_t)(j - 1) * ni + (i - 1)] - 1.0;
            double sv = 0.0, svc = 0.0;
            for (int k = kf; k <= nk; ++k) {
                double s = (nk > kf) ? 2.0 * (k - kf) / (double)(nk - kf) - 1.0 : 0.0;
                sv += o->VolumeZOld[G3(i, j, k)];
                svc += o->VolumeZOld[G3(i, j, k)] * g * s;
            }
            double cbar = svc / sv;
            for (int k = kf; k <= nk; ++k) {
                size_t a = G3(i, j, k);
                double s = (nk > kf) ? 2.0 * (k - kf) / (double)(nk - kf) - 1.0 : 0.0;
                o->VolumeZ[a] = o->VolumeZOld[a] * (1.0 + gp->vol_var * (g * s - cbar));
            }
        }
    /* vertical transport from continuity (positive upwards, face k below cell k) */
    for (int j = 1; j <= nj; ++j)
        for (int i = 1; i <= ni; ++i) {
            if (!o->WaterPoints2D[G2(i, j)]) continue;
            int kf = o->KFloorZ[G2(i, j)];
            double qz = 0.0;
            for (int k = kf; k <= nk; ++k) {
                size_t a = G3(i, j, k);
                o->Wflux_Z[a] = qz;
                qz = qz + o->Wflux_X[a] - o->Wflux_X[G3(i, j + 1, k)] + o->Wflux_Y[a] -
                     o->Wflux_Y[G3(i + 1, j, k)] - (o->VolumeZ[a] - o->VolumeZOld[a]) / gp->dt;
            }
            o->Wflux_Z[G3(i, j, nk + 1)] = 0.0;   /* closed surface: residual is round-off */
        }

    /* diffusivities */
    uint64_t s = seed * 37 + 19;
    for (size_t q = 0; q < n3; ++q) o->Visc_H[q] = gp->visc_h;
    for (int k = 1; k <= nk; ++k)
        for (int j = 1; j <= nj; ++j)
            for (int i = 1; i <= ni; ++i)
                o->Diff_V[G3(i, j, k)] = exp(log(gp->kz_median) + gp->kz_logsigma * nrand(&s));

    free(fland); free(fbat); free(wet); free(psi); free(fps); free(fal); free(prof); free(fvv);
    return 0;
}

int mohid_synth_tracer(const mohid_synth_params* gp, const mohid_synth_out* o, int kind, double a,
                    double b, uint64_t seed, double* P)
{
    const int ni = gp->ni, nj = gp->nj, nk = gp->nk;
    ext_t E = {ni + 2, nj + 2, nk + 2};
    const size_t n3 = (size_t)E.NI * E.NJ * E.NK, nw = (size_t)ni * nj;
    memset(P, 0, sizeof(double) * n3);
    double* f = (double*)malloc(sizeof(double) * nw);
    smooth2d(ni, nj, 12, 4, 1.0, seed * 41 + 23, f);
    uint64_t s = seed * 43 + 29;
    double ic = 1 + (ni - 1) * (0.3 + 0.4 * urand(&s));
    double jc = 1 + (nj - 1) * (0.3 + 0.4 * urand(&s));
    double kc = 1 + (nk - 1) * (0.3 + 0.4 * urand(&s));
    double ph = 2 * PI * urand(&s);
    for (int k = 1; k <= nk; ++k)
        for (int j = 1; j <= nj; ++j)
            for (int i = 1; i <= ni; ++i) {
                size_t q = G3(i, j, k);
                if (!o->WaterPoints3D[q]) continue;
                double h = f[(size_t)(j - 1) * ni + (i - 1)];
                double zc = 0.0;   /* depth of the cell centre below the surface */
                for (int kk = nk; kk > k; --kk) zc += o->DWZ[G3(i, j, kk)];
                zc += 0.5 * o->DWZ[q];
                double v;
                switch (kind) {
                case 0:
                    v = a * exp(-((i - ic) * (i - ic) + (j - jc) * (j - jc) + (k - kc) * (k - kc)) / (2 * b * b));
                    break;
                case 1: {
                    double t = zc / (gp->hmax > 0 ? gp->hmax : 1.0);
                    v = b - (b - a) * (0.85 * t + 0.15 * h);
                    break;
                }
                case 2:
                    v = a + (b - a) * (0.8 * h + 0.2 * (1.0 - zc / (gp->hmax > 0 ? gp->hmax : 1.0)));
                    break;
                case 3:
                    v = exp(log(a) + b * (3.0 * (h - 0.5) + 0.5 * sin(2 * PI * k / (nk + 1.0) + ph)));
                    break;
                default:
                    v = a;
                }
                P[q] = v;
            }
    free(f);
    return 0;
}

int mohid_synth_reference(const mohid_synth_params* gp, const mohid_synth_out* o, double c0, double rel,
                       uint64_t seed, double* R)
{
    const int ni = gp->ni, nj = gp->nj, nk = gp->nk;
    ext_t E = {ni + 2, nj + 2, nk + 2};
    const size_t n3 = (size_t)E.NI * E.NJ * E.NK, nw = (size_t)ni * nj;
    (void)o;
    memset(R, 0, sizeof(double) * n3);
    double* f = (double*)malloc(sizeof(double) * nw);
    smooth2d(ni, nj, 6, 2, 1.0, seed * 47 + 31, f);
    for (int k = 1; k <= nk; ++k)
        for (int j = 1; j <= nj; ++j)
            for (int i = 1; i <= ni; ++i)
                R[G3(i, j, k)] = c0 * (1.0 + rel * (2.0 * f[(size_t)(j - 1) * ni + (i - 1)] - 1.0) +
                                       0.1 * rel * (double)k / nk);
    free(f);
    return 0;
}
