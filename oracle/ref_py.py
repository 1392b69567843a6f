"""TEST INFRASTRUCTURE ONLY: pure-Python restatement of one AdvectionDiffusion call.

A second, independent reading of the Fortran, written as plain loops over
Python floats (IEEE double, no fused multiply-add), for grids of a few hundred
cells.  tests/ require it to agree bit for bit with the C oracle
(oracle/ad_oracle.c).  It follows, in call order:

  Convert_Dif_Vertical        Software/MOHIDBase2/ModuleAdvectionDiffusion.F90:2364-2443
  Convert_Visc_Dif_Horizontal ModuleAdvectionDiffusion.F90:2453-2595
  AdvectionDiffusionIteration ModuleAdvectionDiffusion.F90:1624-1922
    VolumeVariation           :3966-4021
    HorizontalDiffusionXX/YY  :5156-5214, :5313-5365
    HorizontalAdvectionXX/YY  :4368-4540, :4739-4910
      ComputeAdvection1D_V2   Software/MOHIDBase1/ModuleFunctions.F90:10534-10591
      ComputeAdvectionFace    ModuleFunctions.F90:10702-10894
    VerticalDiffusion         ModuleAdvectionDiffusion.F90:2708-2784
    VerticalAdvection         :2941-3140
    OpenBoundaryCondition     :5369-5742
      OrlanskiCelerity2D      ModuleFunctions.F90:4129-4490
    SetMatrixValue(TI, null)  :1753
    THOMASZ_NewType2          ModuleFunctions.F90:4026-4123
"""
from __future__ import annotations

import numpy as np

NULL_REAL = -9.9e15
MIN_VALUE = 1.0e-16


def _mn(a, b):
    return b if b < a else a


def _mx(a, b):
    return b if b > a else a


def face(P, V, du, dt, Q, vrm, method, limiter, nb, up2):
    """ComputeAdvectionFace; P, V, du are 4-lists for cells f-2..f+1."""
    cup1 = [0.0, 0.0, 0.0, 0.0]
    if Q > 0.0:
        cup1[1] = 1.0
    else:
        cup1[2] = 1.0
    Cr = 0.0
    vrel = 0.0
    if not nb:
        if Q > 0:
            Cr = Q * dt / V[1]
            vrel = _mx(_mx(V[0], V[1]), V[2]) / _mn(_mn(V[0], V[1]), V[2])
        else:
            Cr = Q * dt / V[2]
            vrel = _mx(_mx(V[1], V[2]), V[3]) / _mn(_mn(V[1], V[2]), V[3])
    if method == 1 or (nb and up2):
        high = list(cup1)
        theta = 0.0
    elif method == 2 and not nb:
        if Q > 0:
            high = [-1.0 / 8.0, 6.0 / 8.0, 3.0 / 8.0, 0.0]
        elif Q < 0:
            high = [0.0, 3.0 / 8.0, 6.0 / 8.0, -1.0 / 8.0]
        else:
            high = [0.0, 0.0, 1.0, 0.0]
        theta = 0.0 if vrel > vrm else 1.0
    elif method == 3 and not nb:
        c = (1 - 2.0 * abs(Cr)) / 6.0
        a = 0.5 + c
        b = 0.5 - c
        d = (1 - abs(Cr)) / 2.0
        if Q > 0:
            high = [-d * b, 1 + d * (b - a), d * a, 0.0]
        elif Q < 0:
            high = [0.0, d * a, 1 + d * (b - a), -d * b]
        else:
            high = [0.0, 0.0, 1.0, 0.0]
        theta = 0.0 if vrel > vrm else 1.0
    elif method in (5, 6):
        high = [0.0, du[2] / (du[1] + du[2]), du[1] / (du[1] + du[2]), 0.0]
        theta = 1.0
    elif method == 4 and not nb:
        high = [0.0, 0.0, 0.0, 0.0]
        if Q > 0.0:
            high[2] = 1.0
            dC = (P[2] - P[1]) / (du[2] + du[1])
            if abs(dC) < MIN_VALUE:
                dC = MIN_VALUE if dC >= 0 else -MIN_VALUE
            r = (P[1] - P[0]) / (du[1] + du[0]) / dC
        else:
            high[1] = 1.0
            dC = (P[1] - P[2]) / (du[2] + du[1])
            if abs(dC) < MIN_VALUE:
                dC = MIN_VALUE if dC >= 0 else -MIN_VALUE
            r = (P[2] - P[3]) / (du[2] + du[3]) / dC
        if limiter == 1:
            theta = _mx(0.0, _mn(1.0, r))
        elif limiter == 2:
            theta = 0.0 if r < 0 else 2.0 * r / (1 + r)
        elif limiter == 3:
            theta = _mx(0.0, _mn(_mn(2.0, 2.0 * r), (1 + r) / 2.0))
        elif limiter == 4:
            theta = _mx(_mx(0.0, _mn(1.0, 2.0 * r)), _mn(r, 2.0))
        elif limiter == 5:
            a = 0.5 + (1 - 2.0 * abs(Cr)) / 6.0
            b = 0.5 - (1 - 2.0 * abs(Cr)) / 6.0
            aux = a + b * r
            if abs(Cr) < MIN_VALUE:
                Cr = MIN_VALUE
            theta = _mx(0.0, _mn(_mn(aux, 2.0 / (1.0 - Cr)), 2.0 * r / Cr))
        else:
            raise ValueError("limiter")
        theta = 0.5 * theta * (1.0 - Cr)
    else:
        raise ValueError("method stops")
    return [(1.0 - theta) * cup1[n] + theta * high[n] for n in range(4)]


def _null_grad(Pl, CU, CV, k, j, i):
    """NullGradProp (AD:2071-2110): mean of the neighbours across compute faces, or None."""
    aux = CV[k][j][i + 1] + CV[k][j][i] + CU[k][j + 1][i] + CU[k][j][i]
    if aux <= 0:
        return None
    return (Pl[k][j][i + 1] * CV[k][j][i + 1] + Pl[k][j][i - 1] * CV[k][j][i] +
            Pl[k][j + 1][i] * CU[k][j + 1][i] + Pl[k][j - 1][i] * CU[k][j][i]) / float(aux)


def _orlanski_normal(ni, nj, i, j):
    """The normal of boundary point (i, j) and its exterior point (AD:5504-5540):
    (di, dj, east_north, iext, jext), or None where the reference stops."""
    if i == 1 or i == ni:
        di, dj = 1, 0
    elif j == 1 or j == nj:
        di, dj = 0, 1
    else:
        return None
    if i == 1 or j == 1:
        return di, dj, False, i - di, j - dj
    return di, dj, True, i + di, j + dj


def _orlanski(NF, OF, Ref, CP, k, ni, nj, di, dj, i, j, en, limit, dt, flow):
    """OrlanskiCelerity2D (ModuleFunctions.F90:4129-4490) as OpenBoundaryCondition
    calls it (AD:5551-5567): implicit, oblique, non-constant celerity, no
    relaxation times given (86400 * 300 s), compute box 1..ni x 1..nj.  NF / OF
    are [k][j][i] lists of the Size box; a point (a, b) is addressed through
    the column-major plane offset a + (ni + 2) * b, as the Fortran does without
    bounds checks.  Updates OF and NF at (i, j, k) and returns the new value."""
    I = ni + 2

    def at(arr, a, b):
        q = a + I * b
        return arr[k][q // I][q % I]

    no_sw = no_ne = False
    s = -1 if en else 1                        # from the exterior point into the domain
    i1n, i1o = at(NF, i + s * di, j + s * dj), at(OF, i + s * di, j + s * dj)
    i2n = at(NF, i + 2 * s * di, j + 2 * s * dj)
    i3n = at(NF, i + 3 * s * di, j + 3 * s * dj)
    i6o = at(OF, i + s * di + dj, j + s * dj + di)
    i7o = at(OF, i + s * di - dj, j + s * dj - di)
    bi, bj = i + s * di, j + s * dj            # the first interior point
    if bi + 3 * dj > ni or bj + 3 * di > nj:
        no_ne = True
    elif at(CP, bi + dj, bj + di) * at(CP, bi + 2 * dj, bj + 2 * di) * at(CP, bi + 3 * dj, bj + 3 * di) == 0:
        no_ne = True
    if bi - 3 * dj < 1 or bj - 3 * di < 1:
        no_sw = True
    elif at(CP, bi - dj, bj - di) * at(CP, bi - 2 * dj, bj - 2 * di) * at(CP, bi - 3 * dj, bj - 3 * di) == 0:
        no_sw = True
    b5 = at(OF, i, j)
    tv = i1n - i1o
    svx = i1n - i2n
    if (i6o - i7o) * tv > 0:
        svy = 0.0 if no_sw else i1o - i7o
    else:
        svy = 0.0 if no_ne else i6o - i1o
    ss = svx * svx + svy * svy
    if ss > 0.0:
        cx = -((tv * svx) / ss)
        cy = -((tv * svy) / ss)
        if abs(cx) > limit:
            cx = limit * cx / abs(cx)
        if abs(cy) > limit:
            cy = limit * cy / abs(cy)
    else:
        cx = cy = 0.0
    ref = at(Ref, i, j)
    trelax = float(86400 * 300)
    cx = cx + flow
    if cx > 0:
        cx = 4 * cx
        adj = 0.0546875 * i3n - 0.2578125 * i2n + 0.6015625 * i1n
    else:
        adj, cx, cy = ref, 0.0, 0.0
    aux = cx * adj
    if cy >= 0 and not no_sw:
        b4, b42, b43 = at(OF, i - dj, j - di), at(OF, i - 2 * dj, j - 2 * di), at(OF, i - 3 * dj, j - 3 * di)
        adjy = 0.0546875 * b43 - 0.2578125 * b42 + 0.6015625 * b4 + 0.6015625 * b5
        aux = aux - 4 * cy * (b5 - adjy)
    elif cy < 0 and not no_ne:
        b3, b32, b33 = at(OF, i + dj, j + di), at(OF, i + 2 * dj, j + 2 * di), at(OF, i + 3 * dj, j + 3 * di)
        adjy = 0.0546875 * b33 - 0.2578125 * b32 + 0.6015625 * b3 + 0.6015625 * b5
        aux = aux - 4 * cy * (adjy - b5)
    q = i + I * j
    OF[k][q // I][q % I] = NF[k][q // I][q % I]
    bound = 1 + cx * (1 - 0.6015625) + dt / trelax
    NF[k][q // I][q % I] = (OF[k][q // I][q % I] + aux + ref * dt / trelax) / bound
    return NF[k][q // I][q % I]


def _thomas_lines(D, E, F, TI, Pl, along_j, ni, nj, nk):
    """THOMAS_3D (FN:3760-3876): a tridiagonal system per work-box line along j
    (or i), first work cell to the halo cell past the last, every layer; the
    answer goes to Pl.  Returns True on a zero pivot."""
    n, m = (nj, ni) if along_j else (ni, nj)
    zero = False

    def at(arr, x, l, k):
        return arr[k][x][l] if along_j else arr[k][l][x]

    for k in range(1, nk + 1):
        for l in range(1, m + 1):
            W = [0.0] * (n + 2)
            G = [0.0] * (n + 2)
            W[1] = -at(F, 1, l, k) / at(E, 1, l, k)
            G[1] = at(TI, 1, l, k) / at(E, 1, l, k)
            for x in range(2, n + 2):
                aux = at(E, x, l, k) + at(D, x, l, k) * W[x - 1]
                if abs(aux) > 0:
                    W[x] = -at(F, x, l, k) / aux
                    G[x] = (at(TI, x, l, k) - at(D, x, l, k) * G[x - 1]) / aux
                else:
                    W[x], G[x], zero = 0.0, 0.0, True
            ans = [0.0] * (n + 2)
            ans[n + 1] = G[n + 1]
            for x in range(n, 0, -1):
                ans[x] = W[x] * ans[x + 1] + G[x]
            for x in range(1, n + 2):
                if along_j:
                    Pl[k][x][l] = ans[x]
                else:
                    Pl[k][l][x] = ans[x]
    return zero


def _adv_flux(Fl, Cc, Cd, Ce, Cf, Pl, CF, wgt, ni, nj, nk, axis):
    """CalcHorizontalAdvFluxXX / YY, CalcVerticalAdvFlux (AD:3356-3619): Flux +=
    Weigth * (C P(-2) + D P(-1) + E P(0) + F P(+1)) at the compute faces."""
    for k in range(1, nk + 1):
        for j in range(1, nj + 1):
            for i in range(1, ni + 1):
                if CF[k][j][i] != 1:
                    continue
                if axis == 0:
                    pm2, pm1, p0, pp1 = Pl[k][j - 2][i], Pl[k][j - 1][i], Pl[k][j][i], Pl[k][j + 1][i]
                elif axis == 1:
                    pm2, pm1, p0, pp1 = Pl[k][j][i - 2], Pl[k][j][i - 1], Pl[k][j][i], Pl[k][j][i + 1]
                else:
                    pm2, pm1, p0, pp1 = Pl[k - 2][j][i], Pl[k - 1][j][i], Pl[k][j][i], Pl[k + 1][j][i]
                Fl[k][j][i] = Fl[k][j][i] + wgt * (Cc[k][j][i] * pm2 + Cd[k][j][i] * pm1 + Ce[k][j][i] * p0 +
                                                   Cf[k][j][i] * pp1)


def _dif_flux_z(Fl, Kz, DUX, DVY, DZZ, Pl, CW, wgt, ni, nj, nk):
    """CalcVerticalDifFlux (AD:3668-3711)."""
    for k in range(1, nk + 1):
        for j in range(1, nj + 1):
            for i in range(1, ni + 1):
                if CW[k][j][i] == 1:
                    Fl[k][j][i] = Fl[k][j][i] - wgt * Kz[k][j][i] * DUX[j][i] * DVY[j][i] / DZZ[k - 1][j][i] * \
                        (Pl[k][j][i] - Pl[k - 1][j][i])


def step(dom, P, p, ReferenceProp=None, SmallDepths=None, fluxes=None, NoFlux=None, Disch=None, PropOld=None):
    """One step on numpy arrays of a tiny Domain; P (float64 Size box) updated in place.
    `p` is a dict of AdvectionDiffusion scalar arguments.  With CellFluxes set
    and a dict `fluxes`, the six face-flux arrays are stored in it.  With
    Orlanski boundaries the field as OpenBoundaryCondition saw it is written
    to `PropOld` when given (AD:5428-5429)."""
    ni, nj, nk = dom.ni, dom.nj, dom.nk
    A = dom.arrays
    f3 = lambda n: A[n].tolist()           # [k][j][i]
    Qx, Qy, Qz = f3("Wflux_X"), f3("Wflux_Y"), f3("Wflux_Z")
    V, Vo = f3("VolumeZ"), f3("VolumeZOld")
    VH, DV = f3("Visc_H"), f3("Diff_V")
    AU, AV, DZZ, DWZ = f3("AreaU"), f3("AreaV"), f3("DZZ"), f3("DWZ")
    OP, LP, WP = f3("OpenPoints3D"), f3("LandPoints3D"), f3("WaterPoints3D")
    CU, CV, CW = f3("ComputeFacesU3D"), f3("ComputeFacesV3D"), f3("ComputeFacesW3D")
    DUX, DVY, DZX, DZY = (A[n].tolist() for n in ("DUX", "DVY", "DZX", "DZY"))
    KF, BP = A["KFloorZ"].tolist(), A["BoundaryPoints2D"].tolist()
    Pl = P.tolist()
    R = ReferenceProp.tolist() if ReferenceProp is not None else None
    SD = SmallDepths.tolist() if SmallDepths is not None else None
    DT = p["DTProp"]
    K, J, I = nk + 2, nj + 2, ni + 2
    z3 = lambda v: [[[v] * I for _ in range(J)] for _ in range(K)]
    Kx, Ky, Kz = z3(NULL_REAL), z3(NULL_REAL), z3(NULL_REAL)
    NFU, NFV, NFW = (m.tolist() for m in NoFlux) if NoFlux is not None else (None, None, None)
    # AdvectionNudging: the advective terms gather in AdvectionTi/D/E/F, the
    # _Nudge routines ignore the NoAdvFlux masks (AD:4151-4165, 3211-3350)
    nudge = bool(p.get("AdvectionNudging"))
    if nudge and (p["ImpExp_AdvXX"] != 0.0 or p["ImpExp_AdvYY"] != 0.0 or p["Vertical1D"]):
        raise ValueError("AdvectionNudging with implicit horizontal advection or Vertical1D")
    no_adv = bool(p.get("NoAdvFlux")) and not nudge
    ATi, AD, AE, AF = z3(0.0), z3(0.0), z3(0.0), z3(0.0)
    for k in range(2, nk + 1):
        for j in range(1, nj + 1):
            for i in range(1, ni + 1):
                if CW[k][j][i] == 1:
                    Kz[k][j][i] = p["SchmidtCoef_V"] * DV[k][j][i] + p["SchmidtBackground_V"]
                    if p["NullDif"] and Qz[k][j][i] == 0.0:
                        Kz[k][j][i] = 0.0
    for k in range(1, nk + 1):
        for j in range(1, nj + 1):
            for i in range(1, ni + 1):
                if CU[k][j][i] == 1:
                    Kx[k][j][i] = p["schmidt_H"] * (VH[k][j][i] * DUX[j - 1][i] + VH[k][j - 1][i] * DUX[j][i]) \
                        / (DUX[j][i] + DUX[j - 1][i])
                    if p.get("NoDifFlux") and NFU[k][j][i] == 1:
                        Kx[k][j][i] = 0.0
                    if p["NullDif"] and Qx[k][j][i] == 0.0:
                        Kx[k][j][i] = 0.0
                if CV[k][j][i] == 1:
                    Ky[k][j][i] = p["schmidt_H"] * (VH[k][j][i] * DVY[j][i - 1] + VH[k][j][i - 1] * DVY[j][i]) \
                        / (DVY[j][i] + DVY[j][i - 1])
                    if p.get("NoDifFlux") and NFV[k][j][i] == 1:
                        Ky[k][j][i] = 0.0
                    if p["NullDif"] and Qy[k][j][i] == 0.0:
                        Ky[k][j][i] = 0.0
    D, E, F, TI = z3(0.0), z3(1.0), z3(0.0), z3(0.0)
    XC, XD, XE, XF = z3(0.0), z3(0.0), z3(0.0), z3(0.0)
    YC, YD, YE, YF = z3(0.0), z3(0.0), z3(0.0), z3(0.0)
    ZC, ZD, ZE, ZF = z3(0.0), z3(0.0), z3(0.0), z3(0.0)
    cflux = bool(p.get("CellFluxes", 0))
    FAX, FAY, FAZ, FDX, FDY, FDZ = (z3(0.0) for _ in range(6))

    # VolumeVariation
    for k in range(1, nk + 1):
        for j in range(1, nj + 1):
            for i in range(1, ni + 1):
                if OP[k][j][i] == 1:
                    TI[k][j][i] = Pl[k][j][i] * (Vo[k][j][i] / V[k][j][i])
                    if k == nk:
                        E[k][j][i] = 1.0 + (DT / V[k][j][i]) * Qz[k + 1][j][i]
                else:
                    TI[k][j][i] = Pl[k][j][i]

    # Discharges (AD:4025-4128)
    if Disch is not None:
        n = 0
        for dis in range(len(Disch["nCells"])):
            if Disch["ignore"][dis]:
                continue
            uniform = int(Disch["vert"][dis]) == 5
            for _ in range(int(Disch["nCells"][dis])):
                i, j = int(Disch["I"][n]), int(Disch["J"][n])
                if uniform:
                    kmin = KF[j][i] if int(Disch["Kmin"][n]) == -9999999 else int(Disch["Kmin"][n])
                    kmax = nk if int(Disch["Kmax"][n]) == -9999999 else int(Disch["Kmax"][n])
                else:
                    kmin = kmax = int(Disch["K"][n])
                wc = 0.0
                for k in range(kmin, kmax + 1):
                    wc = wc + DWZ[k][j][i]
                flow0, conc, cmf = float(Disch["Flow"][n]), float(Disch["Conc"][n]), float(Disch["ConcMF"][n])
                for k in range(kmin, kmax + 1):
                    dtv = DT / V[k][j][i]
                    flow = flow0 * DWZ[k][j][i] / wc if uniform else flow0
                    if OP[k][j][i] == 1:
                        if Disch["bypass"][dis] or flow > 0.0:
                            TI[k][j][i] = TI[k][j][i] + flow * dtv * conc
                        else:
                            E[k][j][i] = E[k][j][i] - flow * dtv * cmf
                    elif flow > 0.0:
                        TI[k][j][i] = Pl[k][j][i] * Vo[k][j][i] / V[k][j][i] + flow * dtv * conc
                n += 1

    mH, lH, u2H = p["AdvMethodH"], p["TVDLimitationH"], bool(p["Upwind2H"])
    if not p["Vertical1D"]:
        for k in range(1, nk + 1):
            for j in range(1, nj + 1):
                for i in range(1, ni + 1):
                    if CU[k][j][i] == 1:
                        aux = Kx[k][j][i] * AU[k][j][i] / DZX[j - 1][i]
                        dP = Pl[k][j][i] - Pl[k][j - 1][i]
                        TI[k][j - 1][i] = TI[k][j - 1][i] + aux * DT / V[k][j - 1][i] * dP
                        TI[k][j][i] = TI[k][j][i] - aux * DT / V[k][j][i] * dP
        if cflux:                                          # CalcHorizontalDifFluxXX
            for k in range(1, nk + 1):
                for j in range(1, nj + 1):
                    for i in range(1, ni + 1):
                        if CU[k][j][i] == 1:
                            FDX[k][j][i] = FDX[k][j][i] - Kx[k][j][i] * AU[k][j][i] / DZX[j - 1][i] * \
                                (Pl[k][j][i] - Pl[k][j - 1][i])
        if not p["XZFlow"]:
            for k in range(1, nk + 1):
                for j in range(1, nj + 1):
                    for i in range(1, ni + 1):
                        if CV[k][j][i] == 1:
                            aux = Ky[k][j][i] * AV[k][j][i] / DZY[j][i - 1]
                            dP = Pl[k][j][i] - Pl[k][j][i - 1]
                            TI[k][j][i - 1] = TI[k][j][i - 1] + aux * DT / V[k][j][i - 1] * dP
                            TI[k][j][i] = TI[k][j][i] - aux * DT / V[k][j][i] * dP
            if cflux:                                      # CalcHorizontalDifFluxYY
                for k in range(1, nk + 1):
                    for j in range(1, nj + 1):
                        for i in range(1, ni + 1):
                            if CV[k][j][i] == 1:
                                FDY[k][j][i] = FDY[k][j][i] - Ky[k][j][i] * AV[k][j][i] / DZY[j][i - 1] * \
                                    (Pl[k][j][i] - Pl[k][j][i - 1])
        TIa = ATi if nudge else TI
        # XX: faces j = 1..nj of every line (i, :, k)
        for k in range(1, nk + 1):
            for i in range(1, ni + 1):
                for j in range(1, nj + 1):
                    if OP[k][j - 1][i] == 1 and OP[k][j][i] == 1:
                        q = Qx[k][j][i]
                        nb = (OP[k][j - 2][i] != 1) if q > 0 else (OP[k][j + 1][i] != 1)
                        cf = face([Pl[k][j + n][i] for n in (-2, -1, 0, 1)],
                                  [V[k][j + n][i] for n in (-2, -1, 0, 1)],
                                  [DUX[j + n][i] for n in (-2, -1, 0, 1)], DT, q,
                                  p["VolumeRelMax"], mH, lH, nb, u2H)
                        XC[k][j][i], XD[k][j][i], XE[k][j][i], XF[k][j][i] = (q * c for c in cf)
                    if no_adv and NFU[k][j][i] == 1:             # AD:4434-4443
                        XC[k][j][i] = XD[k][j][i] = XE[k][j][i] = XF[k][j][i] = 0.0
        for k in range(1, nk + 1):
            for j in range(1, nj + 1):
                for i in range(1, ni + 1):
                    if CU[k][j][i] != 1:
                        continue
                    if p["ImpExp_AdvXX"] == 0.0:
                        fl = XC[k][j][i] * Pl[k][j - 2][i] + XD[k][j][i] * Pl[k][j - 1][i] + \
                            XE[k][j][i] * Pl[k][j][i] + XF[k][j][i] * Pl[k][j + 1][i]
                        TIa[k][j][i] = TIa[k][j][i] + fl * DT / V[k][j][i]
                        TIa[k][j - 1][i] = TIa[k][j - 1][i] - fl * DT / V[k][j - 1][i]
                    else:                                  # implicit, AD:4490-4515
                        dt2, dt1 = DT / V[k][j][i], DT / V[k][j - 1][i]
                        D[k][j][i] = D[k][j][i] - XD[k][j][i] * dt2
                        E[k][j][i] = E[k][j][i] - XE[k][j][i] * dt2
                        E[k][j - 1][i] = E[k][j - 1][i] + XD[k][j][i] * dt1
                        F[k][j - 1][i] = F[k][j - 1][i] + XE[k][j][i] * dt1
        if cflux and p["ImpExp_AdvXX"] == 0.0:
            _adv_flux(FAX, XC, XD, XE, XF, Pl, CU, 1.0 - p["ImpExp_AdvXX"], ni, nj, nk, 0)
        if not p["XZFlow"]:
            for k in range(1, nk + 1):
                for j in range(1, nj + 1):
                    for i in range(1, ni + 1):
                        if OP[k][j][i - 1] == 1 and OP[k][j][i] == 1:
                            q = Qy[k][j][i]
                            nb = (OP[k][j][i - 2] != 1) if q > 0 else (OP[k][j][i + 1] != 1)
                            cf = face([Pl[k][j][i + n] for n in (-2, -1, 0, 1)],
                                      [V[k][j][i + n] for n in (-2, -1, 0, 1)],
                                      [DVY[j][i + n] for n in (-2, -1, 0, 1)], DT, q,
                                      p["VolumeRelMax"], mH, lH, nb, u2H)
                            YC[k][j][i], YD[k][j][i], YE[k][j][i], YF[k][j][i] = (q * c for c in cf)
                        if no_adv and NFV[k][j][i] == 1:         # AD:4804-4813
                            YC[k][j][i] = YD[k][j][i] = YE[k][j][i] = YF[k][j][i] = 0.0
            for k in range(1, nk + 1):
                for j in range(1, nj + 1):
                    for i in range(1, ni + 1):
                        if CV[k][j][i] != 1:
                            continue
                        if p["ImpExp_AdvYY"] == 0.0:
                            fl = YC[k][j][i] * Pl[k][j][i - 2] + YD[k][j][i] * Pl[k][j][i - 1] + \
                                YE[k][j][i] * Pl[k][j][i] + YF[k][j][i] * Pl[k][j][i + 1]
                            TIa[k][j][i] = TIa[k][j][i] + fl * DT / V[k][j][i]
                            TIa[k][j][i - 1] = TIa[k][j][i - 1] - fl * DT / V[k][j][i - 1]
                        else:                              # implicit, AD:4855-4880
                            dt2, dt1 = DT / V[k][j][i], DT / V[k][j][i - 1]
                            D[k][j][i] = D[k][j][i] - YD[k][j][i] * dt2
                            E[k][j][i] = E[k][j][i] - YE[k][j][i] * dt2
                            E[k][j][i - 1] = E[k][j][i - 1] + YD[k][j][i] * dt1
                            F[k][j][i - 1] = F[k][j][i - 1] + YE[k][j][i] * dt1
            if cflux and p["ImpExp_AdvYY"] == 0.0:
                _adv_flux(FAY, YC, YD, YE, YF, Pl, CV, 1.0 - p["ImpExp_AdvYY"], ni, nj, nk, 1)
        # 3-D: the implicit direction is solved now, the vertical step starts
        # again from D = 0, E = 1, F = 0, TI = PROP (AD:4167-4254)
        if (p["ImpExp_AdvXX"] == 1.0 or p["ImpExp_AdvYY"] == 1.0) and nk > 1:
            zero_h = _thomas_lines(D, E, F, TI, Pl, p["ImpExp_AdvXX"] == 1.0, ni, nj, nk)
            D, E, F = z3(0.0), z3(1.0), z3(0.0)
            TI = [[row[:] for row in layer] for layer in Pl]

    if nk > 1:
        ie = p["ImpExp_DifV"]
        for k in range(1, nk + 1):
            for j in range(1, nj + 1):
                for i in range(1, ni + 1):
                    sd = SD is not None and SD[j][i] != 0
                    if CW[k][j][i] == 1 and not sd:
                        auxk = Kz[k][j][i] * DUX[j][i] * DVY[j][i] / DZZ[k - 1][j][i]
                        if p.get("NoDifFlux") and NFW[k][j][i] == 1:   # AD:2741-2745
                            auxk = 0.0
                        a1 = auxk * DT / V[k - 1][j][i]
                        a2 = auxk * DT / V[k][j][i]
                        dP = Pl[k][j][i] - Pl[k - 1][j][i]
                        E[k - 1][j][i] = E[k - 1][j][i] + a1 * ie
                        F[k - 1][j][i] = F[k - 1][j][i] - a1 * ie
                        TI[k - 1][j][i] = TI[k - 1][j][i] + a1 * dP * (1.0 - ie)
                        D[k][j][i] = D[k][j][i] - a2 * ie
                        E[k][j][i] = E[k][j][i] + a2 * ie
                        TI[k][j][i] = TI[k][j][i] - a2 * dP * (1.0 - ie)
        if cflux and ie < 1.0:
            _dif_flux_z(FDZ, Kz, DUX, DVY, DZZ, Pl, CW, 1.0 - ie, ni, nj, nk)
        if not p["Vertical1D"]:
            mV, lV, u2V = p["AdvMethodV"], p["TVDLimitationV"], bool(p["Upwind2V"])
            for j in range(1, nj + 1):
                for i in range(1, ni + 1):
                    if OP[nk][j][i] != 1:
                        continue
                    for k in range(1, nk + 1):
                        if OP[k - 1][j][i] == 1 and OP[k][j][i] == 1:
                            q = Qz[k][j][i]
                            nb = (OP[k - 2][j][i] != 1) if q > 0 else (OP[k + 1][j][i] != 1)
                            cf = face([Pl[k + n][j][i] for n in (-2, -1, 0, 1)],
                                      [V[k + n][j][i] for n in (-2, -1, 0, 1)],
                                      [DWZ[k + n][j][i] for n in (-2, -1, 0, 1)], DT, q,
                                      p["VolumeRelMax"], mV, lV, nb, u2V)
                            ZC[k][j][i], ZD[k][j][i], ZE[k][j][i], ZF[k][j][i] = (q * c for c in cf)
                    if no_adv:                                     # AD:3004-3013
                        for k in range(max(KF[j][i], 0), nk + 1):
                            if NFW[k][j][i] == 1:
                                ZC[k][j][i] = ZD[k][j][i] = ZE[k][j][i] = ZF[k][j][i] = 0.0
            TIv = ATi if nudge else TI
            if p["ImpExp_AdvV"] == 0.0:
                for k in range(1, nk + 1):
                    for j in range(1, nj + 1):
                        for i in range(1, ni + 1):
                            if CW[k][j][i] == 1:
                                fl = ZC[k][j][i] * Pl[k - 2][j][i] + ZD[k][j][i] * Pl[k - 1][j][i] + \
                                    ZE[k][j][i] * Pl[k][j][i] + ZF[k][j][i] * Pl[k + 1][j][i]
                                TIv[k - 1][j][i] = TIv[k - 1][j][i] - fl * DT / V[k - 1][j][i]
                                TIv[k][j][i] = TIv[k][j][i] + fl * DT / V[k][j][i]
            elif nudge:                                # VerticalAdvection_Nudge, by layers
                for k in range(1, nk + 1):
                    for j in range(1, nj + 1):
                        for i in range(1, ni + 1):
                            if CW[k][j][i] == 1:
                                dt1, dt2 = DT / V[k - 1][j][i], DT / V[k][j][i]
                                AD[k][j][i] = AD[k][j][i] - ZD[k][j][i] * dt2
                                AE[k][j][i] = AE[k][j][i] - ZE[k][j][i] * dt2
                                AE[k - 1][j][i] = AE[k - 1][j][i] + ZD[k][j][i] * dt1
                                AF[k - 1][j][i] = AF[k - 1][j][i] + ZE[k][j][i] * dt1
            else:
                def upd(k, j, i, dt1, dt2):
                    D[k][j][i] = D[k][j][i] - ZD[k][j][i] * dt2
                    E[k][j][i] = E[k][j][i] - ZE[k][j][i] * dt2
                    E[k - 1][j][i] = E[k - 1][j][i] + ZD[k][j][i] * dt1
                    F[k - 1][j][i] = F[k - 1][j][i] + ZE[k][j][i] * dt1
                if p["Docycle_method"] == 1:
                    for j in range(1, nj + 1):
                        for i in range(1, ni + 1):
                            if CW[nk][j][i] == 1:
                                kb = KF[j][i]
                                vb = V[kb][j][i]
                                for k in range(kb + 1, nk + 1):
                                    dt1 = DT / vb
                                    dt2 = DT / V[k][j][i]
                                    vb = V[k][j][i]
                                    upd(k, j, i, dt1, dt2)
                else:
                    for k in range(1, nk + 1):
                        for j in range(1, nj + 1):
                            for i in range(1, ni + 1):
                                if CW[k][j][i] == 1:
                                    upd(k, j, i, DT / V[k - 1][j][i], DT / V[k][j][i])
            if cflux and p["ImpExp_AdvV"] < 1.0:
                _adv_flux(FAZ, ZC, ZD, ZE, ZF, Pl, CW, 1.0 - p["ImpExp_AdvV"], ni, nj, nk, 2)

    if nudge:                                          # AdvectionNudging AD:1989-2068
        nc = p["AdvectionNudgingCells"]
        in_ = jn_ = 0                                  # kept across cells, as in one OpenMP thread
        for j in range(1, nj + 1):
            for i in range(1, ni + 1):
                cell = False
                if i < nc + 1:
                    cell, in_ = True, max(0, i)
                elif i > ni - nc:
                    cell, in_ = True, max(0, ni - i + 1)
                if j < nc + 1:
                    cell, jn_ = True, max(0, j)
                elif j > nj - nc:
                    cell, jn_ = True, max(0, nj - j + 1)
                n = float(min(in_, jn_)) / nc if cell else 1.0
                for k in range(1, nk + 1):
                    if OP[k][j][i] == 1:
                        TI[k][j][i] = TI[k][j][i] + n * ATi[k][j][i]
                        D[k][j][i] = D[k][j][i] + n * AD[k][j][i]
                        E[k][j][i] = E[k][j][i] + n * AE[k][j][i]
                        F[k][j][i] = F[k][j][i] + n * AF[k][j][i]

    if R is not None:
        bc = p["BoundaryCondition"]
        tdec = 1.0 / (1.0 + p["DecayTime"] / DT)
        PO = [[row[:] for row in lay] for lay in Pl] if bc == 6 else None
        for j in range(1, nj + 1):
            for i in range(1, ni + 1):
                if BP[j][i] != 1:
                    continue
                for k in range(abs(KF[j][i]), nk + 1):
                    if OP[k][j][i] != 1:
                        continue
                    dtv = DT / V[k][j][i]
                    if bc in (2, 5):
                        a1 = OP[k][j][i + 1] * (1 - BP[j][i + 1])
                        a2 = OP[k][j][i - 1] * (1 - BP[j][i - 1])
                        a3 = OP[k][j + 1][i] * (1 - BP[j + 1][i])
                        a4 = OP[k][j - 1][i] * (1 - BP[j - 1][i])
                        at = float(a1 + a2 + a3 + a4)
                        if at > 0:
                            inner = (Pl[k][j][i + 1] * a1 + Pl[k][j][i - 1] * a2 + Pl[k][j + 1][i] * a3 +
                                     Pl[k][j - 1][i] * a4) / at
                            ext = inner * (1.0 - tdec) + R[k][j][i] * tdec
                        else:
                            ext = R[k][j][i]
                        TI[k][j][i] = ext
                        D[k][j][i], E[k][j][i], F[k][j][i] = 0.0, 1.0, 0.0
                    elif bc in (4, 8):                 # AD:5645-5650
                        TI[k][j][i] = Pl[k][j][i]
                        D[k][j][i], E[k][j][i], F[k][j][i] = 0.0, 1.0, 0.0
                    elif bc == 7:                      # AD:5603-5631
                        wf = Qx[k][j][i] * CU[k][j][i] - Qx[k][j + 1][i] * CU[k][j + 1][i] + \
                            Qy[k][j][i] * CV[k][j][i] - Qy[k][j][i + 1] * CV[k][j][i + 1] + \
                            Qz[k][j][i] * CW[k][j][i] - Qz[k + 1][j][i] * CW[k + 1][j][i] - \
                            (V[k][j][i] - Vo[k][j][i]) / DT
                        if wf < 0.0:
                            g = _null_grad(Pl, CU, CV, k, j, i)
                            TI[k][j][i] = Pl[k][j][i] if g is None else g
                            D[k][j][i], E[k][j][i], F[k][j][i] = 0.0, 1.0, 0.0
                        else:
                            E[k][j][i] = E[k][j][i] + wf * dtv
                    else:
                        wf = Qx[k][j][i] * CU[k][j][i] - Qx[k][j + 1][i] * CU[k][j + 1][i] + \
                            Qy[k][j][i] * CV[k][j][i] - Qy[k][j][i + 1] * CV[k][j][i + 1] + \
                            Qz[k][j][i] * CW[k][j][i] - Qz[k + 1][j][i] * CW[k + 1][j][i] - \
                            (V[k][j][i] - Vo[k][j][i]) / DT
                        if bc == 6:                    # AD:5496-5569
                            nrm = _orlanski_normal(ni, nj, i, j)
                            if nrm is None:
                                raise ValueError("Orlanski Advection 2")
                            di, dj, en, ie, je = nrm
                            limit = 10. * DT / (DUX[j][i] + DVY[j][i]) * 2
                            ext = _orlanski(Pl, PO, R, OP, k, ni, nj, di, dj, ie, je, en, limit, DT, wf * dtv)
                        else:
                            ext = Pl[k][j][i] * (1.0 - tdec) + R[k][j][i] * tdec
                        if wf < 0.0:
                            TI[k][j][i] = TI[k][j][i] - wf * ext * dtv
                        else:
                            E[k][j][i] = E[k][j][i] + wf * dtv

        if PO is not None and PropOld is not None:
            PropOld[...] = PO

    for k in range(K):
        for j in range(J):
            for i in range(I):
                if LP[k][j][i] == 1:
                    TI[k][j][i] = NULL_REAL

    # a one-layer domain solves the implicit direction instead (AD:1758-1858)
    if nk == 1 and (p["ImpExp_AdvXX"] == 1.0 or p["ImpExp_AdvYY"] == 1.0):
        _thomas_lines(D, E, F, TI, Pl, p["ImpExp_AdvXX"] == 1.0, ni, nj, nk)
        solve_columns = False
    else:
        solve_columns = True
    # THOMASZ_NewType2
    W = [0.0] * (nk + 2)
    G = [0.0] * (nk + 2)
    for j in range(1, nj + 1) if solve_columns else ():
        for i in range(1, ni + 1):
            if WP[nk][j][i] != 1:
                continue
            W[1] = -F[1][j][i] / E[1][j][i]
            G[1] = TI[1][j][i] / E[1][j][i]
            for k in range(2, nk + 2):
                aux = E[k][j][i] + D[k][j][i] * W[k - 1]
                if abs(aux) > 0:
                    W[k] = -F[k][j][i] / aux
                    G[k] = (TI[k][j][i] - D[k][j][i] * G[k - 1]) / aux
                else:
                    W[k] = 0.0
                    G[k] = 0.0
            Pl[nk + 1][j][i] = G[nk + 1]
            for k in range(nk, 0, -1):
                Pl[k][j][i] = W[k] * Pl[k + 1][j][i] + G[k]

    # boundary conditions applied after the solve (AD:1874-1880)
    if p["BoundaryCondition"] == 4:                  # ImposeNullGradient AD:1926-1987
        for j in range(1, nj + 1):
            for i in range(1, ni + 1):
                if BP[j][i] != 1:
                    continue
                for k in range(abs(KF[j][i]), nk + 1):
                    g = _null_grad(Pl, CU, CV, k, j, i)
                    if g is not None:
                        Pl[k][j][i] = g
    elif p["BoundaryCondition"] == 8:                # Prop_CyclicBoundary AD:2121-2224
        for j in range(1, nj + 1):
            for i in range(1, ni + 1):
                if BP[j][i] == 1:
                    for k in range(1, nk + 1):
                        Pl[k][j][i] = R[k][j][i]
        for i in range(2, ni):
            if BP[1][i] == 1 and BP[nj][i] == 1:
                for k in range(max(KF[nj - 1][i], 0), nk + 1):
                    Pl[k][1][i] = Pl[k][nj - 1][i]
                for k in range(max(KF[2][i], 0), nk + 1):
                    Pl[k][nj][i] = Pl[k][2][i]
        for j in range(2, nj):
            if BP[j][1] == 1 and BP[j][ni] == 1:
                for k in range(max(KF[j][ni - 1], 0), nk + 1):
                    Pl[k][j][1] = Pl[k][j][ni - 1]
                for k in range(max(KF[j][2], 0), nk + 1):
                    Pl[k][j][ni] = Pl[k][j][2]
    if cflux:                                        # implicit parts, new field (AD:1882-1916)
        if p["ImpExp_AdvV"] > 0.0 and nk > 1:
            _adv_flux(FAZ, ZC, ZD, ZE, ZF, Pl, CW, p["ImpExp_AdvV"], ni, nj, nk, 2)
        if p["ImpExp_DifV"] > 0.0 and nk > 1:
            _dif_flux_z(FDZ, Kz, DUX, DVY, DZZ, Pl, CW, p["ImpExp_DifV"], ni, nj, nk)
        if p["ImpExp_AdvXX"] == 1.0:
            _adv_flux(FAX, XC, XD, XE, XF, Pl, CU, p["ImpExp_AdvXX"], ni, nj, nk, 0)
        if p["ImpExp_AdvYY"] == 1.0:
            _adv_flux(FAY, YC, YD, YE, YF, Pl, CV, p["ImpExp_AdvYY"], ni, nj, nk, 1)
        if fluxes is not None:
            for n, a in zip(("AdvFluxX", "AdvFluxY", "AdvFluxZ", "DifFluxX", "DifFluxY", "DifFluxZ"),
                            (FAX, FAY, FAZ, FDX, FDY, FDZ)):
                fluxes[n] = np.array(a)
    P[...] = Pl
