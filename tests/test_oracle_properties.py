"""Known-answer properties of the FP64 oracle (the reference has no tests for this path)."""
import numpy as np
import pytest

from mohid_gb300 import synth
from oracle import oracle as O
from tests.cases import domain

NULL = -9.9e15


def test_thomasz_matches_dense_solve(built):
    rng = np.random.default_rng(0)
    ni, nj, nk = 5, 4, 7
    sh = (nk + 2, nj + 2, ni + 2)
    D = rng.uniform(-1, 0, sh); F = rng.uniform(-1, 0, sh)
    E = 2.5 + rng.uniform(0, 1, sh); TI = rng.normal(size=sh)
    # row KUB+1 as AdvectionDiffusion leaves it: D = F = 0, E = 1, TI = 0
    D[nk + 1] = 0.0; F[nk + 1] = 0.0; E[nk + 1] = 1.0; TI[nk + 1] = 0.0
    D[1] = 0.0                      # row 1 has no sub-diagonal (THOMASZ ignores it)
    F[nk] = 0.0                     # couple rows 1..nk only
    WP = np.ones(sh, dtype=np.int32); WP[nk, 2, 3] = 0   # one column not solved
    RES = np.full(sh, 7.0)
    assert O.thomasz(D, E, F, TI, RES, WP) == 0
    for j in range(1, nj + 1):
        for i in range(1, ni + 1):
            if WP[nk, j, i] != 1:
                assert np.all(RES[:, j, i] == 7.0)
                continue
            A = np.zeros((nk + 1, nk + 1)); b = TI[1:, j, i].copy()
            for r in range(nk + 1):
                k = r + 1
                A[r, r] = E[k, j, i]
                if r > 0: A[r, r - 1] = D[k, j, i]
                if r < nk: A[r, r + 1] = F[k, j, i]
            x = np.linalg.solve(A, b)
            np.testing.assert_allclose(RES[1:, j, i], x, rtol=1e-12, atol=1e-14)


def test_thomasz_zero_pivot_reported(built):
    sh = (5, 3, 3)
    D = np.zeros(sh); E = np.ones(sh); F = np.zeros(sh); TI = np.ones(sh)
    D[2, 1, 1] = 1.0; E[2, 1, 1] = 0.0              # aux = 0 + 1 * W(1) = 0 (W(1) = 0)
    WP = np.ones(sh, dtype=np.int32)
    RES = np.zeros(sh)
    assert O.thomasz(D, E, F, TI, RES, WP) == 6      # MOHID_AD_ERR_ZERO_PIVOT


@pytest.mark.parametrize("grid", ["coast", "zlevel", "open", "nsopen"])
# (implicit horizontal advection is a fractional step in the reference -- a
# line solve in one direction, then the columns -- and keeps a constant only to
# the splitting error, so it is not in this list)
@pytest.mark.parametrize("opt", [dict(), dict(AdvMethodH=4, TVDLimitationH=4, Upwind2H=1),
                                 dict(AdvMethodH=4, TVDLimitationH=1, Upwind2H=1)])
@pytest.mark.parametrize("bc", [1, 2, 4, 7, 8])
def test_constancy_preserved(built, grid, opt, bc):
    d = domain(grid)
    wp = d.water_mask()
    P = np.where(wp, 3.25, 0.0)
    R = np.full(d.shape3, 3.25) if d.spec.open_sides else None
    if R is None and bc == 8:
        pytest.skip("cyclic boundaries read the reference")
    p = O.params(DTProp=30.0, BoundaryCondition=bc, **opt)
    for _ in range(5):
        assert O.step(d, P, p, ReferenceProp=R) == 0
    assert np.max(np.abs(P[wp] - 3.25)) < 1e-12


@pytest.mark.parametrize("grid", ["coast", "zlevel", "layer1"])
@pytest.mark.parametrize("opt", [dict(), dict(AdvMethodH=4, TVDLimitationH=4, Upwind2H=1), dict(ImpExp_AdvXX=1.0),
                                 dict(ImpExp_AdvYY=1.0, AdvMethodH=4, TVDLimitationH=1, Upwind2H=1),
                                 dict(ImpExp_DifV=0.5), dict(AdvMethodV=4, TVDLimitationV=4, Upwind2V=1)])
def test_mass_conserved_closed(built, grid, opt):
    d = domain(grid)
    P = d.tracer(3, 1.0, 0.8, seed=4)
    p = O.params(DTProp=30.0, **opt)
    m0 = O.mass(d, P)
    for _ in range(20):
        assert O.step(d, P, p) == 0
    m1 = O.mass(d, P)
    assert abs(m1 - m0) / abs(m0) < 1e-13


def test_mass_with_moving_volumes(built):
    # sum V*P_new equals sum Vold*P_old when volumes change inside columns
    d = synth.generate(synth.GenSpec(ni=12, nj=10, nk=6, land_frac=0.15, land_kind=1,
                                     vol_var=0.02, seed=21, dt=30.0))
    P = d.tracer(1, 5.0, 25.0, seed=2)
    wp = d.water_mask()
    before = np.sum(d.VolumeZOld[wp] * P[wp])
    assert O.step(d, P, O.params(DTProp=30.0)) == 0
    after = np.sum(d.VolumeZ[wp] * P[wp])
    assert abs(after - before) / before < 1e-13


@pytest.mark.parametrize("spec", [dict(ni=10, nj=6, nk=3, land_frac=0.0, seed=7, open_sides=12, bathy_kind=1),
                                  dict(ni=11, nj=9, nk=5, land_frac=0.15, land_kind=1, seed=9, open_sides=3,
                                       bathy_kind=1)])
@pytest.mark.parametrize("opt", [dict(), dict(AdvMethodH=4, TVDLimitationH=1, Upwind2H=1)])
@pytest.mark.parametrize("decay", [0.0, 300.0])
def test_mass_budget_open_boundaries(built, spec, opt, decay):
    # static volumes, MassConservation open boundaries: the mass changes by
    # exactly the flux through the boundary cells' exterior faces
    from tests.cases import boundary_flux
    d = synth.generate(synth.GenSpec(**spec, dt=30.0))
    P = d.tracer(3, 1.0, 0.6, seed=5)
    R = d.reference(2.5, 0.3, seed=6)
    p = O.params(DTProp=30.0, BoundaryCondition=1, DecayTime=decay, **opt)
    wp = d.water_mask()
    scale = np.sum(np.abs(d.VolumeZ[wp] * P[wp]))
    moved = 0.0
    for _ in range(5):
        m0, P0 = O.mass(d, P), P.copy()
        assert O.step(d, P, p, ReferenceProp=R) == 0
        phi = boundary_flux(d, P0, P, R, 30.0, decay)
        assert abs(O.mass(d, P) - m0 - phi) <= 1e-13 * scale
        moved += abs(phi)
    assert moved > 1e-6 * scale                  # the boundaries do move mass


@pytest.mark.parametrize("opt", [dict(), dict(AdvMethodH=4, TVDLimitationH=4, Upwind2H=1), dict(ImpExp_DifV=0.5),
                                 dict(ImpExp_AdvV=0.0, AdvMethodV=4, TVDLimitationV=1, Upwind2V=1),
                                 dict(AdvMethodV=4, TVDLimitationV=4, Upwind2V=1), dict(Docycle_method=2)])
@pytest.mark.parametrize("grid", ["coast", "zlevel"])
def test_cell_fluxes_close_each_cell_budget(built, grid, opt):
    # closed domain, static volumes: in every water cell
    # V * P_new - VOld * P_old = DT * (net advective + diffusive flux in)
    d = domain(grid)
    P = d.tracer(3, 1.0, 0.6, seed=8)
    P0 = P.copy()
    work = O.Work(d)
    assert O.step(d, P, O.params(DTProp=30.0, CellFluxes=1, **opt), work=work) == 0
    f = O.cell_fluxes(d, work)
    FX, FY, FZ = (f["AdvFlux" + c] + f["DifFlux" + c] for c in "XYZ")
    nk, nj, ni = d.nk, d.nj, d.ni
    c = (slice(1, nk + 1), slice(1, nj + 1), slice(1, ni + 1))
    net = (FX[c] - FX[1:nk + 1, 2:nj + 2, 1:ni + 1] + FY[c] - FY[1:nk + 1, 1:nj + 1, 2:ni + 2] + FZ[c] -
           FZ[2:nk + 2, 1:nj + 1, 1:ni + 1])
    wp = d.water_mask()[c]
    lhs = d.VolumeZ[c] * P[c] - d.VolumeZOld[c] * P0[c]
    scale = np.max(np.abs(d.VolumeZ[c] * P[c]))
    assert np.max(np.abs((lhs - 30.0 * net)[wp])) <= 1e-12 * scale
    assert np.abs(net[wp]).max() > 1e-6 * scale / 30.0         # the fluxes are not all zero


def test_noflux_everywhere_freezes_static_field(built):
    # every face masked for advection and diffusion, static volumes: the step
    # is VolumeVariation alone, P * VOld / V = P
    d = domain("coast")
    P = d.tracer(3, 1.0, 0.5, seed=6)
    P0 = P.copy()
    ones = tuple(np.ones(d.shape3, dtype=np.int32) for _ in range(3))
    p = O.params(DTProp=30.0, NoAdvFlux=1, NoDifFlux=1, AdvMethodH=4, TVDLimitationH=4, Upwind2H=1)
    assert O.step(d, P, p, NoFlux=ones) == 0
    wp = d.water_mask()
    assert np.array_equal(P[wp], P0[wp])
    # the masks are required when the flags are set
    assert O.step(d, P.copy(), p) == 9


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_discharge_mass_budget(built, seed):
    # closed domain, static volumes, discharges into open cells: the mass
    # changes by the inflows (flow * DT * concentration, bypasses included) and
    # the withdrawals (flow * DT * DischConcMF * new value)
    from tests.cases import discharges
    d = domain("zlevel")
    ds = discharges(d, seed=seed)
    P = d.tracer(3, 1.0, 0.5, seed=7)
    P0 = P.copy()
    assert O.step(d, P, O.params(DTProp=30.0, AdvMethodH=4, TVDLimitationH=4, Upwind2H=1), Disch=ds) == 0
    a = d.arrays
    dm, n = 0.0, 0
    for dis in range(len(ds["nCells"])):
        if ds["ignore"][dis]:
            continue
        for _ in range(ds["nCells"][dis]):
            i, j = ds["I"][n], ds["J"][n]
            if ds["vert"][dis] == 5:
                k0 = a["KFloorZ"][j, i] if ds["Kmin"][n] == -9999999 else ds["Kmin"][n]
                k1 = d.nk if ds["Kmax"][n] == -9999999 else ds["Kmax"][n]
            else:
                k0 = k1 = ds["K"][n]
            wc = sum(a["DWZ"][k, j, i] for k in range(k0, k1 + 1))
            for k in range(k0, k1 + 1):
                assert a["OpenPoints3D"][k, j, i] == 1
                flow = ds["Flow"][n] * (a["DWZ"][k, j, i] / wc if ds["vert"][dis] == 5 else 1.0)
                if ds["bypass"][dis] or flow > 0:
                    dm += flow * 30.0 * ds["Conc"][n]
                else:
                    dm += flow * 30.0 * ds["ConcMF"][n] * P[k, j, i]
            n += 1
    m0, m1 = O.mass(d, P0), O.mass(d, P)
    assert abs((m1 - m0) - dm) <= 1e-12 * abs(m0)
    assert abs(dm) > 1e-9 * abs(m0)
    # discharge cells outside the work box are rejected
    bad = dict(ds, I=ds["I"].copy())
    bad["I"][0] = d.ni + 1
    assert O.step(d, P0.copy(), O.params(DTProp=30.0), Disch=bad) == 1


def test_upwind_one_layer_matches_textbook_update(built):
    # one layer, no diffusion, no surface flux: the step is the first-order
    # upwind finite-volume update
    #   V P_new = VOld P + DT * (sum over U and V faces of Q * P_upstream, signed)
    # with fluxes only where both cells are open and the face computes
    d = domain("layer1")
    a = d.arrays
    rng = np.random.default_rng(3)
    a["Visc_H"][:] = 0.0
    a["Diff_V"][:] = 0.0
    a["Wflux_Z"][:] = 0.0
    a["Wflux_X"][:] = rng.uniform(-2.0, 2.0, a["Wflux_X"].shape) * a["ComputeFacesU3D"]
    a["Wflux_Y"][:] = rng.uniform(-2.0, 2.0, a["Wflux_Y"].shape) * a["ComputeFacesV3D"]
    P = d.tracer(3, 1.0, 0.5, seed=9)
    P0 = P.copy()
    DT = 30.0
    assert O.step(d, P, O.params(DTProp=DT, SchmidtBackground_V=0.0)) == 0
    OP, CU, CV = a["OpenPoints3D"], a["ComputeFacesU3D"], a["ComputeFacesV3D"]
    V, Vo = a["VolumeZ"], a["VolumeZOld"]
    k = 1
    for j in range(1, d.nj + 1):
        for i in range(1, d.ni + 1):
            if a["WaterPoints3D"][k, j, i] != 1:
                continue
            net = 0.0
            for (jj, ii, sign, q, cf) in ((j, i, 1, a["Wflux_X"], CU), (j + 1, i, -1, a["Wflux_X"], CU),
                                          (j, i, 1, a["Wflux_Y"], CV), (j, i + 1, -1, a["Wflux_Y"], CV)):
                if cf[k, jj, ii] != 1:
                    continue
                up = (jj - 1, ii) if q is a["Wflux_X"] else (jj, ii - 1)
                if OP[k, jj, ii] != 1 or OP[k, up[0], up[1]] != 1:
                    continue
                qf = q[k, jj, ii]
                pu = P0[k, up[0], up[1]] if qf > 0 else P0[k, jj, ii]
                net += sign * qf * pu
            want = (Vo[k, j, i] * P0[k, j, i] + DT * net) / V[k, j, i]
            if OP[k, j, i] != 1:
                want = P0[k, j, i]
            assert P[k, j, i] == pytest.approx(want, rel=1e-13, abs=1e-13)


@pytest.mark.parametrize("limiter", [1, 2, 3, 4])
def test_tvd_face_value_matches_textbook(built, limiter):
    # uniform cells: ComputeAdvectionFace's P2_TVD face value is the textbook
    # limited upwind value  P_up + 0.5 * psi(r) * w * (P_down - P_up),
    # r = (P_up - P_farup) / (P_down - P_up), with the reference's signed
    # Courant number Cr = Q dt / V_up (FN:11045-11052): w = 1 - Cr, which is
    # 1 - |Cr| for Q > 0 and 1 + |Cr| for Q < 0
    psi = {1: lambda r: max(0.0, min(1.0, r)),                             # MinMod
           2: lambda r: 0.0 if r < 0 else 2.0 * r / (1.0 + r),             # VanLeer
           3: lambda r: max(0.0, min(2.0, 2.0 * r, (1.0 + r) / 2.0)),      # MUSCL
           4: lambda r: max(0.0, min(1.0, 2.0 * r), min(r, 2.0))}[limiter]  # SuperBee
    rng = np.random.default_rng(limiter)
    V4, du4, dt = np.full(4, 50.0), np.full(4, 10.0), 5.0
    n = 0
    for _ in range(200):
        P4 = rng.uniform(0.0, 10.0, 4)
        Q = float(rng.uniform(-3.0, 3.0))
        if abs(Q) < 0.1:
            continue
        up, down, far = (1, 2, 0) if Q > 0 else (2, 1, 3)
        if abs(P4[down] - P4[up]) < 1e-3:
            continue
        rc, CF = O.advection_face(P4, V4, du4, dt, Q, 1.5, 4, limiter, False, True)
        assert rc == 0
        r = (P4[up] - P4[far]) / (P4[down] - P4[up])
        Cr = Q * dt / V4[up]
        want = P4[up] + 0.5 * psi(r) * (1.0 - Cr) * (P4[down] - P4[up])
        assert float(np.dot(CF, P4)) == pytest.approx(want, rel=1e-12, abs=1e-12)
        n += 1
    assert n > 150


def test_quick_and_central_face_values_match_textbook(built):
    # UpwindOrder2 (FaceConcUpSecondOrder FN:11055) is the QUICK face value
    # 6/8 P_up + 3/8 P_down - 1/8 P_farup where the volumes vary by less than
    # VolumeRelMax (first order beyond); CentralDif is the distance-weighted mean
    rng = np.random.default_rng(11)
    du4, dt = np.array([10.0, 12.0, 9.0, 11.0]), 5.0
    for _ in range(100):
        P4 = rng.uniform(0.0, 10.0, 4)
        Q = float(rng.choice([-1.0, 1.0]) * rng.uniform(0.1, 3.0))
        up, down, far = (1, 2, 0) if Q > 0 else (2, 1, 3)
        V4 = np.full(4, 50.0)
        rc, CF = O.advection_face(P4, V4, du4, dt, Q, 1.5, 2, 4, False, True)
        assert rc == 0
        quick = 6.0 / 8.0 * P4[up] + 3.0 / 8.0 * P4[down] - 1.0 / 8.0 * P4[far]
        assert float(np.dot(CF, P4)) == pytest.approx(quick, rel=1e-13, abs=1e-13)
        V4[up] = 100.0                                    # VolumeRel 2 > 1.5: first order
        rc, CF = O.advection_face(P4, V4, du4, dt, Q, 1.5, 2, 4, False, True)
        assert float(np.dot(CF, P4)) == pytest.approx(P4[up], rel=1e-13, abs=1e-13)
        rc, CF = O.advection_face(P4, np.full(4, 50.0), du4, dt, Q, 1.5, 5, 4, False, True)
        central = (du4[2] * P4[1] + du4[1] * P4[2]) / (du4[1] + du4[2])
        assert float(np.dot(CF, P4)) == pytest.approx(central, rel=1e-13, abs=1e-13)


def test_pure_vertical_diffusion_matches_discrete_solve(built):
    d = synth.generate(synth.GenSpec(ni=1, nj=1, nk=9, land_frac=0.0, seed=2, dt=600.0,
                                     kz_median=1e-2, kz_logsigma=0.8))
    a = d.arrays
    for n in ("Wflux_X", "Wflux_Y", "Wflux_Z"):
        a[n][...] = 0.0
    # a lone column has no horizontal compute face, so MOHID would not open its
    # W faces (ModuleMap.F90:1598-1608); open them here to isolate the solve
    a["ComputeFacesW3D"][2:d.nk + 1, 1, 1] = 1
    a["OpenPoints3D"][1:d.nk + 1, 1, 1] = 1
    P = d.tracer(1, 5.0, 25.0, seed=1)
    dt = 600.0
    p = O.params(DTProp=dt, SchmidtBackground_V=0.0)
    P0 = P.copy()
    assert O.step(d, P, p) == 0
    nk = d.nk
    V = a["VolumeZ"][:, 1, 1]; Kz = a["Diff_V"][:, 1, 1]; DZZ = a["DZZ"][:, 1, 1]
    area = a["DUX"][1, 1] * a["DVY"][1, 1]
    M = np.eye(nk)
    for k in range(2, nk + 1):           # face k between cells k-1 and k
        g = Kz[k] * area / DZZ[k - 1] * dt
        r, s = k - 2, k - 1
        M[r, r] += g / V[k - 1]; M[r, s] -= g / V[k - 1]
        M[s, s] += g / V[k]; M[s, r] -= g / V[k]
    x = np.linalg.solve(M, P0[1:nk + 1, 1, 1])
    np.testing.assert_allclose(P[1:nk + 1, 1, 1], x, rtol=1e-12)


@pytest.mark.parametrize("limiter", [1, 2, 3, 4])
def test_tvd_step_creates_no_new_extrema(built, limiter):
    # quasi 1-D channel, west-east through-flow, a step profile
    d = synth.generate(synth.GenSpec(ni=1, nj=60, nk=1, land_frac=0.0, open_sides=3,
                                     seed=5, dt=30.0, umax=0.5))
    a = d.arrays
    P = np.zeros(d.shape3)
    P[1, 1, 1:31] = 1.0; P[1, 1, 31:61] = 0.2
    R = np.full(d.shape3, 0.6)
    p = O.params(DTProp=30.0, AdvMethodH=4, TVDLimitationH=limiter, Upwind2H=1)
    for _ in range(30):
        assert O.step(d, P, p, ReferenceProp=R) == 0
        w = P[1, 1, 1:61]
        assert w.max() <= 1.0 + 1e-12 and w.min() >= 0.2 - 1e-12


def test_land_and_halo_handling(built):
    d = domain("zlevel")
    a = d.arrays
    P = d.tracer(4, 2.0, 0.0, seed=1) + 0.0
    P[a["WaterPoints3D"] == 0] = 5.0                  # land and halo values to watch
    P0 = P.copy()
    assert O.step(d, P, O.params(DTProp=30.0)) == 0
    nk = d.nk
    solved = a["WaterPoints3D"][nk] == 1
    for j in range(1, d.nj + 1):
        for i in range(1, d.ni + 1):
            col = P[:, j, i]
            if not solved[j, i]:
                assert np.array_equal(col, P0[:, j, i])       # untouched
                continue
            kf = a["KFloorZ"][j, i]
            assert np.all(col[1:kf] == NULL)                   # below KFloor: null_real
            assert col[nk + 1] == 0.0                          # row KUB+1 solved to 0
            assert col[0] == P0[0, j, i]                       # row 0 untouched
    # halo columns untouched
    assert np.array_equal(P[:, 0, :], P0[:, 0, :]) and np.array_equal(P[:, :, 0], P0[:, :, 0])


@pytest.mark.parametrize("bad,code", [
    (dict(ImpExp_DifH=1.0), 3), (dict(ImpExp_AdvXX=1.0, ImpExp_AdvYY=1.0), 3),
    (dict(AdvMethodV=2, Upwind2V=1), 3), (dict(AdvMethodH=4, Upwind2H=0), 3),
    (dict(AdvMethodH=9), 3), (dict(ImpExp_AdvV=0.5), 3), (dict(Docycle_method=3), 3),
    (dict(ImpExp_AdvXX=0.5), 3), (dict(NoAdvFlux=1), 9),
    (dict(AdvectionNudging=1, AdvectionNudgingCells=2, ImpExp_AdvXX=1.0), 4),
    (dict(AdvectionNudging=1, AdvectionNudgingCells=2, Vertical1D=1), 4),
])
def test_rejected_options(built, bad, code):
    d = domain("coast")
    P = d.tracer(4, 1.0, 0.0, seed=1)
    P0 = P.copy()
    assert O.step(d, P, O.params(DTProp=30.0, **bad)) == code
    assert np.array_equal(P, P0)


def test_boundary_condition_rules(built):
    d = domain("open")
    P = d.tracer(4, 1.0, 0.0, seed=1)
    R = d.reference(2.0, 0.3, seed=2)
    # cyclic boundaries read the reference (AD:2150)
    assert O.step(d, P.copy(), O.params(DTProp=30.0, BoundaryCondition=8)) == 3
    assert O.step(d, P.copy(), O.params(DTProp=30.0, BoundaryCondition=3), ReferenceProp=R) == 3
    # without a reference a BC other than 4 and 8 changes nothing (AD:1874-1880, AD:5816)
    a, b = P.copy(), P.copy()
    assert O.step(d, a, O.params(DTProp=30.0, BoundaryCondition=6)) == 0
    assert O.step(d, b, O.params(DTProp=30.0, BoundaryCondition=1)) == 0
    assert np.array_equal(a, b)


def test_null_gradient_sets_boundary_to_neighbour_mean(built):
    # the solve as without open boundaries, then every boundary cell with a
    # compute face takes the mean of its neighbours across compute faces, swept
    # in the reference's order (a cell sees the new values of the boundary
    # cells swept before it)
    d = domain("nsopen")
    P = d.tracer(3, 1.0, 0.5, seed=4)
    X = P.copy()
    assert O.step(d, P, O.params(DTProp=30.0, BoundaryCondition=4)) == 0
    assert O.step(d, X, O.params(DTProp=30.0, BoundaryCondition=1)) == 0
    a = d.arrays
    CU, CV, BP, KF = a["ComputeFacesU3D"], a["ComputeFacesV3D"], a["BoundaryPoints2D"], a["KFloorZ"]
    n = 0
    for j in range(1, d.nj + 1):
        for i in range(1, d.ni + 1):
            if BP[j, i] != 1:
                continue
            for k in range(abs(KF[j, i]), d.nk + 1):
                aux = CV[k, j, i + 1] + CV[k, j, i] + CU[k, j + 1, i] + CU[k, j, i]
                if aux > 0:
                    X[k, j, i] = (X[k, j, i + 1] * CV[k, j, i + 1] + X[k, j, i - 1] * CV[k, j, i] +
                                  X[k, j + 1, i] * CU[k, j + 1, i] + X[k, j - 1, i] * CU[k, j, i]) / aux
                    n += 1
    assert n > 0
    assert np.array_equal(P, X)


def test_cyclic_boundary_copies_opposite_interior(built):
    d = domain("nsopen")                                  # boundary rows i = 1 and i = ni
    P = d.tracer(3, 1.0, 0.5, seed=4)
    R = d.reference(2.0, 0.3, seed=5)
    assert O.step(d, P, O.params(DTProp=30.0, BoundaryCondition=8), ReferenceProp=R) == 0
    KF = d.arrays["KFloorZ"]
    for j in range(2, d.nj):
        for k in range(KF[j, d.ni - 1], d.nk + 1):
            assert P[k, j, 1] == P[k, j, d.ni - 1]
        for k in range(KF[j, 2], d.nk + 1):
            assert P[k, j, d.ni] == P[k, j, 2]
    # the corner columns keep the reference
    assert np.array_equal(P[1:d.nk + 1, 1, 1], R[1:d.nk + 1, 1, 1])


def test_compute_face_on_lower_edge_rejected(built):
    d = domain("coast")
    d.arrays["ComputeFacesU3D"][2, 1, 3] = 1               # U face at j = JLB (k=2, i=3)
    P = d.tracer(4, 1.0, 0.0, seed=1)
    assert O.step(d, P, O.params(DTProp=30.0)) == 1
