"""Plain FP64 drop-in on the GPU against the FP64 oracle (through the C-ABI).

Tolerance: the kernel evaluates every term in the reference's order without
fused multiply-add, so results are expected to be bit-identical; the bar
asserted is max relative difference <= 1e-12 over water cells plus exact
equality of land/null/halo cells.
"""
import ctypes as C

import numpy as np
import pytest

from mohid_gb300 import advdiff, configs, synth
from oracle import oracle as O
from tests.cases import SMALL, OPTIONS, domain

pytestmark = pytest.mark.gpu
RTOL = 1e-12


def _compare(d, Pg, Po):
    wp = d.water_mask()
    other = ~wp
    assert np.array_equal(Pg[other], Po[other])
    scale = np.maximum(np.abs(Po[wp]), 1e-30)
    rel = np.max(np.abs(Pg[wp] - Po[wp]) / scale) if wp.any() else 0.0
    assert rel <= RTOL, f"max rel diff {rel:.3e}"
    return rel


@pytest.mark.parametrize("grid", sorted(SMALL))
@pytest.mark.parametrize("opt", sorted(OPTIONS))
def test_gpu_matches_oracle_one_step(gpu, grid, opt):
    d = domain(grid)
    P0 = d.tracer(3, 1.0, 0.7, seed=9)
    pd = dict(DTProp=30.0, **OPTIONS[opt])
    Po = P0.copy()
    assert O.step(d, Po, O.params(**pd)) == 0
    ad = advdiff.AdvectionDiffusion(d)
    ad.set_hydro()
    Pg = P0.copy()
    ad.step(Pg, advdiff.params(**pd))
    ad.kill()
    _compare(d, Pg, Po)
    assert np.array_equal(Pg, Po), "expected bit-identical FP64 results"


@pytest.mark.parametrize("grid", ["open", "nsopen"])
@pytest.mark.parametrize("bc,decay", [(1, 0.0), (1, 600.0), (2, 0.0), (2, 300.0), (5, 0.0), (4, 0.0), (7, 0.0),
                                      (8, 0.0)])
@pytest.mark.parametrize("opt", ["upwind1", "tvd_minmod", "tvd_superbee"])
def test_gpu_open_boundaries(gpu, grid, bc, decay, opt):
    d = domain(grid)
    P0 = d.tracer(3, 1.0, 0.5, seed=1)
    R = d.reference(2.0, 0.3, seed=2)
    pd = dict(DTProp=30.0, BoundaryCondition=bc, DecayTime=decay, **OPTIONS[opt])
    Po = P0.copy()
    assert O.step(d, Po, O.params(**pd), ReferenceProp=R) == 0
    ad = advdiff.AdvectionDiffusion(d)
    ad.set_hydro()
    Pg = P0.copy()
    ad.step(Pg, advdiff.params(**pd), ReferenceProp=R)
    ad.kill()
    _compare(d, Pg, Po)
    assert np.array_equal(Pg, Po)


@pytest.mark.parametrize("bc", [4, 7, 8])
@pytest.mark.parametrize("with_ref", [True, False])
def test_gpu_boundary_sweeps_many_steps(gpu, bc, with_ref):
    # all four sides open (cyclic rows and columns, corners), a few steps on
    # the host and the device entry points: the post-solve sweeps in the
    # reference's order, bit for bit
    if bc in (7, 8) and not with_ref:
        pytest.skip("needs the reference")
    d = synth.generate(synth.GenSpec(ni=61, nj=47, nk=7, land_frac=0.1, land_kind=1, seed=13, open_sides=15,
                                     bathy_kind=1, dt=30.0))
    P0 = d.tracer(3, 1.0, 0.5, seed=1)
    R = d.reference(2.0, 0.3, seed=2) if with_ref else None
    pd = dict(DTProp=30.0, BoundaryCondition=bc, **OPTIONS["tvd_superbee"])
    Po = P0.copy()
    for _ in range(4):
        assert O.step(d, Po, O.params(**pd), ReferenceProp=R) == 0
    ad = advdiff.AdvectionDiffusion(d)
    ad.set_hydro()
    Pg = P0.copy()
    for _ in range(4):
        ad.step(Pg, advdiff.params(**pd), R)
    assert np.array_equal(Pg, Po)
    import torch
    a = torch.from_numpy(P0.copy()).cuda()
    b = torch.empty_like(a)
    Rd = torch.from_numpy(R).cuda() if with_ref else None
    for _ in range(4):
        ad.step_device(a, b, advdiff.params(**pd), Rd)
        a, b = b, a
    ad.sync()
    ad.kill()
    assert np.array_equal(a.cpu().numpy(), Po)


@pytest.mark.parametrize("opt", ["implicit_xx", "implicit_yy_tvd", "implicit_xx_central"])
@pytest.mark.parametrize("nk", [7, 1])
def test_gpu_implicit_horizontal_many_steps(gpu, opt, nk):
    # the line solve along j (XX) or i (YY), then the columns (or, with one
    # layer, the line solve alone), open boundaries, host and device entry
    # points, a few steps: bit for bit
    d = synth.generate(synth.GenSpec(ni=61, nj=47, nk=nk, land_frac=0.1, land_kind=1, seed=17, open_sides=15,
                                     bathy_kind=1, dt=30.0))
    P0 = d.tracer(3, 1.0, 0.5, seed=1)
    R = d.reference(2.0, 0.3, seed=2)
    pd = dict(DTProp=30.0, BoundaryCondition=1, DecayTime=300.0, **OPTIONS[opt])
    Po = P0.copy()
    for _ in range(4):
        assert O.step(d, Po, O.params(**pd), ReferenceProp=R) == 0
    ad = advdiff.AdvectionDiffusion(d)
    ad.set_hydro()
    Pg = P0.copy()
    for _ in range(4):
        ad.step(Pg, advdiff.params(**pd), R)
    assert np.array_equal(Pg, Po)
    import torch
    a = torch.from_numpy(P0.copy()).cuda()
    b = torch.empty_like(a)
    Rd = torch.from_numpy(R).cuda()
    for _ in range(4):
        ad.step_device(a, b, advdiff.params(**pd), Rd)
        a, b = b, a
    ad.sync()
    ad.kill()
    assert np.array_equal(a.cpu().numpy(), Po)


@pytest.mark.parametrize("grid", ["coast", "zlevel", "open", "layer1"])
@pytest.mark.parametrize("opt", ["upwind1", "tvd_superbee", "explicit_v_tvd", "theta_difv", "implicit_xx",
                                 "implicit_yy_tvd", "docycle2", "tvd_vertical", "vertical1d", "xzflow", "nulldif"])
def test_gpu_cell_fluxes_match_oracle(gpu, grid, opt):
    # CellFluxes: the six face-flux arrays of the step, bit for bit
    d = domain(grid)
    P0 = d.tracer(3, 1.0, 0.5, seed=2)
    R = d.reference(2.0, 0.3, seed=3) if d.spec.open_sides else None
    pd = dict(DTProp=30.0, CellFluxes=1, **OPTIONS[opt])
    Po = P0.copy()
    work = O.Work(d)
    assert O.step(d, Po, O.params(**pd), ReferenceProp=R, work=work) == 0
    fo = O.cell_fluxes(d, work)
    ad = advdiff.AdvectionDiffusion(d)
    ad.set_hydro()
    Pg = P0.copy()
    ad.step(Pg, advdiff.params(**pd), R)
    fg = ad.cell_fluxes()
    assert np.array_equal(Pg, Po)
    for n in O.FLUX_NAMES:
        assert np.array_equal(fg[n], fo[n]), n
    # a step without CellFluxes leaves none to read
    ad.step(Pg, advdiff.params(DTProp=30.0), R)
    with pytest.raises(advdiff.N.MohidAdError) as ei:
        ad.cell_fluxes()
    assert ei.value.code == 3
    ad.kill()


@pytest.mark.parametrize("grid", ["coast", "zlevel", "open"])
@pytest.mark.parametrize("flags", [dict(NoAdvFlux=1), dict(NoDifFlux=1), dict(NoAdvFlux=1, NoDifFlux=1)])
@pytest.mark.parametrize("opt", ["upwind1", "tvd_superbee", "explicit_v_tvd", "theta_difv", "implicit_xx"])
def test_gpu_noflux_masks(gpu, grid, flags, opt):
    from tests.cases import noflux_masks
    d = domain(grid)
    P0 = d.tracer(3, 1.0, 0.5, seed=4)
    R = d.reference(2.0, 0.3, seed=3) if d.spec.open_sides else None
    nf = noflux_masks(d, seed=5)
    pd = dict(DTProp=30.0, CellFluxes=1, **flags, **OPTIONS[opt])
    Po = P0.copy()
    work = O.Work(d)
    assert O.step(d, Po, O.params(**pd), ReferenceProp=R, work=work, NoFlux=nf) == 0
    fo = O.cell_fluxes(d, work)
    ad = advdiff.AdvectionDiffusion(d)
    ad.set_hydro()
    with pytest.raises(advdiff.N.MohidAdError) as ei:        # the masks are required
        ad.step(P0.copy(), advdiff.params(**pd), R)
    assert ei.value.code == 9
    ad.set_noflux(nf)
    Pg = P0.copy()
    ad.step(Pg, advdiff.params(**pd), R)
    fg = ad.cell_fluxes()
    ad.kill()
    assert np.array_equal(Pg, Po)
    for n in O.FLUX_NAMES:
        assert np.array_equal(fg[n], fo[n]), n


@pytest.mark.parametrize("grid", ["coast", "zlevel", "open", "layer1"])
@pytest.mark.parametrize("opt", ["upwind1", "tvd_superbee", "theta_difv", "implicit_xx"])
@pytest.mark.parametrize("seed", [0, 1])
def test_gpu_discharges(gpu, grid, opt, seed):
    # SetDischarges: point and uniform discharges, inflows, withdrawals,
    # a bypass and an ignored discharge; three steps through the host entry
    # point, then the same through the device one; bit for bit
    from tests.cases import discharges
    d = domain(grid)
    P0 = d.tracer(3, 1.0, 0.5, seed=2)
    R = d.reference(2.0, 0.3, seed=3) if d.spec.open_sides else None
    ds = discharges(d, seed=seed)
    pd = dict(DTProp=30.0, **OPTIONS[opt])
    Po = P0.copy()
    for _ in range(3):
        assert O.step(d, Po, O.params(**pd), ReferenceProp=R, Disch=ds) == 0
    ad = advdiff.AdvectionDiffusion(d)
    ad.set_hydro()
    ad.set_discharges(ds)
    Pg = P0.copy()
    for _ in range(3):
        ad.step(Pg, advdiff.params(**pd), R)
    assert np.array_equal(Pg, Po)
    import torch
    a = torch.from_numpy(P0.copy()).cuda()
    b = torch.empty_like(a)
    Rd = torch.from_numpy(R).cuda() if R is not None else None
    for _ in range(3):
        ad.step_device(a, b, advdiff.params(**pd), Rd)
        a, b = b, a
    ad.sync()
    assert np.array_equal(a.cpu().numpy(), Po)
    # unset: the step without discharges again
    ad.set_discharges(None)
    Pq, Pr = P0.copy(), P0.copy()
    ad.step(Pq, advdiff.params(**pd), R)
    assert O.step(d, Pr, O.params(**pd), ReferenceProp=R) == 0
    assert np.array_equal(Pq, Pr)
    # cells outside the work box are rejected
    bad = dict(ds, J=ds["J"].copy())
    bad["J"][0] = d.nj + 1
    with pytest.raises(advdiff.N.MohidAdError) as ei:
        ad.set_discharges(bad)
    assert ei.value.code == 1
    ad.kill()


def test_gpu_boundary_condition_rules(gpu):
    d = domain("open")
    P = d.tracer(4, 1.0, 0.0, seed=1)
    R = d.reference(2.0, 0.3, seed=2)
    ad = advdiff.AdvectionDiffusion(d)
    ad.set_hydro()
    for pd, ref, code in [(dict(BoundaryCondition=8), None, 3), (dict(BoundaryCondition=3), R, 3)]:
        assert O.step(d, P.copy(), O.params(DTProp=30.0, **pd), ReferenceProp=ref) == code
        with pytest.raises(advdiff.N.MohidAdError) as ei:
            ad.step(P.copy(), advdiff.params(DTProp=30.0, **pd), ref)
        assert ei.value.code == code
    ad.kill()


def test_gpu_small_depths(gpu):
    d = domain("coast")
    sd = np.zeros(d.shape2, dtype=np.int32)
    sd[2:5, 3:6] = 1
    P0 = d.tracer(1, 10.0, 20.0, seed=3)
    Po = P0.copy()
    assert O.step(d, Po, O.params(DTProp=30.0), SmallDepths=sd) == 0
    ad = advdiff.AdvectionDiffusion(d)
    ad.set_hydro(SmallDepths=sd)
    Pg = P0.copy()
    ad.step(Pg, advdiff.params(DTProp=30.0))
    ad.kill()
    assert np.array_equal(Pg, Po)


def test_gpu_cfg1_100_steps_device_resident(gpu):
    """Config 1 at full size: 100 steps device-resident (ping-pong) vs 100 oracle steps."""
    import torch
    w = configs.cfg1()
    d = synth.generate(w.spec)
    P0 = d.tracer(*w.tracers[0], seed=11)
    pd = w.params()
    Po = P0.copy()
    work = O.Work(d)
    for _ in range(w.steps):
        assert O.step(d, Po, O.params(**pd), work=work) == 0
    ad = advdiff.AdvectionDiffusion(d)
    ad.set_hydro()
    a = torch.from_numpy(P0).cuda()
    b = torch.empty_like(a)
    p = advdiff.params(**pd)
    torch.cuda.synchronize()
    for _ in range(w.steps):
        ad.step_device(a, b, p)
        a, b = b, a
    ad.sync()
    Pg = a.cpu().numpy()
    ad.kill()
    wp = d.water_mask()
    rel_l2 = np.linalg.norm(Pg[wp] - Po[wp]) / np.linalg.norm(Po[wp])
    assert rel_l2 <= 1e-12
    assert np.array_equal(Pg, Po)
    m0, m1 = O.mass(d, P0), O.mass(d, Pg)
    assert abs(m1 - m0) / m0 < 1e-12


def test_gpu_cfg2_full_size_one_step(gpu):
    """Config 2 grid (512x512x40, P2_TVD SuperBee) at full size, both tracers."""
    w = configs.cfg2()
    d = synth.generate(w.spec)
    ad = advdiff.AdvectionDiffusion(d)
    ad.set_hydro()
    for t, (kind, a_, b_) in enumerate(w.tracers):
        P0 = d.tracer(kind, a_, b_, seed=100 + t)
        Po = P0.copy()
        assert O.step(d, Po, O.params(**w.params())) == 0
        Pg = P0.copy()
        ad.step(Pg, advdiff.params(**w.params()))
        _compare(d, Pg, Po)
    ad.kill()


def test_gpu_thomasz_matches_oracle(gpu):
    rng = np.random.default_rng(1)
    ni, nj, nk = 37, 29, 23
    sh = (nk + 2, nj + 2, ni + 2)
    D = rng.uniform(-1, 0, sh); F = rng.uniform(-1, 0, sh)
    E = 2.5 + rng.uniform(0, 1, sh); TI = rng.normal(size=sh)
    WP = (rng.random(sh) < 0.8).astype(np.int32)
    R1 = rng.normal(size=sh); R2 = R1.copy()
    assert O.thomasz(D, E, F, TI, R1, WP) == 0
    advdiff.thomasz(D, E, F, TI, R2, WP)
    assert np.array_equal(R1, R2)


def test_gpu_zero_pivot_reported(gpu):
    sh = (5, 3, 3)
    D = np.zeros(sh); E = np.ones(sh); F = np.zeros(sh); TI = np.ones(sh)
    D[2, 1, 1] = 1.0; E[2, 1, 1] = 0.0
    WP = np.ones(sh, dtype=np.int32)
    RES = np.zeros(sh)
    with pytest.raises(advdiff.N.MohidAdError) as ei:
        advdiff.thomasz(D, E, F, TI, RES, WP)
    assert ei.value.code == 6


@pytest.mark.parametrize("bad,code", [
    (dict(ImpExp_DifH=1.0), 3), (dict(ImpExp_AdvXX=1.0, ImpExp_AdvYY=1.0), 3),
    (dict(AdvMethodV=2, Upwind2V=1), 3), (dict(AdvMethodH=4, Upwind2H=0), 3),
    (dict(AdvMethodH=9), 3), (dict(ImpExp_AdvV=0.5), 3), (dict(Docycle_method=3), 3),
    (dict(ImpExp_AdvXX=0.5), 3), (dict(NoAdvFlux=1), 9),
    (dict(AdvectionNudging=1, AdvectionNudgingCells=2, ImpExp_AdvXX=1.0), 4),
    (dict(AdvectionNudging=1, AdvectionNudgingCells=2, Vertical1D=1), 4),
])
def test_gpu_rejects_options_like_oracle(gpu, bad, code):
    d = domain("coast")
    P = d.tracer(4, 1.0, 0.0, seed=1)
    P0 = P.copy()
    assert O.step(d, P.copy(), O.params(DTProp=30.0, **bad)) == code
    ad = advdiff.AdvectionDiffusion(d)
    ad.set_hydro()
    with pytest.raises(advdiff.N.MohidAdError) as ei:
        ad.step(P, advdiff.params(DTProp=30.0, **bad))
    ad.kill()
    assert ei.value.code == code
    assert np.array_equal(P, P0)


def test_gpu_rejects_lower_edge_face(gpu):
    d = domain("coast")
    d.arrays["ComputeFacesU3D"][2, 1, 3] = 1
    ad = advdiff.AdvectionDiffusion(d)
    with pytest.raises(advdiff.N.MohidAdError) as ei:
        ad.set_hydro()
    assert ei.value.code == 1
    ad.kill()


def test_gpu_unknown_id_and_bad_bounds(gpu):
    lib = advdiff.N.ad_lib()
    st = C.c_int(0)
    bogus = C.c_int(987654)
    assert lib.mohid_ad_sync(C.byref(bogus), C.byref(st)) == 2 and st.value == 2
    size = advdiff.N.T_Size3D(0, 5, 0, 5, 0, 5)
    work = advdiff.N.T_Size3D(1, 4, 1, 3, 1, 4)      # JUB inconsistent with Size
    z = np.zeros((6, 6)); zi = np.zeros((6, 6), dtype=np.int32)
    idv = C.c_int(0)
    rc = lib.mohid_ad_init(C.byref(idv), C.byref(size), C.byref(work), advdiff.N.ptr(z),
                           advdiff.N.ptr(z), advdiff.N.ptr(z), advdiff.N.ptr(z),
                           advdiff.N.iptr(zi), advdiff.N.iptr(zi), C.byref(st))
    assert rc == 1


@pytest.mark.parametrize("grid", ["open", "nsopen", "allopen", "narrow", "flat", "wide"])
@pytest.mark.parametrize("opt", ["upwind1", "tvd_minmod", "implicit_xx", "theta_difv"])
def test_gpu_orlanski(gpu, grid, opt):
    # Orlanski open boundaries (AD:5496-5569, FN:4129-4490) over four steps:
    # the field with its radiated exterior values and PropOld, through the host
    # and the device entry points, bit for bit against the oracle
    import torch
    from tests.test_oracle_crosscheck import _orlanski_grids
    if grid == "wide":
        d = synth.generate(synth.GenSpec(ni=61, nj=47, nk=7, land_frac=0.1, land_kind=1, seed=13, open_sides=15,
                                         bathy_kind=1, vol_var=0.01, dt=30.0))
    else:
        d = _orlanski_grids()[grid]
    P0 = d.tracer(3, 1.0, 0.5, seed=1)
    R = d.reference(2.0, 0.3, seed=2)
    pd = dict(DTProp=30.0, BoundaryCondition=6, **OPTIONS[opt])
    Po, oo = P0.copy(), np.zeros_like(P0)
    olds = []
    for _ in range(4):
        assert O.step(d, Po, O.params(**pd), ReferenceProp=R, PropOld=oo) == 0
        olds.append(oo.copy())
    ad = advdiff.AdvectionDiffusion(d)
    ad.set_hydro()
    Pg, og = P0.copy(), np.zeros_like(P0)
    ad.set_prop_old(og)
    for q in range(4):
        ad.step(Pg, advdiff.params(**pd), R)
        assert np.array_equal(og, olds[q])
    assert np.array_equal(Pg, Po)
    a = torch.from_numpy(P0.copy()).cuda()
    b = torch.empty_like(a)
    od = torch.zeros_like(a)
    ad.set_prop_old(od, device=True)
    Rd = torch.from_numpy(R).cuda()
    for _ in range(4):
        ad.step_device(a, b, advdiff.params(**pd), Rd)
        a, b = b, a
    ad.sync()
    ad.set_prop_old(None)
    ad.kill()
    assert np.array_equal(a.cpu().numpy(), Po)
    assert np.array_equal(od.cpu().numpy(), olds[-1])


def test_gpu_orlanski_rejects_interior_boundary_points(gpu):
    # a boundary point off the work box's edges: the reference stops, the
    # drop-in returns MOHID_AD_ERR_OPTION like the oracle
    from tests.test_oracle_crosscheck import _orlanski_grids
    d = _orlanski_grids()["allopen"]
    bp = d.arrays["BoundaryPoints2D"].copy()
    bp[3, 4] = 1
    d.arrays["BoundaryPoints2D"] = bp
    P = d.tracer(3, 1.0, 0.5, seed=1)
    R = d.reference(2.0, 0.3, seed=2)
    pd = dict(DTProp=30.0, BoundaryCondition=6)
    assert O.step(d, P.copy(), O.params(**pd), ReferenceProp=R) == 3
    ad = advdiff.AdvectionDiffusion(d)
    ad.set_hydro()
    with pytest.raises(advdiff.N.MohidAdError) as ei:
        ad.step(P.copy(), advdiff.params(**pd), R)
    assert ei.value.code == 3
    Q = P.copy()                                     # the instance stays usable
    ad.step(Q, advdiff.params(**dict(pd, BoundaryCondition=1)), R)
    ad.kill()


@pytest.mark.parametrize("grid", ["coast", "zlevel", "open", "layer1", "nsopen"])
@pytest.mark.parametrize("opt", ["upwind1", "tvd_superbee", "explicit_v_tvd", "docycle2", "theta_difv", "xzflow"])
@pytest.mark.parametrize("nc", [1, 3])
def test_gpu_nudging(gpu, grid, opt, nc):
    # AdvectionNudging (AD:1989-2068): the advective terms gathered apart and
    # scaled by the edge factor, with the cell fluxes; bit for bit
    d = domain(grid)
    P0 = d.tracer(3, 1.0, 0.5, seed=1)
    R = d.reference(2.0, 0.3, seed=2) if d.spec.open_sides else None
    pd = dict(DTProp=30.0, AdvectionNudging=1, AdvectionNudgingCells=nc, CellFluxes=1, **OPTIONS[opt])
    Po = P0.copy()
    work = O.Work(d)
    assert O.step(d, Po, O.params(**pd), ReferenceProp=R, work=work) == 0
    fo = O.cell_fluxes(d, work)
    ad = advdiff.AdvectionDiffusion(d)
    ad.set_hydro()
    Pg = P0.copy()
    ad.step(Pg, advdiff.params(**pd), R)
    fg = ad.cell_fluxes()
    ad.kill()
    assert np.array_equal(Pg, Po)
    for n in O.FLUX_NAMES:
        assert np.array_equal(fg[n], fo[n]), n


def test_gpu_nudging_many_steps(gpu):
    # a larger open grid, several steps, host and device entry points
    import torch
    d = synth.generate(synth.GenSpec(ni=61, nj=47, nk=7, land_frac=0.1, land_kind=1, seed=13, open_sides=15,
                                     bathy_kind=1, dt=30.0))
    P0 = d.tracer(3, 1.0, 0.5, seed=1)
    R = d.reference(2.0, 0.3, seed=2)
    pd = dict(DTProp=30.0, AdvectionNudging=1, AdvectionNudgingCells=5, **OPTIONS["tvd_superbee"])
    Po = P0.copy()
    for _ in range(4):
        assert O.step(d, Po, O.params(**pd), ReferenceProp=R) == 0
    ad = advdiff.AdvectionDiffusion(d)
    ad.set_hydro()
    Pg = P0.copy()
    for _ in range(4):
        ad.step(Pg, advdiff.params(**pd), R)
    assert np.array_equal(Pg, Po)
    a = torch.from_numpy(P0.copy()).cuda()
    b = torch.empty_like(a)
    Rd = torch.from_numpy(R).cuda()
    for _ in range(4):
        ad.step_device(a, b, advdiff.params(**pd), Rd)
        a, b = b, a
    ad.sync()
    ad.kill()
    assert np.array_equal(a.cpu().numpy(), Po)
