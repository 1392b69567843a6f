"""The C oracle against the independent pure-Python restatement, bit for bit."""
import numpy as np
import pytest

from oracle import oracle as O, ref_py
from tests.cases import SMALL, OPTIONS, domain


@pytest.mark.parametrize("grid", sorted(SMALL))
@pytest.mark.parametrize("opt", sorted(OPTIONS))
def test_c_oracle_equals_python_restatement(built, grid, opt):
    d = domain(grid)
    P0 = d.tracer(3, 1.0, 0.7, seed=9)
    pd = dict(O.DEFAULTS, DTProp=30.0, **OPTIONS[opt])
    Pc, Pp = P0.copy(), P0.copy()
    assert O.step(d, Pc, O.params(**pd)) == 0
    ref_py.step(d, Pp, pd)
    assert np.array_equal(Pc, Pp)


@pytest.mark.parametrize("grid", ["open", "nsopen"])
@pytest.mark.parametrize("bc,decay", [(1, 0.0), (1, 600.0), (2, 0.0), (2, 300.0), (5, 0.0), (4, 0.0), (7, 0.0),
                                      (8, 0.0)])
@pytest.mark.parametrize("opt", ["upwind1", "tvd_minmod", "implicit_xx", "implicit_yy_tvd"])
def test_open_boundaries_c_equals_python(built, grid, bc, decay, opt):
    d = domain(grid)
    P0 = d.tracer(3, 1.0, 0.5, seed=1)
    R = d.reference(2.0, 0.3, seed=2)
    pd = dict(O.DEFAULTS, DTProp=30.0, BoundaryCondition=bc, DecayTime=decay, **OPTIONS[opt])
    Pc, Pp = P0.copy(), P0.copy()
    assert O.step(d, Pc, O.params(**pd), ReferenceProp=R) == 0
    ref_py.step(d, Pp, pd, ReferenceProp=R)
    assert np.array_equal(Pc, Pp)


@pytest.mark.parametrize("grid", ["open", "nsopen"])
def test_null_gradient_without_reference_c_equals_python(built, grid):
    # ImposeNullGradient runs after the solve whether or not a reference is given (AD:1874-1876)
    d = domain(grid)
    P0 = d.tracer(3, 1.0, 0.5, seed=3)
    pd = dict(O.DEFAULTS, DTProp=30.0, BoundaryCondition=4, **OPTIONS["tvd_minmod"])
    Pc, Pp = P0.copy(), P0.copy()
    assert O.step(d, Pc, O.params(**pd)) == 0
    ref_py.step(d, Pp, pd)
    assert np.array_equal(Pc, Pp)
    Q = P0.copy()
    assert O.step(d, Q, O.params(**dict(pd, BoundaryCondition=1))) == 0
    assert not np.array_equal(Pc, Q)                 # the boundary columns changed


def test_small_depths_c_equals_python(built):
    d = domain("coast")
    sd = np.zeros(d.shape2, dtype=np.int32)
    sd[2:5, 3:6] = 1
    P0 = d.tracer(1, 10.0, 20.0, seed=3)
    pd = dict(O.DEFAULTS, DTProp=30.0)
    Pc, Pp = P0.copy(), P0.copy()
    assert O.step(d, Pc, O.params(**pd), SmallDepths=sd) == 0
    ref_py.step(d, Pp, pd, SmallDepths=sd)
    assert np.array_equal(Pc, Pp)


@pytest.mark.parametrize("grid", ["coast", "zlevel", "open", "layer1"])
@pytest.mark.parametrize("opt", ["upwind1", "tvd_superbee", "explicit_v_tvd", "theta_difv", "implicit_xx",
                                 "implicit_yy_tvd", "docycle2", "tvd_vertical", "vertical1d", "xzflow", "nulldif"])
def test_cell_fluxes_c_equals_python(built, grid, opt):
    # CellFluxes (AD:1458-1468, 1882-1916, 3356-3954): the six face-flux arrays
    d = domain(grid)
    P0 = d.tracer(3, 1.0, 0.5, seed=2)
    R = d.reference(2.0, 0.3, seed=3) if d.spec.open_sides else None
    pd = dict(O.DEFAULTS, DTProp=30.0, CellFluxes=1, **OPTIONS[opt])
    Pc, Pp = P0.copy(), P0.copy()
    work = O.Work(d)
    assert O.step(d, Pc, O.params(**pd), ReferenceProp=R, work=work) == 0
    fc = O.cell_fluxes(d, work)
    fp = {}
    ref_py.step(d, Pp, pd, ReferenceProp=R, fluxes=fp)
    assert np.array_equal(Pc, Pp)
    for n in O.FLUX_NAMES:
        assert np.array_equal(fc[n], fp[n]), n


@pytest.mark.parametrize("grid", ["coast", "zlevel", "open"])
@pytest.mark.parametrize("flags", [dict(NoAdvFlux=1), dict(NoDifFlux=1), dict(NoAdvFlux=1, NoDifFlux=1)])
@pytest.mark.parametrize("opt", ["upwind1", "tvd_superbee", "explicit_v_tvd", "theta_difv"])
def test_noflux_c_equals_python(built, grid, flags, opt):
    from tests.cases import noflux_masks
    d = domain(grid)
    P0 = d.tracer(3, 1.0, 0.5, seed=4)
    R = d.reference(2.0, 0.3, seed=3) if d.spec.open_sides else None
    nf = noflux_masks(d, seed=5)
    pd = dict(O.DEFAULTS, DTProp=30.0, CellFluxes=1, **flags, **OPTIONS[opt])
    Pc, Pp = P0.copy(), P0.copy()
    work = O.Work(d)
    assert O.step(d, Pc, O.params(**pd), ReferenceProp=R, work=work, NoFlux=nf) == 0
    fp = {}
    ref_py.step(d, Pp, pd, ReferenceProp=R, fluxes=fp, NoFlux=nf)
    assert np.array_equal(Pc, Pp)
    fc = O.cell_fluxes(d, work)
    for n in O.FLUX_NAMES:
        assert np.array_equal(fc[n], fp[n]), n
    Q = P0.copy()                                   # the masks change the step
    assert O.step(d, Q, O.params(**dict(pd, NoAdvFlux=0, NoDifFlux=0)), ReferenceProp=R) == 0
    assert not np.array_equal(Q, Pc)


@pytest.mark.parametrize("grid", ["coast", "zlevel", "open", "layer1"])
@pytest.mark.parametrize("opt", ["upwind1", "tvd_superbee", "theta_difv", "implicit_xx"])
@pytest.mark.parametrize("seed", [0, 1])
def test_discharges_c_equals_python(built, grid, opt, seed):
    from tests.cases import discharges
    d = domain(grid)
    P0 = d.tracer(3, 1.0, 0.5, seed=2)
    R = d.reference(2.0, 0.3, seed=3) if d.spec.open_sides else None
    ds = discharges(d, seed=seed)
    pd = dict(O.DEFAULTS, DTProp=30.0, CellFluxes=1, **OPTIONS[opt])
    Pc, Pp = P0.copy(), P0.copy()
    assert O.step(d, Pc, O.params(**pd), ReferenceProp=R, Disch=ds) == 0
    ref_py.step(d, Pp, pd, ReferenceProp=R, Disch=ds)
    assert np.array_equal(Pc, Pp)


def _orlanski_grids():
    from mohid_gb300 import synth
    g = {n: domain(n) for n in ("open", "nsopen")}
    # all four sides open (every edge, every corner), and a grid 3 cells wide in i
    g["allopen"] = synth.generate(synth.GenSpec(ni=8, nj=7, nk=3, land_frac=0.1, land_kind=1, seed=11,
                                                open_sides=15, vol_var=0.01, bathy_kind=1, dt=30.0))
    g["narrow"] = synth.generate(synth.GenSpec(ni=3, nj=9, nk=3, land_frac=0.0, seed=12, open_sides=15,
                                               bathy_kind=1, dt=30.0))
    # 3 cells in j: the top row's radiation reads the corner's exterior point
    # (IUB-1, JLB) after the corner wrote it
    g["flat"] = synth.generate(synth.GenSpec(ni=9, nj=3, nk=3, land_frac=0.0, seed=14, open_sides=15,
                                             bathy_kind=1, dt=30.0))
    return g


@pytest.mark.parametrize("grid", ["open", "nsopen", "allopen", "narrow", "flat"])
@pytest.mark.parametrize("opt", ["upwind1", "tvd_minmod", "implicit_xx", "theta_difv"])
def test_orlanski_c_equals_python(built, grid, opt):
    # OpenBoundaryCondition with OrlanskiCelerity2D (AD:5496-5569, FN:4129-4490):
    # the field, its radiated exterior values and PropOld, bit for bit
    d = _orlanski_grids()[grid]
    P0 = d.tracer(3, 1.0, 0.5, seed=1)
    R = d.reference(2.0, 0.3, seed=2)
    pd = dict(O.DEFAULTS, DTProp=30.0, BoundaryCondition=6, **OPTIONS[opt])
    Pc, Pp = P0.copy(), P0.copy()
    oc, op = np.full_like(P0, np.nan), np.full_like(P0, np.nan)
    assert O.step(d, Pc, O.params(**pd), ReferenceProp=R, PropOld=oc) == 0
    ref_py.step(d, Pp, pd, ReferenceProp=R, PropOld=op)
    assert np.array_equal(Pc, Pp)
    assert np.array_equal(oc, op)
    if opt != "implicit_xx":                        # PropOld = PROP as the step got it
        assert np.array_equal(oc, P0)
    Q = P0.copy()                                   # radiation changes the result
    assert O.step(d, Q, O.params(**dict(pd, BoundaryCondition=1)), ReferenceProp=R) == 0
    assert not np.array_equal(Q, Pc)
    # the exterior points of the open boundary cells carry the radiated values
    halo = np.ones(d.shape3, dtype=bool)
    halo[:, 1:-1, 1:-1] = False
    assert (Pc[halo] != P0[halo]).any()


def test_orlanski_keeps_constants(built):
    # a constant field with a constant reference stays constant where
    # continuity holds (tv = svx = 0, the radiated value is the constant)
    d = _orlanski_grids()["allopen"]
    P0 = np.full(d.shape3, 7.5)
    R = np.full(d.shape3, 7.5)
    pd = dict(O.DEFAULTS, DTProp=30.0, BoundaryCondition=6, **OPTIONS["tvd_superbee"])
    P = P0.copy()
    assert O.step(d, P, O.params(**pd), ReferenceProp=R) == 0
    wp = d.water_mask()
    assert np.max(np.abs(P[wp] - 7.5)) <= 1e-12 * 7.5


def test_orlanski_rejects_interior_boundary_points(built):
    # a boundary point off the work box's edges has no normal: the reference
    # stops ('Orlanski Advection 2'); the restatements refuse it
    d = _orlanski_grids()["allopen"]
    bp = d.arrays["BoundaryPoints2D"].copy()
    bp[3, 4] = 1
    d.arrays["BoundaryPoints2D"] = bp
    P = d.tracer(3, 1.0, 0.5, seed=1)
    R = d.reference(2.0, 0.3, seed=2)
    pd = dict(O.DEFAULTS, DTProp=30.0, BoundaryCondition=6)
    assert O.step(d, P.copy(), O.params(**pd), ReferenceProp=R) == 3   # MOHID_AD_ERR_OPTION
    with pytest.raises(ValueError):
        ref_py.step(d, P.copy(), pd, ReferenceProp=R)


@pytest.mark.parametrize("grid", sorted(SMALL))
@pytest.mark.parametrize("opt", ["upwind1", "tvd_superbee", "explicit_v_tvd", "docycle2", "theta_difv", "xzflow",
                                 "central", "background"])
@pytest.mark.parametrize("nc", [1, 2, 3, 50])
def test_nudging_c_equals_python(built, grid, opt, nc):
    # AdvectionNudging (AD:1989-2068) with the _Nudge advection routines
    # (AD:4586-4733, 4957-5118, 3211-3350), open boundaries where the grid has them
    d = domain(grid)
    P0 = d.tracer(3, 1.0, 0.5, seed=1)
    R = d.reference(2.0, 0.3, seed=2) if d.spec.open_sides else None
    pd = dict(O.DEFAULTS, DTProp=30.0, AdvectionNudging=1, AdvectionNudgingCells=nc, CellFluxes=1, **OPTIONS[opt])
    Pc, Pp = P0.copy(), P0.copy()
    work = O.Work(d)
    assert O.step(d, Pc, O.params(**pd), ReferenceProp=R, work=work) == 0
    fp = {}
    ref_py.step(d, Pp, pd, ReferenceProp=R, fluxes=fp)
    assert np.array_equal(Pc, Pp)
    fc = O.cell_fluxes(d, work)
    for n in O.FLUX_NAMES:
        assert np.array_equal(fc[n], fp[n]), n


def _nudge_factor_serial(ni, nj, nc):
    """n(i, j) as AdvectionNudging's loop computes it on one thread: in / jn
    keep the value of the last cell that set them (AD:2012-2042)."""
    n = np.ones((nj + 2, ni + 2))
    in_ = jn_ = None
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
            if cell:
                assert in_ is not None and jn_ is not None      # never read before it is set
                n[j, i] = float(min(in_, jn_)) / nc
    return n


@pytest.mark.parametrize("ni,nj", [(1, 1), (3, 9), (9, 3), (8, 7), (20, 13)])
@pytest.mark.parametrize("nc", [-1, 0, 1, 2, 3, 5, 12])
def test_nudging_factor_closed_form(ni, nj, nc):
    # on one thread the distance not set at a cell is always nCells, so
    # n = min(in*, jn*) / nCells with in* = i near the low edge, IUB - i + 1
    # near the high edge, else nCells (the form the GPU kernel evaluates)
    ref = _nudge_factor_serial(ni, nj, nc)
    for j in range(1, nj + 1):
        for i in range(1, ni + 1):
            if nc < 1:
                cf = 1.0
            else:
                a = i if i < nc + 1 else (ni - i + 1 if i > ni - nc else nc)
                b = j if j < nc + 1 else (nj - j + 1 if j > nj - nc else nc)
                cf = float(min(a, b)) / nc
            assert cf == ref[j, i], (i, j)


@pytest.mark.parametrize("grid", ["coast", "zlevel", "open"])
def test_nudging_properties(built, grid):
    d = domain(grid)
    P0 = d.tracer(3, 1.0, 0.5, seed=1)
    R = d.reference(2.0, 0.3, seed=2) if d.spec.open_sides else None
    base = dict(O.DEFAULTS, DTProp=30.0, **OPTIONS["tvd_superbee"])
    run = lambda **kw: (lambda P: (O.step(d, P, O.params(**dict(base, **kw)), ReferenceProp=R), P)[1])(P0.copy())
    plain = run()
    # no nudging cells: n = 1 everywhere, the regular step up to the order of the sums
    for nc in (0, -2):
        Q = run(AdvectionNudging=1, AdvectionNudgingCells=nc)
        wp = d.water_mask()
        assert np.max(np.abs(Q[wp] - plain[wp]) / np.maximum(np.abs(plain[wp]), 1e-30)) <= 1e-14
    # the _Nudge vertical advection runs by layers whatever Docycle_method says
    assert np.array_equal(run(AdvectionNudging=1, AdvectionNudgingCells=2, Docycle_method=1),
                          run(AdvectionNudging=1, AdvectionNudgingCells=2, Docycle_method=2))
    # nudging scales advection down near the edges: the step differs there only
    Q = run(AdvectionNudging=1, AdvectionNudgingCells=2)
    diff = np.abs(Q - plain) > 1e-12 * np.maximum(np.abs(plain), 1.0)
    assert diff.any()
    assert not diff[:, 4:-4, 4:-4].any() if min(d.ni, d.nj) > 8 else True
