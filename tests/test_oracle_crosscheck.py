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
