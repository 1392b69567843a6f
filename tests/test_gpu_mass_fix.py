"""Mass fixer of the batched FP32 form.

With closed boundaries, a step that maps constants onto themselves and static
volumes, the reference conserves every tracer's mass (sum of VolumeZ * PROP
over water cells) to FP64 round-off.  The FP32 form alone drifts by ~1e-7 over
hundreds of steps; with the fixer the relative defect against the FP64 mass of
the loaded field stays <= 1e-12, and the field still agrees with the FP64
oracle to the form's tolerance (relative L2 over water cells <= 1e-5).
"""
import numpy as np
import pytest

from mohid_gb300 import advdiff, batched, configs, synth
from oracle import oracle as O
from tests.cases import domain

pytestmark = pytest.mark.gpu
DEFECT = 1e-12


def _run(d, tracers, pd, steps, fix=True, graph=True, refs=None):
    ad = advdiff.AdvectionDiffusion(d)
    ad.set_hydro()
    b = batched.Batch(ad, len(tracers))
    b.set_mass_fix(fix)
    for t, P in enumerate(tracers):
        b.set_tracer(t, P)
        if refs is not None:
            b.set_reference(t, refs[t])
    b.step(advdiff.params(**pd), nsteps=steps, graph=graph)
    b.sync()
    got = [b.get_tracer(t) for t in range(len(tracers))]
    masses = [b.mass(t) for t in range(len(tracers))]
    b.destroy()
    ad.kill()
    return got, masses


def _rel_l2(d, a, b):
    wp = d.water_mask()
    return float(np.linalg.norm(a[wp] - b[wp]) / np.linalg.norm(b[wp]))


def test_mass_fix_cfg2_grid_300_steps(gpu):
    """Config 2 options on a 128x128x40 cut: defect <= 1e-12 with the fixer,
    FP32 drift without it, both within the oracle tolerance."""
    w = configs.cfg2().scaled(ni=128, nj=128)
    d = synth.generate(w.spec)
    tr = [d.tracer(k, a, b, seed=100 + t) for t, (k, a, b) in enumerate(w.tracers)]
    m0 = [O.mass(d, P) for P in tr]
    got, masses = _run(d, tr, w.params(), 300, fix=True)
    off, masses_off = _run(d, tr, w.params(), 300, fix=False)
    work = O.Work(d)
    for t, P in enumerate(tr):
        # the budget the library reports and the oracle's FP64 sum of the returned field
        assert abs(masses[t] - m0[t]) <= DEFECT * abs(m0[t])
        assert abs(O.mass(d, got[t]) - m0[t]) <= DEFECT * abs(m0[t])
        assert abs(masses_off[t] - m0[t]) > DEFECT * abs(m0[t])       # the FP32 drift it removes
        Q = P.copy()
        for _ in range(300):
            assert O.step(d, Q, O.params(**w.params()), work=work) == 0
        assert _rel_l2(d, got[t], Q) <= 1e-5
        assert _rel_l2(d, off[t], Q) <= 1e-5


@pytest.mark.parametrize("grid", ["coast", "zlevel"])
def test_mass_fix_small_grids(gpu, grid):
    d = domain(grid)
    tr = [d.tracer(3, 2.0 + t, 0.5, seed=7 + t) for t in range(3)]
    pd = dict(DTProp=30.0, AdvMethodH=4, TVDLimitationH=4, Upwind2H=1)
    got, masses = _run(d, tr, pd, 50)
    for t, P in enumerate(tr):
        m0 = O.mass(d, P)
        assert abs(masses[t] - m0) <= DEFECT * abs(m0)
        assert abs(O.mass(d, got[t]) - m0) <= DEFECT * abs(m0)


def test_mass_fix_graph_equals_direct(gpu):
    d = domain("coast")
    tr = [d.tracer(3, 1.0, 0.5, seed=2), d.tracer(1, 5.0, 20.0, seed=3)]
    pd = dict(DTProp=30.0, AdvMethodH=4, TVDLimitationH=4, Upwind2H=1)
    g1, m1 = _run(d, tr, pd, 20, graph=True)
    g2, m2 = _run(d, tr, pd, 20, graph=False)
    for a, b in zip(g1, g2):
        assert np.array_equal(a, b)
    assert m1 == m2


def test_mass_fix_off_where_mass_is_not_conserved(gpu):
    """Open boundaries and moving volumes: the fixer does not run (results equal with it on or off)."""
    d = domain("open")                       # open boundaries, moving volumes
    tr = [d.tracer(3, 1.0, 0.5, seed=1), d.tracer(1, 5.0, 20.0, seed=4)]
    refs = [d.reference(2.0, 0.3, seed=2), d.reference(12.0, 0.2, seed=3)]
    pd = dict(DTProp=30.0, BoundaryCondition=1, DecayTime=0.0)
    a, _ = _run(d, tr, pd, 5, fix=True, refs=refs)
    b, _ = _run(d, tr, pd, 5, fix=False, refs=refs)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    # closed, but moving volumes
    dm = synth.generate(synth.GenSpec(ni=9, nj=8, nk=4, land_frac=0.1, land_kind=1, seed=5, vol_var=0.01,
                                      bathy_kind=1, dt=30.0))
    tr = [dm.tracer(3, 1.0, 0.5, seed=1)]
    a, _ = _run(dm, tr, dict(DTProp=30.0), 5, fix=True)
    b, _ = _run(dm, tr, dict(DTProp=30.0), 5, fix=False)
    assert np.array_equal(a[0], b[0])


def test_mass_fix_ensemble(gpu):
    """Members of an ensemble keep their masses too."""
    specs = [dict(ni=40, nj=30, nk=6, land_frac=0.1, land_kind=1, seed=31, dt=20.0),
             dict(ni=33, nj=65, nk=9, land_frac=0.25, land_kind=1, seed=33, dt=15.0, zlevel=True,
                  hmin=2.0, hmax=60.0, bathy_kind=2)]
    objs, pars, loads = [], [], []
    for sp in specs:
        d = synth.generate(synth.GenSpec(**sp))
        ad = advdiff.AdvectionDiffusion(d)
        ad.set_hydro()
        b = batched.Batch(ad, 2)
        tr = [d.tracer(3, 1.0 + t, 0.6, seed=t) for t in range(2)]
        for t, P in enumerate(tr):
            b.set_tracer(t, P)
        objs.append((d, ad, b))
        loads.append([O.mass(d, P) for P in tr])
        pars.append(advdiff.params(DTProp=sp["dt"], AdvMethodH=4, TVDLimitationH=4, Upwind2H=1))
    ens = batched.Ensemble([b for _, _, b in objs])
    ens.step(pars, nsteps=40, graph=True)
    ens.sync()
    for (d, ad, b), m0 in zip(objs, loads):
        for t in range(2):
            assert abs(b.mass(t) - m0[t]) <= DEFECT * abs(m0[t])
    ens.destroy()
    for _, ad, b in objs:
        b.destroy()
        ad.kill()
