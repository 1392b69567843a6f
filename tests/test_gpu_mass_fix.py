"""Mass fixer of the batched FP32 form.

With a step that maps constants onto themselves and static volumes, the
reference's mass budget (sum of VolumeZ * PROP over water cells) closes to FP64
round-off: constant on closed domains, changed by exactly the boundary flux
with MassConservation open boundaries.  The FP32 form alone drifts by ~1e-7
over hundreds of steps; with the fixer the relative defect (mass now - mass
loaded - boundary flux since, over the loaded mass) stays <= 1e-12, and the
field still agrees with the FP64 oracle to the form's tolerance (relative L2
over water cells <= 1e-5).
"""
import numpy as np
import pytest

from mohid_gb300 import advdiff, batched, configs, synth
from oracle import oracle as O
from tests.cases import domain

pytestmark = pytest.mark.gpu
DEFECT = 1e-12


def _run(d, tracers, pd, steps, fix=True, graph=True, refs=None, fluxes=None):
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
    if fluxes is not None:
        fluxes.extend(b.boundary_flux(t) for t in range(len(tracers)))
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


@pytest.mark.parametrize("calls", [[1] * 12, [5, 7], [12], [4, 1, 1, 6]])
def test_mass_fix_once_per_call(gpu, calls):
    """On closed domains the fixer runs after the last step of each step call;
    however the steps are split into calls, the mass ends at its target and the
    fields agree to FP64 round-off of the tracer's constant."""
    d = domain("zlevel")
    tr = [d.tracer(3, 2.0, 0.5, seed=2), d.tracer(1, 5.0, 20.0, seed=3)]
    pd = advdiff.params(DTProp=30.0, AdvMethodH=4, TVDLimitationH=4, Upwind2H=1)
    ad = advdiff.AdvectionDiffusion(d)
    ad.set_hydro()
    b = batched.Batch(ad, 2)
    for t, P in enumerate(tr):
        b.set_tracer(t, P)
    for n in calls:
        b.step(pd, nsteps=n, graph=n > 1)
    b.sync()
    got = [b.get_tracer(t) for t in range(2)]
    for t, P in enumerate(tr):
        m0 = O.mass(d, P)
        assert abs(b.mass(t) - m0) <= DEFECT * abs(m0)
        assert abs(O.mass(d, got[t]) - m0) <= DEFECT * abs(m0)
    assert b.schedule()["per_call"] == 1
    b.destroy()
    ad.kill()
    one, _ = _run(d, tr, dict(DTProp=30.0, AdvMethodH=4, TVDLimitationH=4, Upwind2H=1), 12)
    wp = d.water_mask()
    for g, o in zip(got, one):
        assert np.max(np.abs(g[wp] - o[wp]) / np.abs(o[wp])) <= 1e-14


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
    """Moving volumes, with and without open boundaries: the fixer does not run
    (results equal with it on or off)."""
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


OPEN_SPECS = {
    "open_ring": dict(ni=40, nj=24, nk=6, land_frac=0.0, seed=7, open_sides=12, bathy_kind=1, dt=30.0),
    "open_coast": dict(ni=45, nj=37, nk=8, land_frac=0.15, land_kind=1, seed=9, open_sides=3, bathy_kind=1,
                       dt=30.0),
}


@pytest.mark.parametrize("grid", list(OPEN_SPECS))
@pytest.mark.parametrize("decay", [0.0, 600.0])
def test_mass_fix_open_boundaries(gpu, grid, decay):
    """MassConservation open boundaries, static volumes: mass now = mass loaded
    + boundary flux to <= 1e-12, the flux agrees with the oracle's own mass
    change, and the field with the oracle's."""
    from tests.cases import boundary_flux
    d = synth.generate(synth.GenSpec(**OPEN_SPECS[grid]))
    tr = [d.tracer(3, 1.0, 0.6, seed=11), d.tracer(1, 5.0, 20.0, seed=12), d.tracer(2, 30.0, 36.0, seed=13)]
    refs = [d.reference(2.5, 0.3, seed=21), d.reference(12.0, 0.2, seed=22), d.reference(33.0, 0.05, seed=23)]
    pd = dict(DTProp=30.0, AdvMethodH=4, TVDLimitationH=1, Upwind2H=1, BoundaryCondition=1, DecayTime=decay)
    steps = 120
    fl = []
    got, masses = _run(d, tr, pd, steps, fix=True, refs=refs, fluxes=fl)
    fl_off = []
    off, masses_off = _run(d, tr, pd, steps, fix=False, refs=refs, fluxes=fl_off)
    work = O.Work(d)
    for t, P in enumerate(tr):
        m0 = O.mass(d, P)
        assert abs(masses[t] - m0 - fl[t]) <= DEFECT * abs(m0)
        assert abs(O.mass(d, got[t]) - m0 - fl[t]) <= DEFECT * abs(m0)
        assert np.isnan(fl_off[t])                  # not followed without the fixer
        Q, moved = P.copy(), 0.0
        for _ in range(steps):
            Q0 = Q.copy()
            assert O.step(d, Q, O.params(**pd), ReferenceProp=refs[t], work=work) == 0
            moved += boundary_flux(d, Q0, Q, refs[t], 30.0, decay, gross=True)[1]
        assert moved > 1e-6 * abs(m0)               # the boundaries move mass
        # the flux the fixer followed is the oracle's mass change, to the FP32
        # field's accuracy on the boundary cells (relative to the mass moved in
        # and out, of which the net flux is a small difference)
        assert abs(fl[t] - (O.mass(d, Q) - m0)) <= 1e-5 * moved
        assert _rel_l2(d, got[t], Q) <= 1e-5
        assert _rel_l2(d, off[t], Q) <= 1e-5


def test_mass_fix_open_graph_equals_direct(gpu):
    d = synth.generate(synth.GenSpec(**OPEN_SPECS["open_coast"]))
    tr = [d.tracer(3, 1.0, 0.6, seed=1), d.tracer(1, 5.0, 20.0, seed=2)]
    refs = [d.reference(2.5, 0.3, seed=3), d.reference(12.0, 0.2, seed=4)]
    pd = dict(DTProp=30.0, BoundaryCondition=1, DecayTime=0.0)
    f1, f2 = [], []
    g1, m1 = _run(d, tr, pd, 20, graph=True, refs=refs, fluxes=f1)
    g2, m2 = _run(d, tr, pd, 20, graph=False, refs=refs, fluxes=f2)
    for a, b in zip(g1, g2):
        assert np.array_equal(a, b)
    assert m1 == m2 and f1 == f2


def test_mass_fix_open_stops_after_a_step_without_it(gpu):
    """With open boundaries a step made without the fixer leaves the targets
    behind: the fixer does not resume for the tracers loaded before."""
    d = synth.generate(synth.GenSpec(**OPEN_SPECS["open_ring"]))
    P, R = d.tracer(3, 1.0, 0.6, seed=1), d.reference(2.5, 0.3, seed=2)
    pd = advdiff.params(DTProp=30.0, BoundaryCondition=1, DecayTime=0.0)
    ad = advdiff.AdvectionDiffusion(d)
    ad.set_hydro()
    b = batched.Batch(ad, 1)
    b.set_tracer(0, P)
    b.set_reference(0, R)
    b.step(pd, nsteps=4)
    assert np.isfinite(b.boundary_flux(0))
    b.set_mass_fix(False)
    b.step(pd, nsteps=2)
    b.set_mass_fix(True)
    b.step(pd, nsteps=2)
    b.sync()
    assert np.isnan(b.boundary_flux(0))
    assert np.all(np.isfinite(b.get_tracer(0)[d.water_mask()]))
    b.set_tracer(0, P)                              # a reload sets a new target
    b.set_reference(0, R)
    b.step(pd, nsteps=3)
    b.sync()
    assert np.isfinite(b.boundary_flux(0))
    m0 = O.mass(d, P)
    assert abs(b.mass(0) - m0 - b.boundary_flux(0)) <= DEFECT * abs(m0)
    b.destroy()
    ad.kill()


def test_mass_fix_open_ensemble(gpu):
    """An open member of an ensemble follows its boundary flux too, to the
    same bits as when stepped alone."""
    specs = [dict(OPEN_SPECS["open_coast"]), dict(ni=33, nj=20, nk=5, land_frac=0.1, land_kind=1, seed=41, dt=30.0)]
    pd = dict(DTProp=30.0, AdvMethodH=4, TVDLimitationH=4, Upwind2H=1, BoundaryCondition=1, DecayTime=0.0)
    objs, loads = [], []
    for q, sp in enumerate(specs):
        d = synth.generate(synth.GenSpec(**sp))
        ad = advdiff.AdvectionDiffusion(d)
        ad.set_hydro()
        b = batched.Batch(ad, 2)
        tr = [d.tracer(3, 1.0 + t, 0.6, seed=t) for t in range(2)]
        refs = [d.reference(2.0 + t, 0.3, seed=10 + t) for t in range(2)] if q == 0 else None
        for t, P in enumerate(tr):
            b.set_tracer(t, P)
            if refs:
                b.set_reference(t, refs[t])
        objs.append((d, ad, b, tr, refs))
        loads.append([O.mass(d, P) for P in tr])
    ens = batched.Ensemble([b for _, _, b, _, _ in objs])
    ens.step([advdiff.params(**pd)] * len(objs), nsteps=30, graph=True)
    ens.sync()
    d, _, b, tr, refs = objs[0]
    alone_f = []
    alone, _ = _run(d, tr, pd, 30, refs=refs, fluxes=alone_f)
    for t in range(2):
        m0 = loads[0][t]
        assert abs(b.mass(t) - m0 - b.boundary_flux(t)) <= DEFECT * abs(m0)
        assert b.boundary_flux(t) == alone_f[t]
        assert np.array_equal(b.get_tracer(t), alone[t])
    for t in range(2):                              # the closed member
        assert abs(objs[1][2].mass(t) - loads[1][t]) <= DEFECT * abs(loads[1][t])
        assert objs[1][2].boundary_flux(t) == 0.0
    ens.destroy()
    for _, ad, b, _, _ in objs:
        b.destroy()
        ad.kill()
