"""Launch schedules of the batched form and the autotuner.

The schedules (one CTA per tile, or a persistent grid over the tiles holding
water with the deepest first; 10, 8, 4 or 2 tracers per launch; tiles of 8 or
4 rows) run the same per-column arithmetic and must give the same result bit
for bit (the mass fixer off: its per-tile sums follow the tile, so with it on
the constant may differ in the last bits); the autotuner must leave the
tracers as they were and report what it chose.
"""
import numpy as np
import pytest

from mohid_gb300 import advdiff, batched, synth
from oracle import oracle as O
from tests.cases import domain

pytestmark = pytest.mark.gpu

ZLEVEL = dict(ni=70, nj=45, nk=12, land_frac=0.35, land_kind=2, seed=41, zlevel=True, hmin=2.0, hmax=80.0,
              bathy_kind=2, dt=20.0)
PD = dict(DTProp=20.0, AdvMethodH=4, TVDLimitationH=4, Upwind2H=1)


def _run(d, tr, sched, split, steps=6, graph=True, rows=8, fix=True):
    ad = advdiff.AdvectionDiffusion(d)
    ad.set_hydro()
    b = batched.Batch(ad, len(tr))
    b.set_mass_fix(fix)
    for t, P in enumerate(tr):
        b.set_tracer(t, P)
    b.set_schedule(sched, split, rows)
    b.step(advdiff.params(**PD), nsteps=steps, graph=graph)
    b.sync()
    info = b.schedule()
    got = [b.get_tracer(t) for t in range(len(tr))]
    b.destroy()
    ad.kill()
    return got, info


@pytest.mark.parametrize("nt", [1, 3, 5, 9, 12])
def test_schedules_agree(gpu, nt):
    d = synth.generate(synth.GenSpec(**ZLEVEL))
    tr = [d.tracer(3, 1.0 + t, 0.5, seed=t) for t in range(nt)]
    ref, info = _run(d, tr, 0, 4)
    groups4 = {1: 1, 3: 2, 5: 2, 9: 3, 12: 3}[nt]          # 4-tracer groups, then 2, then 1
    assert info == {"launches": groups4, "sched": 0, "split": 4, "per_call": 1, "rows": 8}
    cands = [(1, 4), (0, 2), (1, 2)] + ([(0, 8), (1, 8)] if nt >= 8 else []) + \
        ([(0, 10), (1, 10)] if nt >= 10 else [])
    for sched, split in cands:
        got, info = _run(d, tr, sched, split)
        assert info["sched"] == sched and info["split"] == split
        for a, b in zip(ref, got):
            assert np.array_equal(a, b)


@pytest.mark.parametrize("nt", [1, 2, 4, 8, 10])
def test_tile_heights_agree(gpu, nt):
    # 4-row tiles step every column to the same bits as 8-row tiles, on both
    # schedules, with the mass fixer off; with it on, within 1e-12 relative
    d = synth.generate(synth.GenSpec(**ZLEVEL))
    tr = [d.tracer(3, 1.0 + t, 0.5, seed=t) for t in range(nt)]
    ref, _ = _run(d, tr, 0, 10, fix=False)
    for sched in (0, 1):
        got, info = _run(d, tr, sched, 10, rows=4, fix=False)
        assert info["rows"] == 4
        for a, b in zip(ref, got):
            assert np.array_equal(a, b)
    wp = d.water_mask()
    ref, _ = _run(d, tr, 0, 10)
    got, _ = _run(d, tr, 1, 10, rows=4)
    for a, b in zip(ref, got):
        assert np.max(np.abs(a[wp] - b[wp])) <= 1e-12 * np.max(np.abs(a[wp]))


def test_tile_list_matches_oracle(gpu):
    d = synth.generate(synth.GenSpec(**ZLEVEL))
    tr = [d.tracer(3, 2.0, 0.5, seed=3), d.tracer(1, 5.0, 20.0, seed=4)]
    got, _ = _run(d, tr, 1, 4, steps=10)
    wp = d.water_mask()
    work = O.Work(d)
    for P, g in zip(tr, got):
        Q = P.copy()
        for _ in range(10):
            assert O.step(d, Q, O.params(**PD), work=work) == 0
        assert np.linalg.norm(g[wp] - Q[wp]) / np.linalg.norm(Q[wp]) <= 1e-5
        assert np.array_equal(g[~wp], Q[~wp])


def test_autotune_keeps_state(gpu):
    d = domain("zlevel")
    tr = [d.tracer(3, 1.0 + t, 0.5, seed=t) for t in range(4)]
    ad = advdiff.AdvectionDiffusion(d)
    ad.set_hydro()
    b = batched.Batch(ad, 4)
    for t, P in enumerate(tr):
        b.set_tracer(t, P)
    before = [b.get_tracer(t) for t in range(4)]
    m0 = [b.mass(t) for t in range(4)]
    b.autotune(advdiff.params(**PD))
    info = b.schedule()
    assert info["sched"] in (0, 1) and info["split"] in (2, 4) and info["rows"] in (8, 4)
    after = [b.get_tracer(t) for t in range(4)]
    for x, y in zip(before, after):
        assert np.array_equal(x, y)
    assert [b.mass(t) for t in range(4)] == m0
    with pytest.raises(advdiff.N.MohidAdError):
        b.set_schedule(2, 4)
    b.destroy()
    ad.kill()


@pytest.mark.parametrize("form", ["mass_conservation", "imposed_value", "discharges"])
@pytest.mark.parametrize("storage", [batched.FP32, batched.FP16_QK])
def test_tile_heights_agree_open(gpu, form, storage):
    # the open-boundary forms (MassConservation alone; every boundary
    # treatment with discharges) at both tile heights and both schedules: the
    # same bits with the mass fixer off
    from tests.cases import discharges
    d = domain("open")
    tr = [d.tracer(3, 1.0 + t, 0.5, seed=t) for t in range(3)]
    refs = [d.reference(2.0 + t, 0.3, seed=10 + t) for t in range(3)]
    pd = dict(PD, DTProp=30.0, BoundaryCondition=2 if form == "imposed_value" else 1)
    ds = discharges(d, seed=1) if form == "discharges" else None

    def run(sched, rows):
        ad = advdiff.AdvectionDiffusion(d)
        ad.set_hydro()
        if ds is not None:
            ad.set_discharges(ds)
        b = batched.Batch(ad, len(tr), storage)
        b.set_mass_fix(False)
        for t, P in enumerate(tr):
            b.set_tracer(t, P)
            if ds is not None:
                b.set_discharge_conc(t, ds["Conc"] * (t + 1))
            b.set_reference(t, refs[t])
        b.set_schedule(sched, 4, rows)
        b.step(advdiff.params(**pd), nsteps=4, graph=True)
        b.sync()
        got = [b.get_tracer(t) for t in range(len(tr))]
        b.destroy()
        ad.kill()
        return got

    ref = run(0, 8)
    for sched, rows in ((1, 8), (0, 4), (1, 4)):
        for a, g in zip(ref, run(sched, rows)):
            assert np.array_equal(a, g)
