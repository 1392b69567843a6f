"""Regression fixtures (tests/golden/small_cases.npz, written by
tests/golden/make_golden.py): the oracle and the FP64 drop-in must reproduce the
stored fields bit for bit on any machine; the batched FP32 form must stay within
its one-step-class tolerance (relative L2 over water cells <= 1e-6 after the
three stored steps)."""
from pathlib import Path

import numpy as np
import pytest

from mohid_gb300 import synth
from oracle import oracle as O

FIX = Path(__file__).resolve().parent / "golden" / "small_cases.npz"
GRIDS = ["coast", "zlevel", "open"]
OPTS = ["upwind1", "tvd_superbee", "tvd_minmod", "upwind3", "explicit_v_tvd", "nulldif"]
BATCHED_OPTS = ["upwind1", "tvd_superbee", "tvd_minmod", "nulldif"]
STEPS = 3


def _load():
    z = np.load(FIX)
    cases = {}
    for g in GRIDS:
        spec = {k.split("/")[-1]: z[k].item() for k in z.files if k.startswith(f"{g}/spec/")}
        arrays = {n: z[f"{g}/{n}"] for n in synth.F3 + synth.I3 + synth.F2 + synth.I2}
        d = synth.Domain(spec=synth.GenSpec(**spec), arrays=arrays)
        ref = z[f"{g}/Ref"] if f"{g}/Ref" in z.files else None
        want = {o: z[f"{g}/{o}/P{STEPS}"] for o in OPTS}
        cases[g] = (d, z[f"{g}/P0"], ref, want)
    return cases


def _params(o, ref):
    from tests.cases import OPTIONS
    pd = dict(DTProp=30.0, **OPTIONS[o])
    if ref is not None:
        pd.update(BoundaryCondition=1, DecayTime=0.0)
    return pd


@pytest.fixture(scope="module")
def cases():
    return _load()


@pytest.mark.parametrize("grid", GRIDS)
def test_oracle_reproduces_fixture(built, cases, grid):
    d, P0, ref, want = cases[grid]
    for o in OPTS:
        P = P0.copy()
        work = O.Work(d)
        for _ in range(STEPS):
            assert O.step(d, P, O.params(**_params(o, ref)), ReferenceProp=ref, work=work) == 0
        assert np.array_equal(P, want[o]), (grid, o)


@pytest.mark.gpu
@pytest.mark.parametrize("grid", GRIDS)
def test_plain_f64_reproduces_fixture(gpu, cases, grid):
    from mohid_gb300 import advdiff
    d, P0, ref, want = cases[grid]
    ad = advdiff.AdvectionDiffusion(d)
    ad.set_hydro()
    for o in OPTS:
        P = P0.copy()
        for _ in range(STEPS):
            ad.step(P, advdiff.params(**_params(o, ref)), ref)
        assert np.array_equal(P, want[o]), (grid, o)
    ad.kill()


@pytest.mark.gpu
@pytest.mark.parametrize("grid", GRIDS)
def test_batched_close_to_fixture(gpu, cases, grid):
    from mohid_gb300 import advdiff, batched
    d, P0, ref, want = cases[grid]
    wp = d.water_mask()
    ad = advdiff.AdvectionDiffusion(d)
    ad.set_hydro()
    for o in BATCHED_OPTS:
        b = batched.Batch(ad, 1)
        b.set_tracer(0, P0)
        if ref is not None:
            b.set_reference(0, ref)
        b.step(advdiff.params(**_params(o, ref)), nsteps=STEPS)
        b.sync()
        g = b.get_tracer(0)
        b.destroy()
        w = want[o]
        assert np.linalg.norm(g[wp] - w[wp]) / np.linalg.norm(w[wp]) <= 1e-6, (grid, o)
        assert np.array_equal(g[~wp], w[~wp]), (grid, o)
    ad.kill()
