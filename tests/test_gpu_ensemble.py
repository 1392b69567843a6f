"""Ensemble launch (many independent domains in one persistent grid).

A member stepped inside an ensemble runs the same tile walk, with the same
arguments, as when it is stepped alone, so the two must agree bit for bit;
one member is also checked against the FP64 oracle at the batched form's
tolerance (relative L2 over water cells <= 1e-5).
"""
import dataclasses

import numpy as np
import pytest

from mohid_gb300 import advdiff, batched, configs, synth
from mohid_gb300._native import MohidAdError
from oracle import oracle as O

pytestmark = pytest.mark.gpu

# three small members: different sizes, layer counts, coasts, DT; a z-level one
MEMBERS = [
    dict(ni=40, nj=30, nk=6, land_frac=0.1, land_kind=1, seed=31, dt=20.0),
    dict(ni=70, nj=45, nk=12, land_frac=0.2, land_kind=0, seed=32, dt=45.0, bathy_kind=1),
    dict(ni=33, nj=65, nk=9, land_frac=0.25, land_kind=1, seed=33, dt=15.0, zlevel=True,
         hmin=2.0, hmax=60.0, bathy_kind=2),
]
OPTS = {
    "upwind1": dict(),
    "tvd_superbee": dict(AdvMethodH=4, TVDLimitationH=4, Upwind2H=1),
}


def _members(nt):
    out = []
    for m, spec in enumerate(MEMBERS):
        d = synth.generate(synth.GenSpec(**spec))
        tr = [d.tracer(3, 1.0 + 0.5 * t, 0.6, seed=100 * m + t) for t in range(nt)]
        out.append((d, tr))
    return out


def _load(members, nt):
    objs = []
    for d, tr in members:
        ad = advdiff.AdvectionDiffusion(d)
        ad.set_hydro()
        b = batched.Batch(ad, nt)
        for t, P in enumerate(tr):
            b.set_tracer(t, P)
        objs.append((ad, b))
    return objs


def _params(members, opt):
    return [advdiff.params(DTProp=d.spec.dt, **OPTS[opt]) for d, _ in members]


def _results(objs, nt):
    return [[b.get_tracer(t) for t in range(nt)] for _, b in objs]


def _free(objs):
    for ad, b in objs:
        b.destroy()
        ad.kill()


@pytest.mark.parametrize("opt", sorted(OPTS))
@pytest.mark.parametrize("nt", [1, 2, 4])
@pytest.mark.parametrize("graph", [False, True])
def test_ensemble_matches_members_stepped_alone(gpu, opt, nt, graph):
    members = _members(nt)
    steps = 5
    alone = _load(members, nt)
    for (ad, b), p in zip(alone, _params(members, opt)):
        b.step(p, nsteps=steps, graph=graph)
        b.sync()
    want = _results(alone, nt)
    _free(alone)

    objs = _load(members, nt)
    ens = batched.Ensemble([b for _, b in objs])
    ens.step(_params(members, opt), nsteps=steps, graph=graph)
    ens.sync()
    got = _results(objs, nt)
    ens.destroy()
    _free(objs)
    for w_m, g_m in zip(want, got):
        for w, g in zip(w_m, g_m):
            assert np.array_equal(w, g)


def test_ensemble_against_oracle(gpu):
    members = _members(4)
    objs = _load(members, 4)
    ens = batched.Ensemble([b for _, b in objs])
    pd = [dict(DTProp=d.spec.dt, **OPTS["tvd_superbee"]) for d, _ in members]
    steps = 20
    # two calls: a graph of 2 x 9 steps then one direct step (parity handling)
    ens.step([advdiff.params(**x) for x in pd], nsteps=19, graph=True)
    ens.step([advdiff.params(**x) for x in pd], nsteps=1, graph=False)
    ens.sync()
    got = _results(objs, 4)
    ens.destroy()
    _free(objs)
    for (d, tr), g_m, x in zip(members, got, pd):
        wp = d.water_mask()
        work = O.Work(d)
        for P, g in zip(tr, g_m):
            Q = P.copy()
            for _ in range(steps):
                assert O.step(d, Q, O.params(**x), work=work) == 0
            assert np.linalg.norm(g[wp] - Q[wp]) / np.linalg.norm(Q[wp]) <= 1e-5
            assert np.array_equal(g[~wp], Q[~wp])


def test_ensemble_cfg4_members_step(gpu):
    """The 64-member ensemble workload, scaled down 4x per axis, runs and stays finite."""
    ws = configs.cfg4_members(n=8)
    objs, pars = [], []
    for w in ws:
        s = w.spec
        d = synth.generate(dataclasses.replace(s, ni=max(8, s.ni // 4), nj=max(8, s.nj // 4)))
        ad = advdiff.AdvectionDiffusion(d)
        ad.set_hydro()
        b = batched.Batch(ad, 4)
        for t, (k, a, bb) in enumerate(w.tracers):
            b.set_tracer(t, d.tracer(k, a, bb, seed=t))
        objs.append((ad, b))
        pars.append(advdiff.params(**w.params()))
    ens = batched.Ensemble([b for _, b in objs])
    ens.step(pars, nsteps=10, graph=True)
    ens.sync()
    for (ad, b), w in zip(objs, ws):
        for t in range(4):
            g = b.get_tracer(t)
            assert np.isfinite(g[ad.domain.water_mask()]).all()
    ens.destroy()
    _free(objs)


def test_ensemble_rejects(gpu):
    members = _members(2)
    objs = _load(members[:2], 2)
    d3, tr3 = members[2]
    ad3 = advdiff.AdvectionDiffusion(d3)
    ad3.set_hydro()
    b1 = batched.Batch(ad3, 1)
    with pytest.raises(MohidAdError) as e:
        batched.Ensemble([objs[0][1], b1])                       # different tracer counts
    assert e.value.code == 3
    b1.destroy()
    b16 = batched.Batch(ad3, 2, batched.FP16_Q)
    with pytest.raises(MohidAdError) as e:
        batched.Ensemble([objs[0][1], b16])                      # FP16 storage
    assert e.value.code == 4
    b16.destroy()
    ad3.kill()
    ens = batched.Ensemble([b for _, b in objs])
    with pytest.raises(MohidAdError) as e:                       # a member stepped alone
        objs[0][1].step(advdiff.params(DTProp=20.0), nsteps=1)
    assert e.value.code == 3
    with pytest.raises(MohidAdError) as e:                       # different advection schemes
        ens.step([advdiff.params(DTProp=20.0), advdiff.params(DTProp=20.0, **OPTS["tvd_superbee"])])
    assert e.value.code == 3
    with pytest.raises(MohidAdError) as e:                       # a member destroyed while in use
        objs[1][1].destroy()
    assert e.value.code == 3
    ens.destroy()
    _free(objs)
