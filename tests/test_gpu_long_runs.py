"""Long runs of the batched FP32 form at the workloads' sizes against the FP64 oracle.

The FP32 form's accuracy target: relative L2 over water cells <= 1e-5 against
the FP64 oracle after the workload's steps, with the relative mass defect
|M_now - M_loaded - boundary flux since| / M_loaded <= 1e-12 (the mass fixer
on, as by default).  Every case runs its steps in one step call with the CUDA
graph, as a time loop would.

* 512x512x40 sigma grid (P2_TVD SuperBee, temperature and salinity, DT 20 s),
  full size, 1000 steps;
* the first 8 members of the 64-domain ensemble at their full sizes
  (226x149x23 .. 495x250x39, 4 tracers each, each its own DT), one ensemble
  launch per step, 100 steps;
* a 512x512x30 cut of the 4096x4096x30 open-boundary workload: P2_TVD MinMod,
  20 lognormal tracers, FP16-stored transports and diffusivities,
  MassConservation open boundaries on the west and east sides with Dirichlet
  inflow (DecayTime 0: inflow takes the reference concentration), 100 steps.
  The oracle runs on the exact FP64 fields, so the bar covers the FP16
  storage as well as the FP32 arithmetic.  (Rounding the fields themselves to
  FP16 would break the transports' FP64 continuity, and the mass fixer only
  runs where the step maps constants onto themselves.)

The oracle takes minutes here (about 1e8 cell-tracer-updates/s on 16 cores);
the cases are marked `long` as well as `gpu`, so a quick GPU run can leave
them out with -m "gpu and not long".
"""
import json

import numpy as np
import pytest

from mohid_gb300 import advdiff, batched, configs, synth
from oracle import oracle as O

pytestmark = [pytest.mark.gpu, pytest.mark.long]
TOL_L2 = 1e-5
TOL_MASS = 1e-12


def _oracle(d, P, pd, steps, ref=None):
    work = O.Work(d)
    Q = P.copy()
    p = O.params(**pd)
    for _ in range(steps):
        assert O.step(d, Q, p, ReferenceProp=ref, work=work) == 0
    return Q


def _check(name, d, tracers, got, masses, fluxes, pd, steps, refs=None):
    """Assert the targets per tracer; print one JSON line per tracer."""
    wp = d.water_mask()
    worst = {}
    for t, P in enumerate(tracers):
        ref = None if refs is None else refs[t]
        Q = _oracle(d, P, pd, steps, ref)
        g = got[t]
        m0 = O.mass(d, P)
        rel = float(np.linalg.norm(g[wp] - Q[wp]) / np.linalg.norm(Q[wp]))
        defect = abs(masses[t] - m0 - fluxes[t]) / abs(m0)
        out = {"case": name, "grid": [d.ni, d.nj, d.nk], "steps": steps, "tracer": t,
               "rel_l2": rel, "max_abs": float(np.max(np.abs(g[wp] - Q[wp]))),
               "mass_defect": defect,
               "mass_change_vs_oracle": abs((masses[t] - m0) - (O.mass(d, Q) - m0)) / abs(m0)}
        print(json.dumps(out), flush=True)
        assert rel <= TOL_L2, out
        assert defect <= TOL_MASS, out
        assert np.array_equal(g[~wp], Q[~wp])       # land, null and halo cells as the reference leaves them
        worst = out if not worst or rel > worst["rel_l2"] else worst
    return worst


def _run_batch(d, tracers, pd, steps, storage=batched.FP32, refs=None):
    ad = advdiff.AdvectionDiffusion(d)
    ad.set_hydro()
    b = batched.Batch(ad, len(tracers), storage)
    for t, P in enumerate(tracers):
        b.set_tracer(t, P)
        if refs is not None:
            b.set_reference(t, refs[t])
    b.step(advdiff.params(**pd), nsteps=steps, graph=True)
    b.sync()
    got = [b.get_tracer(t) for t in range(len(tracers))]
    masses = [b.mass(t) for t in range(len(tracers))]
    fluxes = [b.boundary_flux(t) if refs is not None else 0.0 for t in range(len(tracers))]
    b.destroy()
    ad.kill()
    return got, masses, fluxes


def test_cfg2_full_size_1000_steps(gpu):
    w = configs.cfg2()
    d = synth.generate(w.spec)
    tr = [d.tracer(k, a, b, seed=100 + t) for t, (k, a, b) in enumerate(w.tracers)]
    got, masses, fluxes = _run_batch(d, tr, w.params(), w.steps)
    _check("512x512x40 SuperBee T+S", d, tr, got, masses, fluxes, w.params(), w.steps)


def test_ensemble_members_full_size(gpu):
    ws = configs.cfg4_members(n=8)
    steps = 100
    members, objs = [], []
    for w in ws:
        d = synth.generate(w.spec)
        tr = [d.tracer(k, a, bb, seed=10 * t + 1) for t, (k, a, bb) in enumerate(w.tracers)]
        ad = advdiff.AdvectionDiffusion(d)
        ad.set_hydro()
        b = batched.Batch(ad, len(tr))
        for t, P in enumerate(tr):
            b.set_tracer(t, P)
        members.append((w, d, tr))
        objs.append((ad, b))
    ens = batched.Ensemble([b for _, b in objs])
    ens.step([advdiff.params(**w.params()) for w in ws], nsteps=steps, graph=True)
    ens.sync()
    res = [([b.get_tracer(t) for t in range(4)], [b.mass(t) for t in range(4)]) for _, b in objs]
    ens.destroy()
    for ad, b in objs:
        b.destroy()
        ad.kill()
    for (w, d, tr), (got, masses) in zip(members, res):
        _check(w.name, d, tr, got, masses, [0.0] * 4, w.params(), steps)


def test_open_boundary_fp16_cut_20_tracers(gpu):
    w = configs.cfg5().scaled(ni=512, nj=512)
    d = synth.generate(w.spec)
    tr = [d.tracer(k, a, b, seed=100 + t) for t, (k, a, b) in enumerate(w.tracers)]
    refs = [d.reference(2.0, 0.2, seed=200 + t) for t in range(len(tr))]
    pd = w.params()
    assert pd["BoundaryCondition"] == 1 and pd["DecayTime"] == 0.0
    got, masses, fluxes = _run_batch(d, tr, pd, w.steps, storage=batched.FP16_QK, refs=refs)
    _check("512x512x30 MinMod open FP16", d, tr, got, masses, fluxes, pd, w.steps, refs)
