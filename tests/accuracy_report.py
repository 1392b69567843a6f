"""Accuracy of the batched FP32 form against the FP64 oracle over long runs.

    python tests/accuracy_report.py --config cfg2 --steps 1000 [--ni 256 --nj 256]

Prints one JSON line per tracer: relative L2 and max-abs error over water
cells after `steps` steps; the relative mass defect of the FP32 form (mass now
- mass at the start - mass moved through open boundaries, over the mass at the
start; the boundary flux as the mass fixer followed it, 0 on closed domains);
and the FP32 form's mass change against the oracle's FP64 one.  Not collected by
pytest (a GPU run of several minutes); the numbers are quoted in the docs.
"""
from __future__ import annotations

import argparse
import json
import sys
import time
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parent.parent))

from mohid_gb300 import advdiff, batched, build, configs, synth  # noqa: E402
from oracle import oracle as O  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", default="cfg2")
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--ni", type=int, default=0)
    ap.add_argument("--nj", type=int, default=0)
    ap.add_argument("--storage", type=int, default=0)
    ap.add_argument("--tracers", type=int, default=0)
    args = ap.parse_args()
    build.build()
    O.build()
    w = configs.ALL[args.config]()
    if args.ni or args.nj:
        w = w.scaled(ni=args.ni or None, nj=args.nj or None)
    d = synth.generate(w.spec)
    specs = w.tracers if not args.tracers else w.tracers[:args.tracers]
    tr = [d.tracer(k, a, b, seed=100 + t) for t, (k, a, b) in enumerate(specs)]
    refs = [d.reference(2.0, 0.2, seed=200 + t) for t in range(len(tr))] if w.open_boundary else None
    pd = w.params()
    ad = advdiff.AdvectionDiffusion(d)
    ad.set_hydro()
    b = batched.Batch(ad, len(tr), args.storage)
    for t, P in enumerate(tr):
        b.set_tracer(t, P)
        if refs:
            b.set_reference(t, refs[t])
    m0 = [O.mass(d, P) for P in tr]                # FP64 mass of the loaded fields
    b.step(advdiff.params(**pd), nsteps=args.steps, graph=True)
    b.sync()
    got = [b.get_tracer(t) for t in range(len(tr))]
    m1 = [b.mass(t) for t in range(len(tr))]
    fl = [b.boundary_flux(t) for t in range(len(tr))]
    b.destroy()
    ad.kill()
    wp = d.water_mask()
    work = O.Work(d)
    for t, P in enumerate(tr):
        Q = P.copy()
        mo0 = O.mass(d, Q)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            assert O.step(d, Q, O.params(**pd), ReferenceProp=None if refs is None else refs[t],
                          work=work) == 0
        el = time.perf_counter() - t0
        mo1 = O.mass(d, Q)
        g = got[t]
        out = {"config": args.config, "grid": [d.ni, d.nj, d.nk], "steps": args.steps,
               "tracer": t, "storage": args.storage,
               "rel_l2": float(np.linalg.norm(g[wp] - Q[wp]) / np.linalg.norm(Q[wp])),
               "max_abs": float(np.max(np.abs(g[wp] - Q[wp]))),
               "boundary_flux": fl[t] / abs(m0[t]),
               "mass_defect_fp32": abs(m1[t] - m0[t] - (fl[t] if refs else 0.0)) / abs(m0[t]),
               "mass_change_fp32_vs_oracle": abs((m1[t] - m0[t]) - (mo1 - mo0)) / abs(mo0),
               "mass_fp32_vs_oracle": abs(m1[t] - mo1) / abs(mo1),
               "oracle_seconds": el}
        print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
