"""Run the transport step of one workload for profiling (ncu) or quick timing.

    python -m mohid_gb300.profile_step --config cfg2 --form batched --steps 5

Every step is the full transport step; the script only leaves out the CPU
baseline and end-to-end phases of bench.py.
"""
from __future__ import annotations

import argparse
import time

from . import advdiff, batched, build, configs, synth


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", default="cfg2", choices=sorted(configs.ALL))
    ap.add_argument("--form", default="batched", choices=["batched", "plain"])
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--storage", type=int, default=0, help="0 FP32, 1 FP16 transports, 2 FP16 transports+K")
    ap.add_argument("--ni", type=int, default=0)
    ap.add_argument("--nj", type=int, default=0)
    ap.add_argument("--tracers", type=int, default=0)
    ap.add_argument("--no-mass-fix", action="store_true", help="batched form without the mass fixer")
    ap.add_argument("--sched", type=int, default=-1,
                    help="batched schedule (0 one CTA per tile, 1 tile list) instead of the autotuner's choice")
    ap.add_argument("--split", type=int, default=4, help="largest tracer group per launch with --sched")
    ap.add_argument("--rows", type=int, default=8, help="tile height (8 or 4) with --sched")
    ap.add_argument("--rebind", action="store_true",
                    help="batched form: a new hydrodynamic state before every step (the FP64 fields bound "
                         "again from device memory, then the repack), as a coupled time loop does")
    args = ap.parse_args()
    build.build()
    import torch
    w = configs.ALL[args.config]()
    if args.ni or args.nj:
        w = w.scaled(ni=args.ni or None, nj=args.nj or None)
    d = synth.generate(w.spec)
    specs = w.tracers if not args.tracers else [w.tracers[t % len(w.tracers)] for t in range(args.tracers)]
    tr = [d.tracer(k, a, b, seed=100 + t) for t, (k, a, b) in enumerate(specs)]
    refs = [d.reference(2.0, 0.2, seed=200 + t) for t in range(len(tr))] if w.open_boundary else None
    ad = advdiff.AdvectionDiffusion(d)
    ad.set_hydro()
    p = advdiff.params(**w.params())
    if args.form == "batched":
        b = batched.Batch(ad, len(tr), args.storage)
        b.set_mass_fix(not args.no_mass_fix)
        if args.sched >= 0:
            b.set_schedule(args.sched, args.split, args.rows)   # no autotuner launches before the profiled ones
        for t, P in enumerate(tr):
            b.set_tracer(t, P)
            if refs:
                b.set_reference(t, refs[t])
        if args.rebind:
            dev = {n: torch.from_numpy(d.arrays[n]).cuda() for n in synth.F3}

            def run(n):
                for _ in range(n):
                    ad.set_fields(dev, bind=True)
                    b.step(p, nsteps=1)
        else:
            def run(n):
                b.step(p, nsteps=n)
        run(args.warmup)
        b.sync()
        t0 = time.perf_counter()
        run(args.steps)
        b.sync()
        el = time.perf_counter() - t0
        print(f"schedule {b.schedule()}")
        b.destroy()
        if args.rebind:
            ad.set_fields(dev, device=True)            # the instance's own copies again
            del dev
    else:
        bufs = [(torch.from_numpy(P).cuda(), torch.empty_like(torch.from_numpy(P)).cuda()) for P in tr]
        R = [torch.from_numpy(r).cuda() for r in refs] if refs else None
        def one():
            for t in range(len(bufs)):
                a_, b_ = bufs[t]
                ad.step_device(a_, b_, p, R[t] if R else None)
                bufs[t] = (b_, a_)
        for _ in range(args.warmup):
            one()
        ad.sync()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            one()
        ad.sync()
        el = time.perf_counter() - t0
    cells = d.ni * d.nj * d.nk * len(tr)
    print(f"{args.config} {args.form}: {el / args.steps * 1e3:.3f} ms/step, "
          f"{cells * args.steps / el:.4e} cell-tracer-updates/s (wall clock)")
    ad.kill()


if __name__ == "__main__":
    main()
