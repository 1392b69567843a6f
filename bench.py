#!/usr/bin/env python3
"""Throughput of the GB300 tracer advection-diffusion step (cell-tracer-updates/s).

Workload (N=1): config 2 -- 512x512x40 sigma grid, bathymetry 5-200 m, P2_TVD
SuperBee horizontal advection, implicit vertical advection/diffusion, 2 tracers
(temperature, salinity), DT 20 s.  Seeded synthetic inputs.  One "step" is one
transport time step of every tracer.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--form plain|batched]
  python bench.py --impl reference ...   # the reference path on the host CPU cores

`value` is measured device-resident (inputs in HBM, CUDA events on the
launching stream); `e2e` goes through the host-pointer C-ABI with pinned host
buffers, host<->device copies inside the timed region.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

L2_BYTES = 129 * 2**20
FALLBACK_HBM_GBS = 6800.0


# ----------------------------------------------------------------------------- helpers
def load_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            d = json.loads(p.read_text())
            return float(d["hbm_gbs"]), "measured"
        except Exception:
            pass
    return FALLBACK_HBM_GBS, "fallback"


class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region (every 200 ms)."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int = 0):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200", "-f", self.path],
                stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        time.sleep(0.3)

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        try:
            for line in Path(self.path).read_text().splitlines():
                f = [x.strip() for x in line.split(",")]
                if len(f) >= 9:
                    rows.append(f)
            os.unlink(self.path)
        except Exception:
            pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [num(r[1]) for r in rows if num(r[1]) is not None]
        mx = [num(r[2]) for r in rows if num(r[2]) is not None]
        pw = [num(r[3]) for r in rows if num(r[3]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[q] for r in rows for q in range(4) if r[5 + q].lower() == "active"})
        loaded = [s for s, p in zip(sm, pw) if pw and p >= 0.5 * max(pw)] or sm
        return {"sm_mhz": statistics.median(loaded) if loaded else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(rows)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x: float, world: int) -> float:
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def workload():
    from mohid_gb300 import configs
    return configs.cfg2()


WORKLOAD_NAME = "cfg2: 512x512x40 sigma, bathymetry 5-200 m, P2_TVD SuperBee, 2 tracers (T, S), DT 20 s"


# ----------------------------------------------------------------------------- CPU baseline
def cpu_baseline(w, d, tracers, budget_s: float = 12.0, nthreads: int = 0):
    """The oracle (FP64 restatement of the reference CPU path, OpenMP) on a bounded
    sample: whole steps of the same grid, one tracer, until `budget_s` is spent."""
    from oracle import oracle as O
    cores = nthreads or os.cpu_count() or 1
    P = tracers[0].copy()
    p = O.params(**w.params())
    work = O.Work(d)
    O.step(d, P, p, work=work, nthreads=cores)          # warm-up (first touch)
    n = 0
    t0 = time.perf_counter()
    while True:
        rc = O.step(d, P, p, work=work, nthreads=cores)
        assert rc == 0
        n += 1
        el = time.perf_counter() - t0
        if el >= budget_s or n >= 50:
            break
    cells = d.ni * d.nj * d.nk
    return {"value": cells * n / el, "unit": "cell-tracer-updates/s", "cores": cores,
            "kind": "port",
            "sample": f"{n} oracle steps of 1 tracer on the {d.ni}x{d.nj}x{d.nk} grid "
                      f"({el:.1f} s, OpenMP, {cores} threads)"}


# ----------------------------------------------------------------------------- GPU: plain FP64
def run_plain(w, d, tracers, steps, warmup, world):
    import numpy as np
    import torch
    from mohid_gb300 import advdiff

    nt = len(tracers)
    ad = advdiff.AdvectionDiffusion(d)
    ad.set_hydro()
    p = advdiff.params(**w.params())
    bufs = [(torch.from_numpy(P).cuda(), torch.empty_like(torch.from_numpy(P)).cuda()) for P in tracers]
    stream = torch.cuda.ExternalStream(ad.stream)

    def one_step():
        nonlocal bufs
        for t in range(nt):
            a, b = bufs[t]
            ad.step_device(a, b, p)
            bufs[t] = (b, a)

    for _ in range(warmup):
        one_step()
    ad.sync()
    torch.cuda.synchronize()
    barrier(world)
    clk = ClockSampler(torch.cuda.current_device())
    clk.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        one_step()
    e1.record(stream)
    e1.synchronize()
    ad.sync()
    clocks = clk.stop()
    ms = e0.elapsed_time(e1) / steps
    barrier(world)

    # e2e: the host-pointer C-ABI (set_hydro once per step + one call per tracer)
    host = [torch.from_numpy(P.copy()).pin_memory() for P in tracers]
    hydro_pinned = {}
    for n in list(d.arrays):
        hydro_pinned[n] = torch.from_numpy(d.arrays[n]).pin_memory().numpy()
    from mohid_gb300.synth import Domain
    dp = Domain(spec=d.spec, arrays=hydro_pinned)
    hv = [h.numpy() for h in host]
    e2e_steps = max(3, min(steps, 20))
    ad.set_hydro(dp)
    for t in range(nt):
        ad.step(hv[t], p)
    torch.cuda.synchronize()
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        ad.set_hydro(dp)
        for t in range(nt):
            ad.step(hv[t], p)
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    from mohid_gb300.synth import F3, I3
    h2d = sum(hydro_pinned[n].nbytes for n in F3 + I3) + nt * tracers[0].nbytes
    d2h = nt * tracers[0].nbytes
    ad.kill()
    cells = d.ni * d.nj * d.nk
    return dict(ms=ms, kernel_ms=ms / nt, launches=steps * nt, e2e_s=e2e_s, h2d=h2d, d2h=d2h,
                cells=cells, nt=nt, bytes_per_update=96.0, bytes_per_launch=96.0 * cells, dtype="f64",
                clocks=clocks,
                kernel="plain_f64_kernel")


# ----------------------------------------------------------------------------- GPU: batched FP32
def run_batched(w, d, tracers, steps, warmup, world, storage=0):
    import torch
    from mohid_gb300 import advdiff, batched
    from mohid_gb300.synth import Domain, F3, I3

    nt = len(tracers)
    ad = advdiff.AdvectionDiffusion(d)
    ad.set_hydro()
    b = batched.Batch(ad, nt, storage)
    for t, P in enumerate(tracers):
        b.set_tracer(t, P)
    p = advdiff.params(**w.params())
    b.step(p, nsteps=warmup, graph=False)
    b.step(p, nsteps=steps, graph=True)          # capture the graph outside the timed region
    b.sync()
    stream = torch.cuda.ExternalStream(ad.stream)
    torch.cuda.synchronize()
    barrier(world)
    clk = ClockSampler(torch.cuda.current_device())
    clk.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    b.step(p, nsteps=steps, graph=True)
    e1.record(stream)
    e1.synchronize()
    b.sync()
    clocks = clk.stop()
    ms = e0.elapsed_time(e1) / steps
    barrier(world)
    groups, left = 0, nt                       # launches per step: groups of 4, 2, 1 tracers
    while left > 0:
        left -= 4 if left >= 4 else (2 if left >= 2 else 1)
        groups += 1
    launches = steps * groups

    # e2e: a host-resident caller sends the step's hydrodynamics and tracers,
    # runs the step through the C-ABI and reads the tracers back, every step
    pinned = {n: torch.from_numpy(d.arrays[n]).pin_memory().numpy() for n in d.arrays}
    dp = Domain(spec=d.spec, arrays=pinned)
    host = [torch.from_numpy(P.copy()).pin_memory().numpy() for P in tracers]
    e2e_steps = max(3, min(steps, 10))

    def e2e_step():
        ad.set_hydro(dp)
        for t in range(nt):
            b.set_tracer(t, host[t])
        b.step(p, nsteps=1)
        for t in range(nt):
            b.get_tracer(t, host[t])
    e2e_step()
    torch.cuda.synchronize()
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_step()
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    h2d = sum(pinned[n].nbytes for n in F3 + I3) + nt * tracers[0].nbytes
    d2h = nt * tracers[0].nbytes
    b.destroy()
    ad.kill()
    cells = d.ni * d.nj * d.nk
    shared = {0: 48.0, 1: 42.0, 2: 38.0}[storage]
    # one launch per step when nt <= 2 or nt == 4: the launch moves cells * (8 nt + shared) bytes
    return dict(ms=ms, kernel_ms=ms / groups, launches=launches, e2e_s=e2e_s, h2d=h2d, d2h=d2h,
                cells=cells, nt=nt, bytes_per_update=8.0 + shared / nt,
                bytes_per_launch=cells * (8.0 * nt + shared) / groups, dtype="f32", clocks=clocks,
                kernel="batched_kernel<2,P2_TVD,SuperBee>")


# ----------------------------------------------------------------------------- main
def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--form", default="batched", choices=["batched", "plain"])
    ap.add_argument("--cpu-budget", type=float, default=12.0)
    args = ap.parse_args()
    world, rank, local = dist_setup()
    if args.warmup < 3 and args.impl != "reference":
        args.warmup = 3

    from mohid_gb300 import build as B
    B.build()
    from mohid_gb300 import synth
    w = workload()
    d = synth.generate(w.spec)
    tracers = [d.tracer(k, a, b, seed=100 + t) for t, (k, a, b) in enumerate(w.tracers)]
    cells = d.ni * d.nj * d.nk
    unit = "cell-tracer-updates/s"
    metric = "cell-tracer-updates/s, FP32 batched vs FP64 plain on 1 GB300 at \u22641e-5 rel L2; HBM GB/s"

    if args.impl == "reference":
        if rank != 0:
            return
        from oracle import oracle as O
        cores = os.cpu_count() or 1
        p = O.params(**w.params())
        work = O.Work(d)
        Ps = [P.copy() for P in tracers]
        for _ in range(args.warmup):
            for P in Ps:
                O.step(d, P, p, work=work, nthreads=cores)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            for P in Ps:
                assert O.step(d, P, p, work=work, nthreads=cores) == 0
        el = time.perf_counter() - t0
        value = cells * len(Ps) * args.steps / el
        line = {"impl": "reference", "metric": metric, "value": value, "unit": unit,
                "n_gpus": 0, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": el / args.steps * 1e3, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
                "config": {"workload": WORKLOAD_NAME, "form": "reference CPU path (FP64 restatement, "
                           "OpenMP, full-array passes as ModuleAdvectionDiffusion)"},
                "cpu_baseline": {"value": value, "unit": unit, "cores": cores, "kind": "port",
                                 "sample": f"{args.steps} full steps x {len(Ps)} tracers"},
                "e2e": {"value": value, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    import torch
    plain = None
    if args.form == "batched":
        r = run_batched(w, d, tracers, args.steps, args.warmup, world)
        plain = run_plain(w, d, tracers, max(3, args.steps // 4), 3, world)
    else:
        r = run_plain(w, d, tracers, args.steps, args.warmup, world)
    ms = max_over_ranks(r["ms"], world)
    value = world * cells * r["nt"] / (ms / 1e3)
    e2e_s = max_over_ranks(r["e2e_s"], world)
    e2e_value = world * cells * r["nt"] / e2e_s
    peak, peak_kind = load_peaks()
    achieved = r["bytes_per_launch"] / (r["kernel_ms"] / 1e3) / 1e9
    traffic = TRAFFIC.get(r["kernel"])
    if rank != 0:
        return
    cpu = cpu_baseline(w, d, tracers, budget_s=args.cpu_budget)
    resident = sum(a.nbytes for a in d.arrays.values()) + 2 * sum(P.nbytes for P in tracers)
    line = {
        "metric": metric, "value": value, "unit": unit, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": r["dtype"],
        "data": "synthetic (seeded generator restating MOHID geometry/mask/continuity rules)",
        "config": {"workload": WORKLOAD_NAME, "form": args.form,
                   "time_loop": "CUDA graph of K steps" if args.form == "batched" else "stream launches",
                   "cells": cells, "tracers": r["nt"],
                   "l2": f"inputs larger than L2 ({resident / 2**30:.2f} GiB resident per step > 129 MiB)",
                   "parallelism": f"replicas x{world}" if world > 1 else "single GPU"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "traffic_unit": "bytes per launch",
                     "bytes_per_launch": r["bytes_per_launch"],
                     "kernel": r["kernel"], "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)"
                     if peak_kind == "measured" else "fallback 6.8 TB/s",
                     "bytes_per_update": r["bytes_per_update"]},
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": unit, "h2d_bytes_per_step": r["h2d"],
                "d2h_bytes_per_step": r["d2h"]},
        "gpu_launches": r["launches"],
        "clocks": r["clocks"],
    }
    if plain is not None:
        pv = world * cells * plain["nt"] / (max_over_ranks(plain["ms"], world) / 1e3)
        line["plain_f64"] = {"value": pv, "unit": unit, "ms_per_step": plain["ms"],
                             "speedup_batched_over_plain": value / pv,
                             "roofline_frac": 96.0 * cells / (plain["kernel_ms"] / 1e3) / 1e9 / peak}
    print(json.dumps(line))


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per launch of the
# dominant kernel, from one ncu capture of the 512x512x40 two-tracer workload
# (profiles/batched_kernel_512x512x40_2tracers.md, profiles/plain_f64_kernel_512x512x40.md).
TRAFFIC: dict = {
    "batched_kernel<2,P2_TVD,SuperBee>": 644.790272e6 + 145.795840e6,
    "plain_f64_kernel": 1181.614e6 + 139.056384e6,
}

if __name__ == "__main__":
    main()
