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
import math
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
    """SM clock, power and clock-event (throttle) reasons sampled during the timed
    region: NVML through ctypes every 2 ms (read-only queries), else nvidia-smi
    every 200 ms.  stop() keeps the samples taken between mark_start() and
    mark_end() (the host window around the timed steps)."""
    NAMES = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown",
             0x40: "hw_thermal_slowdown", 0x80: "hw_power_brake_slowdown"}

    def __init__(self, index: int = 0):
        self.index = index
        self.uuid = None
        try:
            import torch
            u = getattr(torch.cuda.get_device_properties(index), "uuid", None)
            if u is not None:
                self.uuid = "GPU-" + str(u)
        except Exception:
            pass
        self.samples = []
        self.t0 = self.t1 = None
        self._stop = threading.Event()
        self._thread = None
        self._smi = None
        self.source = None

    def _nvml(self):
        import ctypes as C
        lib = C.CDLL("libnvidia-ml.so.1")
        if lib.nvmlInit_v2() != 0:
            raise RuntimeError("nvmlInit failed")
        h = C.c_void_p()
        if not (self.uuid and lib.nvmlDeviceGetHandleByUUID(self.uuid.encode(), C.byref(h)) == 0):
            if lib.nvmlDeviceGetHandleByIndex_v2(C.c_uint(self.index), C.byref(h)) != 0:
                raise RuntimeError("nvml handle")
        reasons_fn = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            getattr(lib, "nvmlDeviceGetCurrentClocksThrottleReasons")

        def sample():
            clk, mx, pw = C.c_uint(), C.c_uint(), C.c_uint()
            rs = C.c_ulonglong()
            lib.nvmlDeviceGetClockInfo(h, C.c_int(1), C.byref(clk))          # NVML_CLOCK_SM
            lib.nvmlDeviceGetMaxClockInfo(h, C.c_int(1), C.byref(mx))
            lib.nvmlDeviceGetPowerUsage(h, C.byref(pw))
            reasons_fn(h, C.byref(rs))
            return (time.perf_counter(), float(clk.value), float(mx.value), pw.value / 1000.0, int(rs.value))
        sample()
        return sample

    def start(self):
        try:
            sample = self._nvml()
            self.source = "nvml, 2 ms"

            def run():
                while not self._stop.is_set():
                    try:
                        self.samples.append(sample())
                    except Exception:
                        pass
                    time.sleep(0.002)
            self._thread = threading.Thread(target=run, daemon=True)
            self._thread.start()
        except Exception:
            self.source = "nvidia-smi, 200 ms"
            try:
                fd, self._path = tempfile.mkstemp(suffix=".csv")
                os.close(fd)
                q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
                     "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
                     "clocks_event_reasons.sw_power_cap")
                self._smi = subprocess.Popen(
                    ["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                     "-lms", "200", "-f", self._path], stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
            except Exception:
                self._smi = None
        time.sleep(0.05)

    def mark_start(self):
        self.t0 = time.perf_counter()

    def mark_end(self):
        self.t1 = time.perf_counter()

    def stop(self):
        time.sleep(0.01)
        self._stop.set()
        if self._thread:
            self._thread.join(timeout=2)
        rows = list(self.samples)
        if self._smi:
            time.sleep(0.25)
            self._smi.terminate()
            try:
                self._smi.wait(timeout=5)
            except Exception:
                self._smi.kill()
            try:
                for line in Path(self._path).read_text().splitlines():
                    f = [x.strip() for x in line.split(",")]
                    if len(f) >= 7:
                        bits = sum(b for b, v in zip((0x8, 0x40, 0x20, 0x4), f[3:7]) if v.lower() == "active")
                        rows.append((None, float(f[0]), float(f[1]), float(f[2]), bits))
                os.unlink(self._path)
            except Exception:
                pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "source": self.source}
        inside = [r for r in rows if r[0] is not None and self.t0 is not None and self.t0 <= r[0] <= self.t1]
        use = inside or rows
        reasons = sorted({n for r in use for bit, n in self.NAMES.items() if r[4] & bit})
        return {"sm_mhz": statistics.median(r[1] for r in use), "sm_max_mhz": max(r[2] for r in use),
                "reasons": reasons, "samples": len(use), "power_w_max": max(r[3] for r in use),
                "window": "timed region" if inside else "around the timed region", "source": self.source}


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


# ----------------------------------------------------------------------------- workloads
# name -> (description, storage of the batched form: 0 FP32, 1 FP16 transports,
#          2 FP16 transports and diffusivities)
WORKLOADS = {
    "cfg2": ("512x512x40 sigma, bathymetry 5-200 m, P2_TVD SuperBee, 2 tracers (T, S), DT 20 s", 0),
    "cfg3": ("2048x1024x50 z-level, 35% fractal coast, columns of 1-50 layers, Upwind1, 8 tracers, "
             "FP16-scaled transports, DT 15 s", 1),
    "cfg4": ("64 independent domains 64x64x10 .. 512x256x40 (log-uniform), Upwind1, 4 tracers each, "
             "DT 10-60 s, one persistent launch per step, CUDA graph", 0),
    "cfg5": ("4096x4096x30 sigma, P2_TVD MinMod, 20 tracers, open W and E boundaries (MassConservation, "
             "Dirichlet inflow), FP16-scaled transports and diffusivities, DT 10 s", 2),
}
SHARED_BYTES = {0: 48.0, 1: 42.0, 2: 38.0}     # per-cell shared fields read once per step


def groups_of(nt: int) -> int:
    """Launches per step of the batched form: tracers go in groups of 4, 2, 1."""
    g, left = 0, nt
    while left > 0:
        left -= 4 if left >= 4 else (2 if left >= 2 else 1)
        g += 1
    return g


class Case:
    """One domain of a workload: grid, tracers (generated on demand) and references."""

    def __init__(self, w, distinct_tracers: int | None = None):
        from mohid_gb300 import synth
        self.w = w
        self.d = synth.generate(w.spec)
        self.nt = len(w.tracers)
        # large workloads reuse a few distinct seeded fields, scaled per tracer
        self.distinct = distinct_tracers or self.nt
        self._base = {}
        self._mass = {}
        self.refs = None
        if w.open_boundary:
            self.refs = [self.d.reference(1.0 + 0.1 * t, 0.3, seed=500 + t) for t in range(min(self.nt, 4))]

    def tracer(self, t: int):
        import numpy as np
        k, a, b = self.w.tracers[t]
        if self.distinct >= self.nt:
            return self.d.tracer(k, a, b, seed=100 + t)
        q = t % self.distinct
        if q not in self._base:
            kq, aq, bq = self.w.tracers[q]
            self._base[q] = self.d.tracer(kq, aq, bq, seed=100 + q)
        scale = a / self.w.tracers[q][1]
        out = self._base[q] * scale
        out[~self.d.water_mask()] = self._base[q][~self.d.water_mask()]
        return np.ascontiguousarray(out)

    def ref(self, t: int):
        return None if self.refs is None else self.refs[t % len(self.refs)]

    def load_mass(self, t: int) -> float:
        """FP64 mass (sum of VolumeZ * value over water cells) of tracer t as
        loaded, layer by layer; a scaled tracer's is the scaled mass of its base."""
        import numpy as np
        q = t % self.distinct if self.distinct < self.nt else t
        if q not in self._mass:
            P = self.tracer(q)
            V, wp = self.d.arrays["VolumeZ"], self.d.water_mask()
            self._mass[q] = float(sum(np.dot(V[k][wp[k]], P[k][wp[k]]) for k in range(V.shape[0])))
        scale = self.w.tracers[t][1] / self.w.tracers[q][1] if self.distinct < self.nt else 1.0
        return self._mass[q] * scale

    @property
    def cells(self) -> int:
        return self.d.ni * self.d.nj * self.d.nk

    def water_fraction(self) -> float:
        return float(self.d.water_mask().sum()) / self.cells


def mem_available_gb() -> float:
    try:
        for line in Path("/proc/meminfo").read_text().splitlines():
            if line.startswith("MemAvailable:"):
                return int(line.split()[1]) / 2**20
    except Exception:
        pass
    return 0.0


def make_cases(name: str):
    from mohid_gb300 import configs
    if name == "cfg4":
        return [Case(w) for w in configs.cfg4_members()]
    if name == "cfg5":
        # about 62 GB of FP64/int32 hydrodynamics plus 4 distinct tracer and 4
        # reference fields (4.3 GB each) and transient copies on the host
        need = 160.0
        have = mem_available_gb()
        if have < need:
            raise SystemExit(f"cfg5 needs about {need:.0f} GB of free host memory, {have:.0f} GB available")
        return [Case(configs.cfg5(), distinct_tracers=4)]
    return [Case({"cfg2": configs.cfg2, "cfg3": configs.cfg3}[name]())]


# ----------------------------------------------------------------------------- CPU baseline
def oracle_cases(cases):
    """The oracle's sample of a workload: the workload itself, or for the
    500 M-cell grid (whose FP64 work arrays alone take ~70 GB) a 1024x1024 cut
    of it with the same layers, options and tracer kinds."""
    if sum(c.cells for c in cases) <= 2.5e8:
        return cases
    return [Case(cases[0].w.scaled(ni=1024, nj=1024), distinct_tracers=1)]


def cpu_baseline(cases, budget_s: float = 12.0, nthreads: int = 0):
    """The oracle (FP64 restatement of the reference CPU path, OpenMP) on a bounded
    sample: whole steps of one tracer on each domain in turn, until `budget_s` is spent."""
    from oracle import oracle as O
    cores = nthreads or os.cpu_count() or 1
    work = [(c, c.tracer(0).copy(), O.params(**c.w.params()), O.Work(c.d)) for c in cases]
    for c, P, p, wk in work[:1]:
        O.step(c.d, P, p, ReferenceProp=c.ref(0), work=wk, nthreads=cores)   # first touch
    n = cells = 0
    t0 = time.perf_counter()
    while True:
        for c, P, p, wk in work:
            assert O.step(c.d, P, p, ReferenceProp=c.ref(0), work=wk, nthreads=cores) == 0
            cells += c.cells
            if time.perf_counter() - t0 >= budget_s:
                break
        n += 1
        el = time.perf_counter() - t0
        if el >= budget_s or n >= 50:
            break
    dims = f"{cases[0].d.ni}x{cases[0].d.nj}x{cases[0].d.nk}" if len(cases) == 1 else f"{len(cases)} domains"
    return {"value": cells / el, "unit": "cell-tracer-updates/s", "cores": cores, "kind": "port",
            "sample": f"oracle steps of 1 tracer over {cells / 1e6:.1f} M cells of the {dims} workload "
                      f"({el:.1f} s, OpenMP, {cores} threads)"}


# ----------------------------------------------------------------------------- GPU: plain FP64
def run_plain(case, steps, warmup, world, ntracers=None):
    """Plain FP64 drop-in: one device-resident launch per tracer per step."""
    import torch
    from mohid_gb300 import advdiff
    from mohid_gb300.synth import F3, I3, Domain

    d = case.d
    nt = ntracers or case.nt
    ad = advdiff.AdvectionDiffusion(d)
    ad.set_hydro()
    p = advdiff.params(**case.w.params())
    bufs = [(torch.from_numpy(case.tracer(t)).cuda(), None) for t in range(nt)]
    bufs = [(a, torch.empty_like(a)) for a, _ in bufs]
    refs = [torch.from_numpy(case.ref(t)).cuda() if case.refs is not None else None for t in range(nt)]
    stream = torch.cuda.ExternalStream(ad.stream)

    def one_step():
        for t in range(nt):
            a, b = bufs[t]
            ad.step_device(a, b, p, refs[t])
            bufs[t] = (b, a)

    for _ in range(warmup):
        one_step()
    ad.sync()
    torch.cuda.synchronize()
    barrier(world)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        one_step()
    e1.record(stream)
    e1.synchronize()
    ad.sync()
    ms = e0.elapsed_time(e1) / steps
    barrier(world)
    ad.kill()
    return dict(ms=ms, kernel_ms=ms / nt, nt=nt, cells=case.cells)


def plain_e2e(case, steps, world):
    """Plain FP64 through the host-pointer C-ABI: set_hydro + one call per tracer per step."""
    import torch
    from mohid_gb300 import advdiff
    from mohid_gb300.synth import F3, I3, Domain
    d = case.d
    ad = advdiff.AdvectionDiffusion(d)
    p = advdiff.params(**case.w.params())
    pinned = {n: torch.from_numpy(d.arrays[n]).pin_memory().numpy() for n in d.arrays}
    dp = Domain(spec=d.spec, arrays=pinned)
    host = [torch.from_numpy(case.tracer(t)).pin_memory().numpy() for t in range(case.nt)]
    ad.set_hydro(dp)
    for t in range(case.nt):
        ad.step(host[t], p, case.ref(t))
    torch.cuda.synchronize()
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(steps):
        ad.set_hydro(dp)
        for t in range(case.nt):
            ad.step(host[t], p, case.ref(t))
    e2e_s = (time.perf_counter() - t0) / steps
    h2d = sum(pinned[n].nbytes for n in F3 + I3) + case.nt * host[0].nbytes
    ad.kill()
    return e2e_s, h2d, case.nt * host[0].nbytes


# ----------------------------------------------------------------------------- GPU: batched FP32
def load_batch(case, storage):
    from mohid_gb300 import advdiff, batched
    ad = advdiff.AdvectionDiffusion(case.d)
    ad.set_hydro()
    b = batched.Batch(ad, case.nt, storage)
    for t in range(case.nt):
        b.set_tracer(t, case.tracer(t))
        if case.refs is not None:
            b.set_reference(t, case.ref(t))
    return ad, b


def time_steps(step, stream, steps, world):
    """K steps between CUDA events on `stream`, clocks sampled meanwhile."""
    import torch
    torch.cuda.synchronize()
    barrier(world)
    clk = ClockSampler(torch.cuda.current_device())
    clk.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    clk.mark_start()
    e0.record(stream)
    step(steps)
    e1.record(stream)
    e1.synchronize()
    clk.mark_end()
    clocks = clk.stop()
    barrier(world)
    return e0.elapsed_time(e1) / steps, clocks


def tracer_groups(nt: int, split: int) -> list:
    """Tracers per step-kernel launch: groups of `split` (8, 4 or 2), then 4, 2, 1."""
    out, left = [], nt
    while left > 0:
        g = 8 if left >= 8 and split >= 8 else 4 if left >= 4 and split >= 4 else 2 if left >= 2 else 1
        out.append(g)
        left -= g
    return out


def mass_defects(objs, cases):
    """Per tracer |mass now - mass loaded - boundary flux since| / mass loaded:
    the FP64 budget of the batched form (NaN where the mass fixer did not run)."""
    out = []
    for (_, b), c in zip(objs, cases):
        for t in range(c.nt):
            m0 = c.load_mass(t)
            out.append(abs(b.mass(t) - m0 - b.boundary_flux(t)) / abs(m0))
    return out


def run_batched(cases, storage, steps, warmup, world, e2e=True):
    import torch
    from mohid_gb300 import advdiff, batched
    from mohid_gb300.synth import Domain, F3, I3

    ensemble = len(cases) > 1
    free, total = torch.cuda.mem_get_info()
    # per cell: the FP64 hydrodynamics and masks, the packed fields, two FP32
    # tracer buffers and the G scratch of the largest tracer group (the open
    # boundaries' references are kept for the boundary columns only)
    nt0 = cases[0].nt
    need = sum(c.cells for c in cases) * (120 + 8 * nt0 + 4 * min(nt0, 10))
    if need > 0.9 * free:
        raise SystemExit(f"the workload needs about {need / 2**30:.0f} GiB of device memory, {free / 2**30:.0f} free")
    objs = [load_batch(c, storage) for c in cases]
    pars = [advdiff.params(**c.w.params()) for c in cases]
    if ensemble:
        ens = batched.Ensemble([b for _, b in objs])
        stepper = lambda n, graph: ens.step(pars, nsteps=n, graph=graph)
    else:
        b0 = objs[0][1]
        stepper = lambda n, graph: b0.step(pars[0], nsteps=n, graph=graph)
    stepper(warmup, False)
    stepper(steps, True)                       # capture the graph outside the timed region
    if steps % 2:
        stepper(1, False)                      # back to the parity the graph was captured at
    for _, b in objs:
        b.sync()
    stream = torch.cuda.ExternalStream(objs[0][0].stream)
    ms, clocks = time_steps(lambda n: stepper(n, True), stream, steps, world)
    for _, b in objs:
        b.sync()
    nt = cases[0].nt
    defects = mass_defects(objs, cases)
    if ensemble:
        # per step one ensemble launch, with open members their boundary flux
        # and the mass fixer's finish; on closed members the finish runs once
        # after the timed call's last step (every ensemble workload here has
        # static volumes)
        nopen = sum(1 for c in cases if c.refs is not None)
        per = 1 + nopen + (1 if nopen else 0)
        per_call = 0 if nopen else 1
        launches = steps * per + per_call
        sched = {"launches": per, "per_call": per_call, "sched": "persistent tile list (ensemble)", "split": nt}
        groups = [min(nt, 4)]
    else:
        sched = objs[0][1].schedule()              # as chosen by the autotuner
        launches = steps * sched["launches"] + sched["per_call"]   # one timed call
        groups = tracer_groups(nt, sched["split"])

    hydro = None
    if not ensemble:
        # a coupled time loop hands over a new hydrodynamic state every step:
        # device-resident FP64 fields (the masks kept), the batched repack and
        # the step, timed on the wall clock over the whole loop
        ad0 = objs[0][0]
        dev = {n: torch.from_numpy(cases[0].d.arrays[n]).cuda() for n in F3}
        hsteps = max(3, min(steps, 20))

        def hydro_step():
            ad0.set_fields(dev, bind=True)         # borrowed in place, a new state each call
            stepper(1, False)
        hydro_step()
        hydro_step()
        objs[0][1].sync()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(hsteps):
            hydro_step()
        objs[0][1].sync()
        torch.cuda.synchronize()
        hms = (time.perf_counter() - t0) / hsteps * 1e3
        hydro = {"ms_per_step": hms, "step_ms": ms, "update_ms": hms - ms, "steps": hsteps,
                 "value": cases[0].cells * cases[0].nt / (hms / 1e3),
                 "definition": "every step: mohid_ad_bind_hydro_dev of the 11 FP64 fields in device "
                               "memory (borrowed in place, masks kept), the batched repack and one "
                               "step; wall clock"}
        ad0.set_fields(dev, device=True)           # back to the instance's own copies
        del dev

    e2e_s = h2d = d2h = None
    if e2e:
        # a host-resident caller sends the step's hydrodynamics and tracers,
        # runs the step through the C-ABI and reads the tracers back, every step
        hosts = []
        for (ad, b), c in zip(objs, cases):
            pinned = {n: torch.from_numpy(c.d.arrays[n]).pin_memory().numpy() for n in c.d.arrays}
            hosts.append((Domain(spec=c.d.spec, arrays=pinned),
                          [torch.from_numpy(c.tracer(t)).pin_memory().numpy() for t in range(c.nt)]))

        def e2e_step(masks=False):
            # the step's FP64 hydrodynamic fields and tracers from pinned host
            # memory; the masks, which only wetting and drying change, once
            for (ad, b), (dp, host) in zip(objs, hosts):
                if masks:
                    ad.set_hydro(dp)
                else:
                    ad.set_fields({n: dp.arrays[n] for n in F3})
                for t in range(len(host)):
                    b.set_tracer(t, host[t])
            stepper(1, False)
            for (ad, b), (dp, host) in zip(objs, hosts):
                for t in range(len(host)):
                    b.get_tracer(t, host[t])
        e2e_step(masks=True)
        torch.cuda.synchronize()
        barrier(world)
        e2e_steps = max(3, min(steps, 10))
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            e2e_step()
        e2e_s = (time.perf_counter() - t0) / e2e_steps
        h2d = sum(sum(dp.arrays[n].nbytes for n in F3) + sum(h.nbytes for h in host) for dp, host in hosts)
        d2h = sum(sum(h.nbytes for h in host) for _, host in hosts)
    if ensemble:
        ens.destroy()
    for ad, b in objs:
        b.destroy()
        ad.kill()
    cells = sum(c.cells for c in cases)
    # step-kernel launches per step (the fixer's and boundary flux's launches
    # excluded; their time stays in ms)
    g = len(groups)
    return dict(ms=ms, kernel_ms=ms / g, launches=launches, e2e_s=e2e_s, h2d=h2d, d2h=d2h, cells=cells, sched=sched,
                nt=nt, bytes_per_update=8.0 + SHARED_BYTES[storage] / nt,
                bytes_per_launch=cells * (8.0 * nt + SHARED_BYTES[storage]) / g, dtype="f32", clocks=clocks,
                kernel=("ensemble_kernel" if ensemble else "batched_kernel") + f"<{max(groups)}>",
                mass_defects=defects, hydro=hydro)


# ----------------------------------------------------------------------------- main
def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--form", default="batched", choices=["batched", "plain"])
    ap.add_argument("--workload", default="cfg2", choices=sorted(WORKLOADS))
    ap.add_argument("--cpu-budget", type=float, default=12.0)
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer leg (large workloads)")
    args = ap.parse_args()
    world, rank, local = dist_setup()
    if args.warmup < 3 and args.impl != "reference":
        args.warmup = 3

    from mohid_gb300 import build as B
    B.build()
    desc, storage = WORKLOADS[args.workload]
    workload_name = f"{args.workload}: {desc}"
    cases = make_cases(args.workload)
    cells = sum(c.cells for c in cases)
    nt = cases[0].nt
    unit = "cell-tracer-updates/s"
    metric = "cell-tracer-updates/s, FP32 batched vs FP64 plain on 1 GB300 at ≤1e-5 rel L2; HBM GB/s"
    water = sum(c.water_fraction() * c.cells for c in cases) / cells

    if args.impl == "reference":
        if rank != 0:
            return
        from oracle import oracle as O
        cores = os.cpu_count() or 1
        cases = oracle_cases(cases)
        cells = sum(c.cells for c in cases)
        for c in cases[:1]:
            P = c.tracer(0).copy()
            for _ in range(args.warmup):
                O.step(c.d, P, O.params(**c.w.params()), ReferenceProp=c.ref(0), work=O.Work(c.d),
                       nthreads=cores)
        # each step: one oracle step of every tracer of every domain, bounded to a
        # sample of the tracers on the large workloads (the metric is per update)
        budget_tracers = max(1, int(2e8 // max(cells, 1)))
        ntr = min(nt, budget_tracers)
        work = [(c, [c.tracer(t).copy() for t in range(ntr)], O.params(**c.w.params()), O.Work(c.d)) for c in cases]
        t0 = time.perf_counter()
        upd = 0
        for _ in range(args.steps):
            for c, Ps, p, wk in work:
                for t, P in enumerate(Ps):
                    assert O.step(c.d, P, p, ReferenceProp=c.ref(t), work=wk, nthreads=cores) == 0
                    upd += c.cells
        el = time.perf_counter() - t0
        value = upd / el
        line = {"impl": "reference", "metric": metric, "value": value, "unit": unit,
                "n_gpus": 0, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": el / args.steps * 1e3, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
                "config": {"workload": workload_name, "form": "reference CPU path (FP64 restatement, "
                           "OpenMP, full-array passes as ModuleAdvectionDiffusion)",
                           "water_fraction": water},
                "cpu_baseline": {"value": value, "unit": unit, "cores": cores, "kind": "port",
                                 "sample": f"{args.steps} full steps x {ntr} of {nt} tracers x {len(cases)} domain(s)"},
                "e2e": {"value": value, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    import torch
    plain = None
    if args.form == "batched":
        r = run_batched(cases, storage, args.steps, args.warmup, world, e2e=not args.no_e2e)
        # plain FP64 on the same workload: every tracer of every domain, one launch each
        # (the largest workloads time a subset of tracers; the rate is per update)
        psteps = max(1, min(3, args.steps // 4))
        pr = [run_plain(c, psteps, 1, world, ntracers=min(c.nt, max(1, int(4e8 // c.cells))))
              for c in cases]
        p_ms = sum(x["ms"] * (c.nt / x["nt"]) for x, c in zip(pr, cases))
        # one tracer over every domain: the time of one launch per domain
        plain = dict(ms=p_ms, kernel_ms=sum(x["kernel_ms"] for x in pr), nt=nt,
                     launches=sum(c.nt for c in cases))
    else:
        if len(cases) > 1:
            raise SystemExit("--form plain runs single-domain workloads")
        pr = run_plain(cases[0], args.steps, args.warmup, world)
        e2e_s, h2d, d2h = plain_e2e(cases[0], max(3, min(args.steps, 10)), world)
        r = dict(ms=pr["ms"], kernel_ms=pr["kernel_ms"], launches=args.steps * nt, e2e_s=e2e_s, h2d=h2d,
                 d2h=d2h, cells=cells, nt=nt, bytes_per_update=96.0, bytes_per_launch=96.0 * cells,
                 dtype="f64", clocks=None, kernel="plain_f64_kernel")
    ms = max_over_ranks(r["ms"], world)
    value = world * cells * r["nt"] / (ms / 1e3)
    e2e = None
    if r["e2e_s"] is not None:
        e2e_s = max_over_ranks(r["e2e_s"], world)
        e2e = {"value": world * cells * r["nt"] / e2e_s, "unit": unit, "h2d_bytes_per_step": r["h2d"],
               "d2h_bytes_per_step": r["d2h"]}
    peak, peak_kind = load_peaks()
    achieved = r["bytes_per_launch"] / (r["kernel_ms"] / 1e3) / 1e9
    traffic = TRAFFIC.get((args.workload, r["kernel"]))
    if rank != 0:
        return
    cpu = cpu_baseline(oracle_cases(cases), budget_s=args.cpu_budget)
    resident = sum(sum(a.nbytes for a in c.d.arrays.values()) for c in cases)
    line = {
        "metric": metric, "value": value, "unit": unit, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": r["dtype"],
        "data": "synthetic (seeded generator restating MOHID geometry/mask/continuity rules)",
        "config": {"workload": workload_name, "form": args.form,
                   "time_loop": "CUDA graph of K steps" if args.form == "batched" else "stream launches",
                   "cells": cells, "tracers": nt, "domains": len(cases), "water_fraction": water,
                   "schedule": r.get("sched"),
                   "l2": f"inputs larger than L2 ({resident / 2**30:.2f} GiB of FP64 hydrodynamics, "
                         f"the packed fields and tracers > 129 MiB)",
                   "parallelism": f"replicas x{world}" if world > 1 else "single GPU"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "traffic_unit": "bytes per launch (committed ncu capture)",
                     "kernel": r["kernel"], "bytes_per_launch": r["bytes_per_launch"],
                     "bytes_per_update": r["bytes_per_update"],
                     "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
                     else "fallback 6.8 TB/s"},
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": r["launches"],
        "clocks": r["clocks"],
    }
    if r.get("hydro"):
        line["hydro_update"] = r["hydro"]
    if r.get("mass_defects"):
        md = r["mass_defects"]
        line["mass_defect"] = {
            "max": None if any(math.isnan(x) for x in md) else max(md), "tracers": len(md),
            "definition": "per tracer |mass now - mass loaded - open-boundary flux since| / mass loaded after "
                          "the warm-up and timed steps; mass = FP64 sum of VolumeZ * value over water cells"}
    if plain is not None:
        pv = world * cells * plain["nt"] / (max_over_ranks(plain["ms"], world) / 1e3)
        line["plain_f64"] = {"value": pv, "unit": unit, "ms_per_step": plain["ms"],
                             "launches_per_step": plain["launches"],
                             "speedup_batched_over_plain": value / pv,
                             "roofline_frac": 96.0 * cells / (plain["kernel_ms"] / 1e3) / 1e9 / peak}
    print(json.dumps(line))


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per launch of the
# dominant kernel, from one ncu capture of the workload's step launch (the
# one-CTA-per-tile schedule the autotuner picks, no mass-fixer sums): not
# measured by this run; the capture and its command are in
# profiles/batched_kernel_512x512x40_2tracers.md.
TRAFFIC: dict = {
    ("cfg2", "batched_kernel<2>"): 623.833856e6 + 113.142528e6,
}

if __name__ == "__main__":
    main()
