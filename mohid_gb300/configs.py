"""The five workloads the transport step is measured and checked on.

Each is a seeded synthetic domain with the shapes, sizes and value
distributions of a MOHID Water tracer run (no public dataset is involved):

  cfg1  100x100x20 sigma, 10 % western coast, Upwind1, 1 Gaussian tracer, DT 30 s, 100 steps
  cfg2  512x512x40 sigma, bathymetry 5-200 m, P2_TVD SuperBee, T and S, DT 20 s, 1000 steps
  cfg3  2048x1024x50 z-level, 35 % fractal coast, columns of 1-50 layers, 8 tracers, DT 15 s, 500 steps
  cfg4  64 domains, 64x64x10 .. 512x256x40 log-uniform, 4 tracers each, DT 10-60 s, 200 steps
  cfg5  4096x4096x30 sigma, P2_TVD MinMod, 20 tracers, open W and E boundaries, DT 10 s, 100 steps
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field, replace

import numpy as np

from .synth import GenSpec, GAUSSIAN, TEMPERATURE, SALINITY, LOGNORMAL

UPWIND1, P2_TVD = 1, 4
MINMOD, SUPERBEE = 1, 4


@dataclass
class Workload:
    name: str
    spec: GenSpec
    steps: int
    method_h: int = UPWIND1
    limiter_h: int = SUPERBEE
    # (kind, a, b) per tracer
    tracers: list = field(default_factory=list)
    open_boundary: bool = False
    description: str = ""

    def params(self, **over) -> dict:
        p = dict(AdvMethodH=self.method_h, TVDLimitationH=self.limiter_h,
                 Upwind2H=int(self.method_h in (2, 3, 4)), DTProp=self.spec.dt,
                 SchmidtBackground_V=0.0, BoundaryCondition=1, DecayTime=0.0)
        p.update(over)
        return p

    def scaled(self, ni: int | None = None, nj: int | None = None, nk: int | None = None,
               steps: int | None = None) -> "Workload":
        """Same workload on a smaller grid (parity tests at sizes the oracle finishes fast)."""
        s = replace(self.spec, ni=ni or self.spec.ni, nj=nj or self.spec.nj, nk=nk or self.spec.nk)
        return replace(self, spec=s, steps=steps if steps is not None else self.steps)


def cfg1(seed: int = 1) -> Workload:
    return Workload(
        name="cfg1", steps=100, method_h=UPWIND1,
        spec=GenSpec(ni=100, nj=100, nk=20, dx=500.0, dy=500.0, hmin=10.0, hmax=50.0,
                     bathy_kind=0, land_frac=0.10, land_kind=0, umax=0.5, dt=30.0, seed=seed),
        tracers=[(GAUSSIAN, 1.0, 5.0)],
        description="100x100x20 sigma, Upwind1, 1 tracer, DT 30 s, 100 steps, closed")


def cfg2(seed: int = 2) -> Workload:
    return Workload(
        name="cfg2", steps=1000, method_h=P2_TVD, limiter_h=SUPERBEE,
        spec=GenSpec(ni=512, nj=512, nk=40, dx=500.0, dy=500.0, hmin=5.0, hmax=200.0,
                     bathy_kind=1, land_frac=0.08, land_kind=1, umax=1.0, dt=20.0, seed=seed),
        tracers=[(TEMPERATURE, 10.0, 25.0), (SALINITY, 30.0, 36.0)],
        description="512x512x40 sigma, P2_TVD SuperBee, T+S, DT 20 s, 1000 steps, closed")


def cfg3(seed: int = 3) -> Workload:
    return Workload(
        name="cfg3", steps=500, method_h=UPWIND1,
        spec=GenSpec(ni=2048, nj=1024, nk=50, dx=500.0, dy=500.0, zlevel=True, hmin=2.0,
                     hmax=500.0, bathy_kind=2, land_frac=0.35, land_kind=2, umax=0.5,
                     dt=15.0, seed=seed),
        tracers=[(TEMPERATURE, 4.0, 25.0), (SALINITY, 30.0, 36.0)] +
                [(LOGNORMAL, m, 0.5) for m in (5.0, 0.3, 1.0, 0.2, 50.0, 250.0)],
        description="2048x1024x50 z-level, 35% fractal coast, 8 tracers, DT 15 s, 500 steps")


def cfg4_members(seed: int = 4, n: int = 64) -> list:
    """64 ensemble members, sizes log-uniform between 64x64x10 and 512x256x40."""
    rng = np.random.default_rng(seed)
    out = []
    for m in range(n):
        t = rng.random()
        ni = int(round(math.exp(math.log(64) + t * (math.log(512) - math.log(64)))))
        nj = int(round(math.exp(math.log(64) + t * (math.log(256) - math.log(64)))))
        nk = int(round(math.exp(math.log(10) + t * (math.log(40) - math.log(10)))))
        dt = float(rng.uniform(10.0, 60.0))
        out.append(Workload(
            name=f"cfg4.{m}", steps=200, method_h=UPWIND1,
            spec=GenSpec(ni=ni, nj=nj, nk=nk, dx=500.0, dy=500.0, hmin=5.0, hmax=100.0,
                         bathy_kind=1, land_frac=0.1, land_kind=1, umax=0.5, dt=dt,
                         seed=seed * 1000 + m),
            tracers=[(TEMPERATURE, 8.0, 22.0), (SALINITY, 33.0, 36.0),
                     (LOGNORMAL, 1.0, 0.5), (LOGNORMAL, 0.1, 0.5)]))
    return out


def cfg5(seed: int = 5) -> Workload:
    return Workload(
        name="cfg5", steps=100, method_h=P2_TVD, limiter_h=MINMOD, open_boundary=True,
        spec=GenSpec(ni=4096, nj=4096, nk=30, dx=500.0, dy=500.0, hmin=10.0, hmax=150.0,
                     bathy_kind=1, land_frac=0.05, land_kind=1, umax=0.5, open_sides=3,
                     dt=10.0, seed=seed),
        tracers=[(LOGNORMAL, 1.0 + 0.1 * t, 0.4) for t in range(20)],
        description="4096x4096x30 sigma, P2_TVD MinMod, 20 tracers, open W/E, DT 10 s, 100 steps")


ALL = {"cfg1": cfg1, "cfg2": cfg2, "cfg3": cfg3, "cfg5": cfg5}
