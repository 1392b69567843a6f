"""Seeded synthetic MOHID domains (numpy views over the native generator).

A `Domain` holds every array AdvectionDiffusion receives, Fortran-ordered over
the Size box: a 3-D field is a numpy array of shape (nk+2, nj+2, ni+2) in C
order, which is the Fortran (0:ni+1, 0:nj+1, 0:nk+1) layout byte for byte.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _native as N

F3 = ("Wflux_X", "Wflux_Y", "Wflux_Z", "VolumeZOld", "VolumeZ", "Visc_H", "Diff_V",
      "AreaU", "AreaV", "DZZ", "DWZ")
I3 = ("OpenPoints3D", "LandPoints3D", "WaterPoints3D", "ComputeFacesU3D", "ComputeFacesV3D",
      "ComputeFacesW3D")
F2 = ("DUX", "DVY", "DZX", "DZY", "depth")
I2 = ("KFloorZ", "BoundaryPoints2D", "WaterPoints2D")

# tracer kinds of mohid_synth_tracer
GAUSSIAN, TEMPERATURE, SALINITY, LOGNORMAL, CONSTANT = 0, 1, 2, 3, 4


@dataclass
class GenSpec:
    ni: int
    nj: int
    nk: int
    dx: float = 500.0
    dy: float = 500.0
    zlevel: bool = False
    hmin: float = 10.0
    hmax: float = 50.0
    bathy_kind: int = 0
    land_frac: float = 0.1
    land_kind: int = 0
    umax: float = 0.5
    visc_h: float = 10.0
    kz_median: float = 1e-4
    kz_logsigma: float = 1.0
    open_sides: int = 0
    vol_var: float = 0.0
    dt: float = 30.0
    seed: int = 1

    def cparams(self) -> N.SynthParams:
        return N.SynthParams(self.ni, self.nj, self.nk, self.dx, self.dy, int(self.zlevel),
                             self.hmin, self.hmax, self.bathy_kind, self.land_frac,
                             self.land_kind, self.umax, self.visc_h, self.kz_median,
                             self.kz_logsigma, self.open_sides, self.vol_var, self.dt,
                             self.seed & 0xFFFFFFFFFFFFFFFF)


@dataclass
class Domain:
    spec: GenSpec
    arrays: dict = field(default_factory=dict)

    @property
    def ni(self) -> int:
        return self.spec.ni

    @property
    def nj(self) -> int:
        return self.spec.nj

    @property
    def nk(self) -> int:
        return self.spec.nk

    @property
    def shape3(self) -> tuple:
        return (self.nk + 2, self.nj + 2, self.ni + 2)

    @property
    def shape2(self) -> tuple:
        return (self.nj + 2, self.ni + 2)

    def __getattr__(self, name):
        arrays = self.__dict__.get("arrays", {})
        if name in arrays:
            return arrays[name]
        raise AttributeError(name)

    def _cout(self) -> N.SynthOut:
        o = N.SynthOut()
        for n in F2 + F3:
            setattr(o, n, N.ptr(self.arrays[n]))
        for n in I2 + I3:
            setattr(o, n, N.iptr(self.arrays[n]))
        return o

    def new_field(self) -> np.ndarray:
        return np.zeros(self.shape3, dtype=np.float64)

    def tracer(self, kind: int, a: float, b: float, seed: int) -> np.ndarray:
        P = self.new_field()
        lib = N.synth_lib()
        cp = self.spec.cparams()
        co = self._cout()
        rc = lib.mohid_synth_tracer(C.byref(cp), C.byref(co), kind, a, b, seed, N.ptr(P))
        if rc != 0:
            raise RuntimeError(f"mohid_synth_tracer failed ({rc})")
        return P

    def reference(self, c0: float, rel: float, seed: int) -> np.ndarray:
        R = self.new_field()
        lib = N.synth_lib()
        cp = self.spec.cparams()
        co = self._cout()
        rc = lib.mohid_synth_reference(C.byref(cp), C.byref(co), c0, rel, seed, N.ptr(R))
        if rc != 0:
            raise RuntimeError(f"mohid_synth_reference failed ({rc})")
        return R

    def water_mask(self) -> np.ndarray:
        """Boolean mask of water cells of the work box (Size-box shaped)."""
        return self.arrays["WaterPoints3D"] == 1

    @property
    def n_work_cells(self) -> int:
        return self.ni * self.nj * self.nk


def generate(spec: GenSpec) -> Domain:
    d = Domain(spec=spec)
    for n in F3:
        d.arrays[n] = np.zeros(d.shape3, dtype=np.float64)
    for n in I3:
        d.arrays[n] = np.zeros(d.shape3, dtype=np.int32)
    for n in F2:
        d.arrays[n] = np.zeros(d.shape2, dtype=np.float64)
    for n in I2:
        d.arrays[n] = np.zeros(d.shape2, dtype=np.int32)
    lib = N.synth_lib()
    cp = spec.cparams()
    co = d._cout()
    rc = lib.mohid_synth_generate(C.byref(cp), C.byref(co))
    if rc != 0:
        raise RuntimeError(f"mohid_synth_generate failed ({rc})")
    return d
