"""Host mirror of the batched FP32 form (mohid_ad_batched_* in include/mohid_ad.h).

One Batch transports the tracers of one MOHID property group -- properties
that Advection_Diffusion_Processes would pass to AdvectionDiffusion one by one
with the same hydrodynamics and options (ModuleWaterProperties.F90:14603-14824)
-- in a single device-resident call per step.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from .advdiff import AdvectionDiffusion

FP32, FP16_Q, FP16_QK = 0, 1, 2


class Batch:
    def __init__(self, ad: AdvectionDiffusion, ntracers: int, storage: int = FP32):
        self.ad = ad
        self.lib = N.ad_lib()
        self.nt = ntracers
        self.storage = storage
        self._bid = C.c_int(0)
        st = C.c_int(0)
        rc = self.lib.mohid_ad_batched_create(C.byref(self._bid), C.byref(ad._id),
                                              C.byref(C.c_int(ntracers)), C.byref(C.c_int(storage)),
                                              C.byref(st))
        N.check(rc, "mohid_ad_batched_create")

    def pack_hydro(self):
        st = C.c_int(0)
        N.check(self.lib.mohid_ad_batched_pack_hydro(C.byref(self._bid), C.byref(st)),
                "mohid_ad_batched_pack_hydro")

    def set_tracer(self, t: int, P):
        """P: float64 Size-box numpy array (host) or torch CUDA tensor (device)."""
        dev, p = self._addr(P)
        st = C.c_int(0)
        rc = self.lib.mohid_ad_batched_set_tracer(C.byref(self._bid), C.byref(C.c_int(t)), p,
                                                  C.byref(C.c_int(dev)), C.byref(st))
        N.check(rc, "mohid_ad_batched_set_tracer")

    def get_tracer(self, t: int, out=None):
        if out is None:
            out = np.zeros(self.ad.domain.shape3, dtype=np.float64)
        dev, p = self._addr(out)
        st = C.c_int(0)
        rc = self.lib.mohid_ad_batched_get_tracer(C.byref(self._bid), C.byref(C.c_int(t)), p,
                                                  C.byref(C.c_int(dev)), C.byref(st))
        N.check(rc, "mohid_ad_batched_get_tracer")
        return out

    def set_reference(self, t: int, R):
        dev, p = self._addr(R)
        st = C.c_int(0)
        rc = self.lib.mohid_ad_batched_set_reference(C.byref(self._bid), C.byref(C.c_int(t)), p,
                                                     C.byref(C.c_int(dev)), C.byref(st))
        N.check(rc, "mohid_ad_batched_set_reference")

    def set_discharge_conc(self, t: int, conc):
        """DischConc of tracer t: one value per discharge cell of the plain
        instance's set_discharges, in its order (mohid_ad_batched_set_discharge_conc)."""
        c = np.ascontiguousarray(conc, dtype=np.float64)
        st = C.c_int(0)
        rc = self.lib.mohid_ad_batched_set_discharge_conc(C.byref(self._bid), C.byref(C.c_int(t)),
                                                          c.ctypes.data_as(C.c_void_p), C.byref(st))
        N.check(rc, "mohid_ad_batched_set_discharge_conc")

    def step(self, p: N.MohidAdParams, nsteps: int = 1, graph: bool = False):
        st = C.c_int(0)
        rc = self.lib.mohid_ad_batched_step(C.byref(self._bid), C.byref(p), C.byref(C.c_int(nsteps)),
                                            C.byref(C.c_int(int(graph))), C.byref(st))
        N.check(rc, "mohid_ad_batched_step")

    def autotune(self, p: N.MohidAdParams):
        """Time the launch schedules on this batch and keep the fastest (mohid_ad_batched_autotune)."""
        st = C.c_int(0)
        N.check(self.lib.mohid_ad_batched_autotune(C.byref(self._bid), C.byref(p), C.byref(st)),
                "mohid_ad_batched_autotune")

    def set_schedule(self, sched: int, split: int = 4, rows: int | None = None):
        """Fix the launch schedule by hand (0 one CTA per tile, 1 tile list; 10, 8, 4 or 2 tracers per
        launch; tiles of 8 or 4 rows, None keeps the height)."""
        st = C.c_int(0)
        r = C.byref(C.c_int(rows)) if rows is not None else None
        N.check(self.lib.mohid_ad_batched_set_schedule(C.byref(self._bid), C.byref(C.c_int(sched)),
                                                       C.byref(C.c_int(split)), r, C.byref(st)),
                "mohid_ad_batched_set_schedule")

    def schedule(self) -> dict:
        """{'launches': kernel launches per step, 'sched': 0 grid / 1 tile list, 'split': 10, 8, 4 or 2,
        'per_call': launches made once per step() call (the closed-domain mass fixer's finish),
        'rows': tile height (rows of 32 columns)}."""
        n, sc, sp, pc, ro, st = C.c_int(0), C.c_int(0), C.c_int(0), C.c_int(0), C.c_int(0), C.c_int(0)
        N.check(self.lib.mohid_ad_batched_schedule(C.byref(self._bid), C.byref(n), C.byref(sc), C.byref(sp),
                                                   C.byref(pc), C.byref(ro), C.byref(st)),
                "mohid_ad_batched_schedule")
        return {"launches": n.value, "sched": sc.value, "split": sp.value, "per_call": pc.value,
                "rows": ro.value}

    def set_mass_fix(self, on: bool):
        """Mass fixer on (default) or off (mohid_ad_batched_set_mass_fix)."""
        st = C.c_int(0)
        N.check(self.lib.mohid_ad_batched_set_mass_fix(C.byref(self._bid), C.byref(C.c_int(int(on))), C.byref(st)),
                "mohid_ad_batched_set_mass_fix")

    def cell_fluxes(self, t: int) -> dict:
        """The face fluxes of tracer t's last step (made with CellFluxes=1):
        AdvFluxX/Y/Z, DifFluxX/Y/Z as Size-box float64 arrays
        (mohid_ad_batched_get_adv_flux / _dif_flux)."""
        shape = self.ad.domain.shape3
        out = {n: np.empty(shape) for n in ("AdvFluxX", "AdvFluxY", "AdvFluxZ", "DifFluxX", "DifFluxY", "DifFluxZ")}
        st = C.c_int(0)
        for fn, names in (("mohid_ad_batched_get_adv_flux", ("AdvFluxX", "AdvFluxY", "AdvFluxZ")),
                          ("mohid_ad_batched_get_dif_flux", ("DifFluxX", "DifFluxY", "DifFluxZ"))):
            rc = getattr(self.lib, fn)(C.byref(self._bid), C.byref(C.c_int(t)),
                                       *(out[n].ctypes.data_as(C.c_void_p) for n in names),
                                       C.byref(C.c_int(0)), C.byref(st))
            N.check(rc, fn)
        return out

    def mass(self, t: int) -> float:
        m = C.c_double(0.0)
        st = C.c_int(0)
        rc = self.lib.mohid_ad_batched_mass(C.byref(self._bid), C.byref(C.c_int(t)), C.byref(m),
                                            C.byref(st))
        N.check(rc, "mohid_ad_batched_mass")
        return m.value

    def boundary_flux(self, t: int) -> float:
        """Mass that entered tracer t through open boundaries since it was
        loaded, as the mass fixer follows it (0 on closed domains, NaN once the
        fixer stopped for the tracer)."""
        m = C.c_double(0.0)
        st = C.c_int(0)
        rc = self.lib.mohid_ad_batched_boundary_flux(C.byref(self._bid), C.byref(C.c_int(t)), C.byref(m),
                                                     C.byref(st))
        N.check(rc, "mohid_ad_batched_boundary_flux")
        return m.value

    def sync(self):
        st = C.c_int(0)
        N.check(self.lib.mohid_ad_batched_sync(C.byref(self._bid), C.byref(st)), "mohid_ad_batched_sync")

    def destroy(self):
        if self._bid.value:
            st = C.c_int(0)
            N.check(self.lib.mohid_ad_batched_destroy(C.byref(self._bid), C.byref(st)),
                    "mohid_ad_batched_destroy")

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass

    @staticmethod
    def _addr(a):
        if isinstance(a, np.ndarray):
            if a.dtype != np.float64 or not a.flags.c_contiguous:
                raise ValueError("expected a C-contiguous float64 array")
            return 0, C.c_void_p(a.ctypes.data)
        return 1, C.c_void_p(a.data_ptr())          # torch CUDA tensor


class Ensemble:
    """Independent batched domains stepped together in one persistent launch
    (mohid_ad_ensemble_*).  Members keep their own grid, hydrodynamics, DT and
    tracers; they need the same tracer count (1, 2 or 4) and FP32 storage."""

    def __init__(self, members: list):
        self.members = list(members)
        self.lib = N.ad_lib()
        self._eid = C.c_int(0)
        ids = (C.c_int * len(self.members))(*[b._bid.value for b in self.members])
        st = C.c_int(0)
        rc = self.lib.mohid_ad_ensemble_create(C.byref(self._eid), C.byref(C.c_int(len(self.members))), ids,
                                               C.byref(st))
        N.check(rc, "mohid_ad_ensemble_create")

    def step(self, params: list, nsteps: int = 1, graph: bool = False):
        """params: one MohidAdParams per member."""
        if len(params) != len(self.members):
            raise ValueError("one parameter set per member")
        arr = (N.MohidAdParams * len(params))(*params)
        st = C.c_int(0)
        rc = self.lib.mohid_ad_ensemble_step(C.byref(self._eid), arr, C.byref(C.c_int(nsteps)),
                                             C.byref(C.c_int(int(graph))), C.byref(st))
        N.check(rc, "mohid_ad_ensemble_step")

    def sync(self):
        for b in self.members:
            b.sync()

    def destroy(self):
        if self._eid.value:
            st = C.c_int(0)
            N.check(self.lib.mohid_ad_ensemble_destroy(C.byref(self._eid), C.byref(st)),
                    "mohid_ad_ensemble_destroy")

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass
