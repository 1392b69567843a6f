"""Host-side mirror of MOHID's transport interface, on the GB300 C-ABI.

    StartAdvectionDiffusion   ModuleAdvectionDiffusion.F90:400    -> AdvectionDiffusion(domain)
    AdvectionDiffusion(...)   ModuleAdvectionDiffusion.F90:1108   -> .step(PROP, params, ReferenceProp)
    KillAdvectionDiffusion    ModuleAdvectionDiffusion.F90:5849   -> .kill()

Argument names and meanings are the reference's; option errors that make the
reference `stop` raise MohidAdError(ERR_OPTION) instead.  Every call runs the
CUDA kernels of libmohid_ad.so; there is no CPU path.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from .synth import Domain, F3, I3


def params(**over) -> N.MohidAdParams:
    """mohid_ad_params with the reference's defaults, then `over` applied."""
    p = N.MohidAdParams()
    N.ad_lib().mohid_ad_default_params(C.byref(p))
    names = {f[0] for f in N.MohidAdParams._fields_}
    for k, v in over.items():
        if k not in names:
            raise KeyError(f"unknown AdvectionDiffusion parameter {k!r}")
        setattr(p, k, v)
    return p


def _size(ni, nj, nk):
    work = N.T_Size3D(1, ni, 1, nj, 1, nk)
    size = N.T_Size3D(0, ni + 1, 0, nj + 1, 0, nk + 1)
    return size, work


class AdvectionDiffusion:
    """One transport instance on the current CUDA device (one grid)."""

    def __init__(self, domain: Domain):
        self.lib = N.ad_lib()
        self.domain = domain
        size, work = _size(domain.ni, domain.nj, domain.nk)
        self._id = C.c_int(0)
        st = C.c_int(0)
        d = domain.arrays
        rc = self.lib.mohid_ad_init(C.byref(self._id), C.byref(size), C.byref(work),
                                    N.ptr(d["DUX"]), N.ptr(d["DVY"]), N.ptr(d["DZX"]),
                                    N.ptr(d["DZY"]), N.iptr(d["KFloorZ"]),
                                    N.iptr(d["BoundaryPoints2D"]), C.byref(st))
        N.check(rc, "mohid_ad_init")
        self._hydro_args = None

    @property
    def id(self) -> int:
        return self._id.value

    def set_hydro(self, domain: Domain | None = None, SmallDepths: np.ndarray | None = None):
        d = (domain or self.domain).arrays
        args = [N.ptr(d[n]) for n in F3] + [N.iptr(d[n]) for n in I3]
        st = C.c_int(0)
        rc = self.lib.mohid_ad_set_hydro(C.byref(self._id), *args,
                                         N.iptr(SmallDepths) if SmallDepths is not None else None,
                                         C.byref(st))
        N.check(rc, "mohid_ad_set_hydro")

    def set_hydro_device(self, t: dict, SmallDepths=None):
        """Hydrodynamics already on the GPU: `t` maps field names to device tensors."""
        args = [C.c_void_p(t[n].data_ptr()) for n in F3] + [C.c_void_p(t[n].data_ptr()) for n in I3]
        st = C.c_int(0)
        rc = self.lib.mohid_ad_set_hydro_dev(
            C.byref(self._id), *[C.cast(a, N.c_double_p) for a in args[:11]],
            *[C.cast(a, N.c_int_p) for a in args[11:]],
            C.cast(C.c_void_p(SmallDepths.data_ptr()), N.c_int_p) if SmallDepths is not None else None,
            C.byref(st))
        N.check(rc, "mohid_ad_set_hydro_dev")

    def set_fields(self, fields: dict, device: bool = False, bind: bool = False):
        """Update some FP64 hydrodynamic fields and keep the rest and the masks
        (mohid_ad_set_hydro[_dev] with NULL for what is kept).  `fields` maps F3
        names to float64 Size-box numpy arrays, or torch CUDA tensors when device.
        bind (device tensors): borrow them in place instead of copying
        (mohid_ad_bind_hydro_dev); the tensors must outlive their use."""
        if device or bind:
            args = [C.cast(C.c_void_p(fields[n].data_ptr()), N.c_double_p) if n in fields else None for n in F3]
        else:
            args = [N.ptr(fields[n]) if n in fields else None for n in F3]
        st = C.c_int(0)
        fn = "mohid_ad_bind_hydro_dev" if bind else ("mohid_ad_set_hydro_dev" if device else "mohid_ad_set_hydro")
        rc = getattr(self.lib, fn)(C.byref(self._id), *args, *([None] * len(I3)), None, C.byref(st))
        N.check(rc, fn)
        if bind:
            self._bound = dict(getattr(self, "_bound", {}), **fields)   # keep the borrowed tensors alive

    def get_fields(self, names=F3) -> dict:
        """The instance's current FP64 hydrodynamic fields (mohid_ad_get_hydro) as numpy arrays."""
        out = {n: np.empty(self.domain.shape3) for n in names}
        args = [N.ptr(out[n]) if n in out else None for n in F3]
        st = C.c_int(0)
        N.check(self.lib.mohid_ad_get_hydro(C.byref(self._id), *args, C.byref(C.c_int(0)), C.byref(st)),
                "mohid_ad_get_hydro")
        return out

    def geometry(self, SZZ, DXX, DYY, faces_option: int = 3, store_old: bool = True):
        """Geometry of a new water level on the device (mohid_ad_geometry_dev): SZZ,
        DXX, DYY torch CUDA float64 tensors (Size box / 2-D Size box)."""
        st = C.c_int(0)
        rc = self.lib.mohid_ad_geometry_dev(C.byref(self._id), C.c_void_p(SZZ.data_ptr()),
                                            C.c_void_p(DXX.data_ptr()), C.c_void_p(DYY.data_ptr()),
                                            C.byref(C.c_int(int(faces_option))), C.byref(C.c_int(int(store_old))),
                                            C.byref(st))
        N.check(rc, "mohid_ad_geometry_dev")

    def vertical_flux(self, dt: float, var_grid: bool = True):
        """Vertical water flux from continuity on the device (mohid_ad_vertical_flux)."""
        st = C.c_int(0)
        rc = self.lib.mohid_ad_vertical_flux(C.byref(self._id), C.byref(C.c_double(dt)),
                                             C.byref(C.c_int(int(var_grid))), C.byref(st))
        N.check(rc, "mohid_ad_vertical_flux")

    def step(self, PROP: np.ndarray, p: N.MohidAdParams, ReferenceProp: np.ndarray | None = None):
        """AdvectionDiffusion for one property: PROP (float64, Size box) updated in place."""
        if PROP.dtype != np.float64 or not PROP.flags.c_contiguous or PROP.shape != self.domain.shape3:
            raise ValueError("PROP must be a C-contiguous float64 array of the Size box")
        st = C.c_int(0)
        rc = self.lib.mohid_ad_step_prop_f64(C.byref(self._id), N.ptr(PROP), N.ptr(ReferenceProp),
                                             C.byref(p), C.byref(st))
        N.check(rc, "mohid_ad_step_prop_f64")

    def step_device(self, Pin, Pout, p: N.MohidAdParams, Ref=None):
        """Device-resident step (torch CUDA float64 tensors); asynchronous on .stream."""
        st = C.c_int(0)
        rc = self.lib.mohid_ad_step_prop_f64_dev(
            C.byref(self._id), C.c_void_p(Pin.data_ptr()), C.c_void_p(Pout.data_ptr()),
            C.c_void_p(Ref.data_ptr()) if Ref is not None else None, C.byref(p), C.byref(st))
        N.check(rc, "mohid_ad_step_prop_f64_dev")

    def set_discharges(self, disch: dict | None):
        """SetDischarges (mohid_ad_set_discharges) from numpy arrays: nCells, ignore,
        bypass, vert per discharge; I, J, K, Kmin, Kmax, Flow, Conc, ConcMF per
        discharge cell.  None: UnSetDischarges."""
        st = C.c_int(0)
        if disch is None:
            N.check(self.lib.mohid_ad_unset_discharges(C.byref(self._id), C.byref(st)), "mohid_ad_unset_discharges")
            return
        ints = [np.ascontiguousarray(disch[n], dtype=np.int32)
                for n in ("nCells", "ignore", "bypass", "vert", "I", "J", "K", "Kmin", "Kmax")]
        dbls = [np.ascontiguousarray(disch[n], dtype=np.float64) for n in ("Flow", "Conc", "ConcMF")]
        rc = self.lib.mohid_ad_set_discharges(C.byref(self._id), C.byref(C.c_int(len(ints[0]))),
                                              *(a.ctypes.data_as(C.c_void_p) for a in ints + dbls), C.byref(st))
        N.check(rc, "mohid_ad_set_discharges")

    def set_noflux(self, masks):
        """NoFluxU/V/W masks (int32 Size-box arrays) for NoAdvFlux / NoDifFlux, or None to clear."""
        st = C.c_int(0)
        if masks is None:
            rc = self.lib.mohid_ad_set_noflux(C.byref(self._id), None, None, None, C.byref(st))
        else:
            ms = [np.ascontiguousarray(m, dtype=np.int32) for m in masks]
            rc = self.lib.mohid_ad_set_noflux(C.byref(self._id), *(m.ctypes.data_as(C.c_void_p) for m in ms),
                                              C.byref(st))
        N.check(rc, "mohid_ad_set_noflux")

    def set_prop_old(self, PropOld, device: bool = False):
        """The PropOld array that steps with Orlanski boundaries write (the field as
        OpenBoundaryCondition saw it): a float64 Size-box numpy array, or a device
        tensor / pointer with device=True; kept by reference (None detaches)."""
        st = C.c_int(0)
        if PropOld is None:
            ptr_, self._prop_old = None, None
        elif device:
            ptr_ = C.c_void_p(PropOld.data_ptr() if hasattr(PropOld, "data_ptr") else int(PropOld))
            self._prop_old = PropOld
        else:
            assert PropOld.dtype == np.float64 and PropOld.flags.c_contiguous and PropOld.shape == self.domain.shape3
            ptr_, self._prop_old = PropOld.ctypes.data_as(C.c_void_p), PropOld
        rc = self.lib.mohid_ad_set_prop_old(C.byref(self._id), ptr_, C.byref(C.c_int(1 if device else 0)),
                                            C.byref(st))
        N.check(rc, "mohid_ad_set_prop_old")

    def cell_fluxes(self) -> dict:
        """The face fluxes of the last step (made with CellFluxes=1): AdvFluxX/Y/Z,
        DifFluxX/Y/Z as Size-box float64 arrays (mohid_ad_get_adv_flux / _dif_flux)."""
        out = {n: np.empty(self.domain.shape3) for n in ("AdvFluxX", "AdvFluxY", "AdvFluxZ", "DifFluxX",
                                                          "DifFluxY", "DifFluxZ")}
        st = C.c_int(0)
        host = C.c_int(0)
        for fn, names in (("mohid_ad_get_adv_flux", ("AdvFluxX", "AdvFluxY", "AdvFluxZ")),
                          ("mohid_ad_get_dif_flux", ("DifFluxX", "DifFluxY", "DifFluxZ"))):
            rc = getattr(self.lib, fn)(C.byref(self._id), *(out[n].ctypes.data_as(C.c_void_p) for n in names),
                                       C.byref(host), C.byref(st))
            N.check(rc, fn)
        return out

    @property
    def stream(self) -> int:
        return self.lib.mohid_ad_stream(C.byref(self._id)) or 0

    def sync(self):
        st = C.c_int(0)
        N.check(self.lib.mohid_ad_sync(C.byref(self._id), C.byref(st)), "mohid_ad_sync")

    def kill(self):
        if self._id.value:
            st = C.c_int(0)
            N.check(self.lib.mohid_ad_kill(C.byref(self._id), C.byref(st)), "mohid_ad_kill")

    def __del__(self):
        try:
            self.kill()
        except Exception:
            pass


def thomasz(D, E, F, TI, RES, WaterPoints):
    """THOMASZ_NewType2 on the GPU (replaces SolveThomas_C dim=2); RES updated in place."""
    nk, nj, ni = (s - 2 for s in D.shape)
    size = N.T_Size3D(0, ni + 1, 0, nj + 1, 0, nk + 1)
    b = [C.c_int(v) for v in (1, ni, 1, nj, 1, nk)]
    st = C.c_int(0)
    rc = N.ad_lib().mohid_thomasz_f64(*[C.byref(x) for x in b], C.byref(size), N.ptr(D), N.ptr(E),
                                      N.ptr(F), N.ptr(TI), N.ptr(RES), N.iptr(WaterPoints),
                                      C.byref(st))
    N.check(rc, "mohid_thomasz_f64")
