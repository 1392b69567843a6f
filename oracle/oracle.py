"""TEST INFRASTRUCTURE ONLY: ctypes wrapper of the FP64 oracle (oracle/ad_oracle.c).

The oracle restates ModuleAdvectionDiffusion's AdvectionDiffusion call
(Software/MOHIDBase2/ModuleAdvectionDiffusion.F90:1108-1922) and THOMASZ_NewType2
(Software/MOHIDBase1/ModuleFunctions.F90:4026-4123) on the CPU.  Parity is
UNPINNED by the reference (no golden vectors for this path exist and its
Fortran cannot be compiled here); the restatement is cross-checked bit for bit
against oracle/ref_py.py and against analytic properties in tests/.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SO = HERE / "_build" / "liboracle.so"

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_fp = C.POINTER(C.c_float)


class OraDischarges(C.Structure):
    _fields_ = [("number", C.c_int)] + [(n, _ip) for n in ("nCells", "ignore", "bypass", "vert", "I", "J", "K",
                                                          "Kmin", "Kmax")] + \
        [(n, _dp) for n in ("Flow", "Conc", "ConcMF")]


DISCH_FIELDS_INT = ("nCells", "ignore", "bypass", "vert", "I", "J", "K", "Kmin", "Kmax")
DISCH_FIELDS_F64 = ("Flow", "Conc", "ConcMF")


def discharges_struct(disch: dict) -> OraDischarges:
    """SetDischarges arguments as numpy arrays: nCells, ignore, bypass, vert (per
    discharge), I, J, K, Kmin, Kmax, Flow, Conc, ConcMF (per discharge cell)."""
    q = OraDischarges()
    q.number = len(disch["nCells"])
    keep = {}
    for n in DISCH_FIELDS_INT:
        keep[n] = np.ascontiguousarray(disch[n], dtype=np.int32)
        setattr(q, n, _p(keep[n], _ip))
    for n in DISCH_FIELDS_F64:
        keep[n] = np.ascontiguousarray(disch[n], dtype=np.float64)
        setattr(q, n, _p(keep[n]))
    q._keep = keep
    return q


class OraDomain(C.Structure):
    _fields_ = [("ni", C.c_int), ("nj", C.c_int), ("nk", C.c_int)] + \
        [(n, _dp) for n in ("DUX", "DVY", "DZX", "DZY")] + \
        [(n, _ip) for n in ("KFloorZ", "BoundaryPoints2D")] + \
        [(n, _dp) for n in ("Wflux_X", "Wflux_Y", "Wflux_Z", "VolumeZOld", "VolumeZ", "Visc_H",
                            "Diff_V", "AreaU", "AreaV", "DZZ", "DWZ")] + \
        [(n, _ip) for n in ("OpenPoints3D", "LandPoints3D", "WaterPoints3D", "ComputeFacesU3D",
                            "ComputeFacesV3D", "ComputeFacesW3D", "SmallDepths", "NoFluxU", "NoFluxV",
                            "NoFluxW")] + [("Disch", C.POINTER(OraDischarges)), ("PROPOld", _dp)]


class Params(C.Structure):
    """Independent mirror of mohid_ad_params (include/mohid_ad.h)."""
    _fields_ = [
        ("schmidt_H", C.c_double), ("SchmidtCoef_V", C.c_double), ("SchmidtBackground_V", C.c_double),
        ("AdvMethodH", C.c_int), ("TVDLimitationH", C.c_int), ("AdvMethodV", C.c_int),
        ("TVDLimitationV", C.c_int), ("Upwind2H", C.c_int), ("Upwind2V", C.c_int),
        ("VolumeRelMax", C.c_double), ("DTProp", C.c_double), ("ImpExp_AdvV", C.c_double),
        ("ImpExp_DifV", C.c_double), ("ImpExp_AdvXX", C.c_double), ("ImpExp_AdvYY", C.c_double),
        ("ImpExp_DifH", C.c_double), ("NullDif", C.c_int), ("BoundaryCondition", C.c_int),
        ("DecayTime", C.c_double), ("AdvectionNudging", C.c_int), ("AdvectionNudgingCells", C.c_int),
        ("CellFluxes", C.c_int), ("NoAdvFlux", C.c_int), ("NoDifFlux", C.c_int),
        ("Optimize", C.c_int), ("FirstProperty", C.c_int), ("Vertical1D", C.c_int),
        ("XZFlow", C.c_int), ("Docycle_method", C.c_int),
    ]


DEFAULTS = dict(schmidt_H=1.0, SchmidtCoef_V=1.0, SchmidtBackground_V=1e-8, AdvMethodH=1,
                TVDLimitationH=4, AdvMethodV=1, TVDLimitationV=4, Upwind2H=0, Upwind2V=0,
                VolumeRelMax=1.5, DTProp=1.0, ImpExp_AdvV=1.0, ImpExp_DifV=1.0,
                ImpExp_AdvXX=0.0, ImpExp_AdvYY=0.0, ImpExp_DifH=0.0, NullDif=0,
                BoundaryCondition=1, DecayTime=0.0, AdvectionNudging=0, AdvectionNudgingCells=0,
                CellFluxes=0, NoAdvFlux=0, NoDifFlux=0, Optimize=0, FirstProperty=0,
                Vertical1D=0, XZFlow=0, Docycle_method=1)


def params(**over) -> Params:
    v = dict(DEFAULTS)
    for k in over:
        if k not in v:
            raise KeyError(k)
    v.update(over)
    return Params(**v)


_lib = None


def build() -> Path:
    r = subprocess.run(["make", "-s", "-C", str(HERE)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    return SO


def lib():
    global _lib
    if _lib is None:
        if not SO.exists():
            build()
        L = C.CDLL(str(SO))
        L.ora_step_f64.restype = C.c_int
        L.ora_step_f64.argtypes = [C.POINTER(OraDomain), _dp, _dp, C.POINTER(Params), C.c_void_p, C.c_int]
        L.ora_work_new.restype = C.c_void_p
        L.ora_work_new.argtypes = [C.c_int, C.c_int, C.c_int]
        L.ora_work_free.restype = None
        L.ora_work_free.argtypes = [C.c_void_p]
        L.ora_thomasz.restype = C.c_int
        L.ora_thomasz.argtypes = [C.c_int, C.c_int, C.c_int, _dp, _dp, _dp, _dp, _dp, _ip]
        L.ora_advection_face.restype = C.c_int
        L.ora_advection_face.argtypes = [_dp, _dp, _dp, C.c_double, C.c_double, C.c_double, C.c_int,
                                         C.c_int, C.c_int, C.c_int, _dp]
        L.ora_cell_flux.restype = _dp
        L.ora_cell_flux.argtypes = [C.c_void_p, C.c_int]
        L.ora_mass.restype = C.c_double
        L.ora_mass.argtypes = [C.POINTER(OraDomain), _dp]
        L.ora_mass_f32.restype = C.c_double
        L.ora_mass_f32.argtypes = [C.POINTER(OraDomain), _fp]
        L.ora_geometry.restype = None
        L.ora_geometry.argtypes = [C.c_int, C.c_int, C.c_int, _dp, _ip, _dp, _dp, _dp, _dp, C.c_int, C.c_int] + \
            [_dp] * 8
        L.ora_vertical_flux.restype = None
        L.ora_vertical_flux.argtypes = [C.c_int, C.c_int, C.c_int, _dp, _dp, _dp, _dp, _dp, _ip, _ip, _ip,
                                        C.c_double, C.c_int]
        _lib = L
    return _lib


def _p(a, t=_dp):
    return None if a is None else a.ctypes.data_as(t)


def cdomain(dom, SmallDepths=None, NoFlux=None, Disch=None, PropOld=None) -> OraDomain:
    a = dom.arrays
    d = OraDomain()
    d.ni, d.nj, d.nk = dom.ni, dom.nj, dom.nk
    for n in ("DUX", "DVY", "DZX", "DZY", "Wflux_X", "Wflux_Y", "Wflux_Z", "VolumeZOld", "VolumeZ",
              "Visc_H", "Diff_V", "AreaU", "AreaV", "DZZ", "DWZ"):
        setattr(d, n, _p(a[n]))
    for n in ("KFloorZ", "BoundaryPoints2D", "OpenPoints3D", "LandPoints3D", "WaterPoints3D",
              "ComputeFacesU3D", "ComputeFacesV3D", "ComputeFacesW3D"):
        setattr(d, n, _p(a[n], _ip))
    d.SmallDepths = _p(SmallDepths, _ip)
    nf = NoFlux if NoFlux is not None else (None, None, None)
    d.NoFluxU, d.NoFluxV, d.NoFluxW = (_p(m, _ip) for m in nf)
    q = discharges_struct(Disch) if Disch is not None else None
    d.Disch = C.pointer(q) if q is not None else None
    d.PROPOld = _p(PropOld)
    d._keep = (dom, SmallDepths, NoFlux, q, PropOld)
    return d


class Work:
    """Oracle work arrays that persist across calls (AllocateVariables, AD:537)."""

    def __init__(self, dom):
        self.ptr = lib().ora_work_new(dom.ni, dom.nj, dom.nk)
        if not self.ptr:
            raise MemoryError("oracle work allocation failed")

    def __del__(self):
        if getattr(self, "ptr", None):
            lib().ora_work_free(self.ptr)
            self.ptr = None


def step(dom, P: np.ndarray, p: Params, ReferenceProp=None, work: Work | None = None,
         nthreads: int = 0, SmallDepths=None, NoFlux=None, Disch=None, PropOld=None) -> int:
    """One FP64 oracle step of one property, in place.  Returns the status code.
    NoFlux: (NoFluxU, NoFluxV, NoFluxW) int32 Size-box masks, or None.
    PropOld: float64 Size-box array written with Orlanski boundaries, or None."""
    assert P.dtype == np.float64 and P.flags.c_contiguous and P.shape == dom.shape3
    if PropOld is not None:
        assert PropOld.dtype == np.float64 and PropOld.flags.c_contiguous and PropOld.shape == dom.shape3
    cd = cdomain(dom, SmallDepths, NoFlux, Disch, PropOld)
    return lib().ora_step_f64(C.byref(cd), _p(P), _p(ReferenceProp), C.byref(p),
                              work.ptr if work is not None else None, nthreads)


FLUX_NAMES = ("AdvFluxX", "AdvFluxY", "AdvFluxZ", "DifFluxX", "DifFluxY", "DifFluxZ")


def cell_fluxes(dom, work: Work) -> dict:
    """Copies of the face fluxes of the last step made with CellFluxes on `work`."""
    out = {}
    for q, n in enumerate(FLUX_NAMES):
        ptr = lib().ora_cell_flux(work.ptr, q)
        if not ptr:
            raise ValueError("no cell fluxes: step with CellFluxes=1 on this work first")
        out[n] = np.ctypeslib.as_array(ptr, shape=(int(np.prod(dom.shape3)),)).reshape(dom.shape3).copy()
    return out


def thomasz(D, E, F, TI, RES, WP) -> int:
    nk, nj, ni = (s - 2 for s in D.shape)
    return lib().ora_thomasz(ni, nj, nk, _p(D), _p(E), _p(F), _p(TI), _p(RES), _p(WP, _ip))


def advection_face(P4, V4, du4, dt, Q, VolumeRelMax, method, limiter, near_boundary, upwind2):
    out = np.zeros(4)
    P4, V4, du4 = (np.ascontiguousarray(x, dtype=np.float64) for x in (P4, V4, du4))
    rc = lib().ora_advection_face(_p(P4), _p(V4), _p(du4), dt, Q, VolumeRelMax, method, limiter,
                                  int(near_boundary), int(upwind2), _p(out))
    return rc, out


def mass(dom, P) -> float:
    cd = cdomain(dom)
    if P.dtype == np.float32:
        return lib().ora_mass_f32(C.byref(cd), _p(P, _fp))
    return lib().ora_mass(C.byref(cd), _p(P))


GEOMETRY_OUT = ("DWZ", "DUZ", "DVZ", "DZZ", "VolumeZ", "VolumeZOld", "AreaU", "AreaV")


def geometry(ni, nj, nk, SZZ, WP, DUX, DVY, DXX, DYY, faces_option, store_old, out: dict) -> None:
    """ComputeDistances / ComputeVolumes / ComputeAreas (and StoreVolumeZOld when
    store_old) of ModuleGeometry, in place on the arrays of `out` (keys
    GEOMETRY_OUT, float64 Size box)."""
    for n in GEOMETRY_OUT:
        assert out[n].dtype == np.float64 and out[n].flags.c_contiguous
    lib().ora_geometry(ni, nj, nk, _p(SZZ), _p(WP, _ip), _p(DUX), _p(DVY), _p(DXX), _p(DYY),
                       int(faces_option), int(store_old), *[_p(out[n]) for n in GEOMETRY_OUT])


def vertical_flux(dom, Qz: np.ndarray, dt: float, var_grid: bool) -> None:
    """WaterFlux_Z_VarGrid (var_grid) / WaterFlux_Z_FixGrid of ModuleHydrodynamic,
    in place on Qz, from the domain's horizontal fluxes, volumes and masks."""
    a = dom.arrays
    assert Qz.dtype == np.float64 and Qz.flags.c_contiguous
    lib().ora_vertical_flux(dom.ni, dom.nj, dom.nk, _p(a["Wflux_X"]), _p(a["Wflux_Y"]), _p(Qz), _p(a["VolumeZ"]),
                            _p(a["VolumeZOld"]), _p(a["ComputeFacesU3D"], _ip), _p(a["ComputeFacesV3D"], _ip),
                            _p(a["WaterPoints3D"], _ip), float(dt), int(bool(var_grid)))
