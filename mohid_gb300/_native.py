"""ctypes bindings of the native libraries (include/mohid_ad.h, csrc/synth.h).

The CUDA library is mandatory: importing a transport entry point when
libmohid_ad.so is missing raises instead of falling back to any CPU code.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

_PKG = Path(__file__).resolve().parent
_LIB = _PKG / "_lib"

c_int_p = C.POINTER(C.c_int)
c_double_p = C.POINTER(C.c_double)
c_float_p = C.POINTER(C.c_float)


class T_Size3D(C.Structure):
    """T_Size3D, ModuleGlobalData.F90:2042-2052."""
    _fields_ = [("ILB", C.c_int), ("IUB", C.c_int), ("JLB", C.c_int),
                ("JUB", C.c_int), ("KLB", C.c_int), ("KUB", C.c_int)]


class MohidAdParams(C.Structure):
    """mohid_ad_params: scalar arguments of AdvectionDiffusion (AD:1108-1198)."""
    _fields_ = [
        ("schmidt_H", C.c_double), ("SchmidtCoef_V", C.c_double),
        ("SchmidtBackground_V", C.c_double),
        ("AdvMethodH", C.c_int), ("TVDLimitationH", C.c_int),
        ("AdvMethodV", C.c_int), ("TVDLimitationV", C.c_int),
        ("Upwind2H", C.c_int), ("Upwind2V", C.c_int),
        ("VolumeRelMax", C.c_double), ("DTProp", C.c_double),
        ("ImpExp_AdvV", C.c_double), ("ImpExp_DifV", C.c_double),
        ("ImpExp_AdvXX", C.c_double), ("ImpExp_AdvYY", C.c_double),
        ("ImpExp_DifH", C.c_double),
        ("NullDif", C.c_int), ("BoundaryCondition", C.c_int),
        ("DecayTime", C.c_double),
        ("AdvectionNudging", C.c_int), ("AdvectionNudgingCells", C.c_int),
        ("CellFluxes", C.c_int), ("NoAdvFlux", C.c_int), ("NoDifFlux", C.c_int),
        ("Optimize", C.c_int), ("FirstProperty", C.c_int),
        ("Vertical1D", C.c_int), ("XZFlow", C.c_int), ("Docycle_method", C.c_int),
    ]


class SynthParams(C.Structure):
    """mohid_synth_params (csrc/synth.h)."""
    _fields_ = [
        ("ni", C.c_int), ("nj", C.c_int), ("nk", C.c_int),
        ("dx", C.c_double), ("dy", C.c_double),
        ("zlevel", C.c_int), ("hmin", C.c_double), ("hmax", C.c_double),
        ("bathy_kind", C.c_int), ("land_frac", C.c_double), ("land_kind", C.c_int),
        ("umax", C.c_double), ("visc_h", C.c_double),
        ("kz_median", C.c_double), ("kz_logsigma", C.c_double),
        ("open_sides", C.c_int), ("vol_var", C.c_double), ("dt", C.c_double),
        ("seed", C.c_uint64),
    ]


class SynthOut(C.Structure):
    """mohid_synth_out (csrc/synth.h)."""
    _fields_ = [(n, c_double_p) for n in ("DUX", "DVY", "DZX", "DZY")] + \
        [(n, c_int_p) for n in ("KFloorZ", "BoundaryPoints2D", "WaterPoints2D")] + \
        [(n, c_double_p) for n in ("Wflux_X", "Wflux_Y", "Wflux_Z", "VolumeZOld", "VolumeZ",
                                   "Visc_H", "Diff_V", "AreaU", "AreaV", "DZZ", "DWZ")] + \
        [(n, c_int_p) for n in ("OpenPoints3D", "LandPoints3D", "WaterPoints3D",
                                "ComputeFacesU3D", "ComputeFacesV3D", "ComputeFacesW3D")] + \
        [("depth", c_double_p)]


# exported symbols of libmohid_ad.so with their ctypes signatures
_AD_SIGS = {
    "mohid_ad_default_params": (None, [C.POINTER(MohidAdParams)]),
    "mohid_ad_last_error": (C.c_char_p, []),
    "mohid_ad_version": (C.c_char_p, []),
    "mohid_ad_init": (C.c_int, [c_int_p, C.POINTER(T_Size3D), C.POINTER(T_Size3D)] +
                      [c_double_p] * 4 + [c_int_p, c_int_p, c_int_p]),
    "mohid_ad_set_hydro": (C.c_int, [c_int_p] + [c_double_p] * 11 + [c_int_p] * 7 + [c_int_p]),
    "mohid_ad_set_hydro_dev": (C.c_int, [c_int_p] + [c_double_p] * 11 + [c_int_p] * 7 + [c_int_p]),
    "mohid_ad_bind_hydro_dev": (C.c_int, [c_int_p] + [c_double_p] * 11 + [c_int_p] * 7 + [c_int_p]),
    "mohid_ad_step_prop_f64": (C.c_int, [c_int_p, c_double_p, c_double_p,
                                         C.POINTER(MohidAdParams), c_int_p]),
    "mohid_ad_step_prop_f64_dev": (C.c_int, [c_int_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                             C.POINTER(MohidAdParams), c_int_p]),
    "mohid_ad_step_f64": (C.c_int, [c_int_p, c_double_p, C.POINTER(MohidAdParams)] +
                          [c_double_p] * 11 + [c_int_p] * 7 + [c_double_p, c_int_p]),
    "mohid_ad_sync": (C.c_int, [c_int_p, c_int_p]),
    "mohid_ad_stream": (C.c_void_p, [c_int_p]),
    "mohid_ad_kill": (C.c_int, [c_int_p, c_int_p]),
    "mohid_thomasz_f64": (C.c_int, [c_int_p] * 6 + [C.POINTER(T_Size3D)] + [c_double_p] * 5 +
                          [c_int_p, c_int_p]),
    "mohid_ad_batched_create": (C.c_int, [c_int_p, c_int_p, c_int_p, c_int_p, c_int_p]),
    "mohid_ad_batched_pack_hydro": (C.c_int, [c_int_p, c_int_p]),
    "mohid_ad_batched_set_tracer": (C.c_int, [c_int_p, c_int_p, C.c_void_p, c_int_p, c_int_p]),
    "mohid_ad_batched_get_tracer": (C.c_int, [c_int_p, c_int_p, C.c_void_p, c_int_p, c_int_p]),
    "mohid_ad_batched_set_reference": (C.c_int, [c_int_p, c_int_p, C.c_void_p, c_int_p, c_int_p]),
    "mohid_ad_batched_set_discharge_conc": (C.c_int, [c_int_p, c_int_p, C.c_void_p, c_int_p]),
    "mohid_ad_batched_step": (C.c_int, [c_int_p, C.POINTER(MohidAdParams), c_int_p, c_int_p, c_int_p]),
    "mohid_ad_batched_mass": (C.c_int, [c_int_p, c_int_p, c_double_p, c_int_p]),
    "mohid_ad_batched_get_adv_flux": (C.c_int, [c_int_p, c_int_p, C.c_void_p, C.c_void_p, C.c_void_p, c_int_p,
                                                c_int_p]),
    "mohid_ad_batched_get_dif_flux": (C.c_int, [c_int_p, c_int_p, C.c_void_p, C.c_void_p, C.c_void_p, c_int_p,
                                                c_int_p]),
    "mohid_ad_batched_boundary_flux": (C.c_int, [c_int_p, c_int_p, c_double_p, c_int_p]),
    "mohid_ad_set_discharges": (C.c_int, [c_int_p, c_int_p] + [C.c_void_p] * 12 + [c_int_p]),
    "mohid_ad_unset_discharges": (C.c_int, [c_int_p, c_int_p]),
    "mohid_ad_set_noflux": (C.c_int, [c_int_p, C.c_void_p, C.c_void_p, C.c_void_p, c_int_p]),
    "mohid_ad_set_prop_old": (C.c_int, [c_int_p, C.c_void_p, c_int_p, c_int_p]),
    "mohid_ad_debug_fail_alloc": (C.c_int, [c_int_p, c_int_p]),
    "mohid_ad_debug_wait_probe": (C.c_int, [c_int_p, c_int_p]),
    "mohid_ad_get_adv_flux": (C.c_int, [c_int_p, C.c_void_p, C.c_void_p, C.c_void_p, c_int_p, c_int_p]),
    "mohid_ad_get_dif_flux": (C.c_int, [c_int_p, C.c_void_p, C.c_void_p, C.c_void_p, c_int_p, c_int_p]),
    "mohid_ad_batched_set_mass_fix": (C.c_int, [c_int_p, c_int_p, c_int_p]),
    "mohid_ad_batched_autotune": (C.c_int, [c_int_p, C.POINTER(MohidAdParams), c_int_p]),
    "mohid_ad_batched_schedule": (C.c_int, [c_int_p, c_int_p, c_int_p, c_int_p, c_int_p, c_int_p, c_int_p]),
    "mohid_ad_batched_set_schedule": (C.c_int, [c_int_p, c_int_p, c_int_p, c_int_p, c_int_p]),
    "mohid_ad_batched_sync": (C.c_int, [c_int_p, c_int_p]),
    "mohid_ad_batched_destroy": (C.c_int, [c_int_p, c_int_p]),
    "mohid_ad_ensemble_create": (C.c_int, [c_int_p, c_int_p, c_int_p, c_int_p]),
    "mohid_ad_ensemble_step": (C.c_int, [c_int_p, C.POINTER(MohidAdParams), c_int_p, c_int_p, c_int_p]),
    "mohid_ad_ensemble_destroy": (C.c_int, [c_int_p, c_int_p]),
    "mohid_ad_get_hydro": (C.c_int, [c_int_p] + [c_double_p] * 11 + [c_int_p, c_int_p]),
    "mohid_ad_geometry_dev": (C.c_int, [c_int_p, C.c_void_p, C.c_void_p, C.c_void_p, c_int_p, c_int_p, c_int_p]),
    "mohid_ad_vertical_flux": (C.c_int, [c_int_p, c_double_p, c_int_p, c_int_p]),
    "mohid_ad_mass_f64_noalloc": (C.c_int, [C.POINTER(T_Size3D), C.c_void_p, C.c_void_p, C.c_void_p,
                                            C.c_void_p, C.c_void_p, c_int_p]),
}

_SYN_SIGS = {
    "mohid_synth_generate": (C.c_int, [C.POINTER(SynthParams), C.POINTER(SynthOut)]),
    "mohid_synth_tracer": (C.c_int, [C.POINTER(SynthParams), C.POINTER(SynthOut), C.c_int,
                                     C.c_double, C.c_double, C.c_uint64, c_double_p]),
    "mohid_synth_reference": (C.c_int, [C.POINTER(SynthParams), C.POINTER(SynthOut), C.c_double,
                                        C.c_double, C.c_uint64, c_double_p]),
}

_cache: dict[str, C.CDLL] = {}


def lib_path(name: str) -> Path:
    return _LIB / name


def _load(name: str, sigs: dict) -> C.CDLL:
    if name in _cache:
        return _cache[name]
    p = lib_path(name)
    if not p.exists():
        raise RuntimeError(f"{p} is missing: run `python -m mohid_gb300.build` "
                           "(or __graft_entry__.build()) first; there is no CPU fallback")
    lib = C.CDLL(str(p), mode=C.RTLD_GLOBAL)
    for sym, (res, args) in sigs.items():
        fn = getattr(lib, sym)
        fn.restype = res
        fn.argtypes = args
    _cache[name] = lib
    return lib


def ad_lib() -> C.CDLL:
    """libmohid_ad.so (CUDA kernels + C-ABI)."""
    return _load("libmohid_ad.so", _AD_SIGS)


def synth_lib() -> C.CDLL:
    """libmohid_synth.so (synthetic-input generator)."""
    return _load("libmohid_synth.so", _SYN_SIGS)


AD_SYMBOLS = tuple(_AD_SIGS)
SYNTH_SYMBOLS = tuple(_SYN_SIGS)

# status codes (include/mohid_ad.h)
STATUS_NAMES = {
    0: "SUCCESS", 1: "ERR_BOUNDS", 2: "ERR_ID", 3: "ERR_OPTION", 4: "ERR_UNSUPPORTED",
    5: "ERR_CUDA", 6: "ERR_ZERO_PIVOT", 7: "ERR_NONFINITE", 8: "ERR_ALLOC", 9: "ERR_NULLPTR",
    10: "ERR_TIMEOUT",
}


class MohidAdError(RuntimeError):
    def __init__(self, code: int, where: str, msg: str = ""):
        self.code = code
        super().__init__(f"{where}: {STATUS_NAMES.get(code, code)} ({code}) {msg}".rstrip())


def check(code: int, where: str) -> None:
    if code != 0:
        msg = ""
        if "libmohid_ad.so" in _cache:
            msg = _cache["libmohid_ad.so"].mohid_ad_last_error().decode(errors="replace")
        raise MohidAdError(code, where, msg)


def ptr(a, ctype=C.c_double):
    """ctypes pointer to a numpy array's data (None passes NULL)."""
    if a is None:
        return None
    return a.ctypes.data_as(C.POINTER(ctype))


def iptr(a):
    return ptr(a, C.c_int)

