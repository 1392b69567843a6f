"""Build the native libraries of mohid_gb300 in-tree (no pip install).

  mohid_gb300/_lib/libmohid_ad.so     CUDA kernels + C-ABI (include/mohid_ad.h), sm_103a
  mohid_gb300/_lib/libmohid_synth.so  seeded synthetic-input generator (plain C)

Translation units are compiled in parallel; one -gencode (sm_103a) only.
The FP64 drop-in kernel is compiled with --fmad=false so that every a*b+c is
rounded twice, as the Fortran reference evaluates it.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
LIB = PKG / "_lib"
OBJ = PKG / "_build"
GENCODE = "-gencode=arch=compute_103a,code=sm_103a"

# (source, extra nvcc flags[, object name])
CUDA_UNITS = [
    ("plain_f64.cu", ["--fmad=false"]),
    ("batched_kernel.cu", []),
    ("batched_kernel_obc.cu", []),
    ("batched_flux.cu", []),
] + [
    # the batched step's kernels: one unit per form (closed, MassConservation
    # open boundaries, every boundary treatment and discharges), storage and
    # tile height
    ("batched_inst.cu", [f"-DMOHID_INST_OBC={o}", f"-DMOHID_INST_STORAGE={st}", f"-DMOHID_INST_TY={ty}"],
     f"batched_inst_{o}{st}_{ty}")
    for o in (0, 1, 2) for st in (0, 1, 2) for ty in (8, 4)
] + [
    ("ensemble_kernel.cu", []),
    ("batched_pack.cu", []),
    ("mass_noalloc.cu", []),
    ("producers.cu", ["--fmad=false"]),
    ("abi.cpp", []),
    ("batched_abi.cpp", []),
]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build mohid_gb300")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> dict:
    LIB.mkdir(exist_ok=True)
    OBJ.mkdir(exist_ok=True)
    nvcc = _nvcc()
    headers = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list(CSRC.glob("*.hpp")) + [PKG.parent / "include" / "mohid_ad.h"]
    common = [nvcc, GENCODE, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O3",
              "-I", str(PKG.parent / "include")]
    jobs = []
    objs = []
    for unit in CUDA_UNITS:
        src, extra = unit[0], unit[1]
        s = CSRC / src
        o = OBJ / ((unit[2] if len(unit) > 2 else Path(src).stem) + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            lang = ["-x", "cu"] if src.endswith(".cu") else []
            jobs.append(common + extra + lang + ["-c", str(s), "-o", str(o)])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 2))) as ex:
        for fut in [ex.submit(_run, j) for j in jobs]:
            fut.result()
    so = LIB / "libmohid_ad.so"
    if force or jobs or _stale(so, objs):
        _run([nvcc, GENCODE, "-shared", "-Xlinker", "--no-undefined", "-o", str(so)] +
             [str(o) for o in objs] + ["-lcudart"])
    # synthetic-input generator (host C)
    cc = os.environ.get("CC", "gcc")
    syn = LIB / "libmohid_synth.so"
    if force or _stale(syn, [CSRC / "synth.c", CSRC / "synth.h"]):
        _run([cc, "-O3", "-fPIC", "-shared", "-std=c11", "-ffp-contract=off", "-o", str(syn),
              str(CSRC / "synth.c"), "-lm"])
    if verbose:
        print(f"built {so} and {syn}", file=sys.stderr)
    return {"ad": str(so), "synth": str(syn)}


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv)
