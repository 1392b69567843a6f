"""Restart files of a batched property group.

The transport step keeps no state between steps beyond the tracers (the
hydrodynamics are handed over every step), so a restart is the tracers'
fields and the step count -- what MOHID's final/restart file holds for the
transported properties (Write_FinalWaterProperties_HDF,
Software/MOHIDWater/ModuleWaterProperties.F90:28164-28404, which writes them as
HDF5).  No HDF5 library is available to this package, so the file is a numpy
archive: one float64 Size-box array per tracer (the values get_tracer
returns), the step count, the grid's bounds and the property names.

Loading sets the tracers again (set_tracer), which starts each tracer's mass
budget anew from the loaded field, as loading a restart does in MOHID.
"""
from __future__ import annotations

from pathlib import Path

import numpy as np

__all__ = ["save", "load", "RestartError"]

_FORMAT = "mohid-gb300-restart-1"


class RestartError(ValueError):
    """A restart file that does not fit the batch it is loaded into."""


def save(batch, path, step: int, names=None) -> None:
    """Write the batch's tracers (get_tracer) and the step count to `path`."""
    shape = tuple(batch.ad.domain.shape3)
    nt = batch.nt
    names = list(names) if names is not None else [f"tracer {t}" for t in range(nt)]
    if len(names) != nt:
        raise RestartError(f"{len(names)} names for {nt} tracers")
    arrays = {f"tracer_{t}": np.asarray(batch.get_tracer(t), dtype=np.float64) for t in range(nt)}
    for t, a in arrays.items():
        if a.shape != shape:
            raise RestartError(f"{t}: shape {a.shape}, grid {shape}")
    np.savez(Path(path), format=np.array(_FORMAT), step=np.array(step, dtype=np.int64),
             shape=np.array(shape, dtype=np.int64), names=np.array(names), **arrays)


def load(batch, path) -> tuple[int, list[str]]:
    """Set the batch's tracers from `path`; returns (step count, names)."""
    p = Path(path)
    if not p.exists() and Path(str(p) + ".npz").exists():      # np.savez appends .npz
        p = Path(str(p) + ".npz")
    with np.load(p, allow_pickle=False) as f:
        if str(f["format"]) != _FORMAT:
            raise RestartError(f"{p}: not a restart file of this format")
        shape = tuple(int(x) for x in f["shape"])
        if shape != tuple(batch.ad.domain.shape3):
            raise RestartError(f"{p}: grid {shape}, batch grid {tuple(batch.ad.domain.shape3)}")
        names = [str(x) for x in f["names"]]
        if len(names) != batch.nt:
            raise RestartError(f"{p}: {len(names)} tracers, batch has {batch.nt}")
        for t in range(batch.nt):
            batch.set_tracer(t, np.ascontiguousarray(f[f"tracer_{t}"]))
        return int(f["step"]), names
