"""Write tests/golden/features.npz: regression fixtures of the transport step's
options beyond tests/golden/small_cases.npz.

Like small_cases.npz, these pin the oracle and the FP64 drop-in against
themselves across machines and revisions (no golden vectors of the reference
exist for this path).  Each case stores its inputs (domain arrays, initial
tracer, reference concentrations, NoFlux masks, discharges) and the oracle's
field after three steps; the cell-flux case also stores the six face-flux
arrays of the last step.  The oracle uses only IEEE +, -, *, / and min/max, so
every output must be reproduced bit for bit.

    python tests/golden/make_features.py        # rewrites the fixture
"""
from __future__ import annotations

import sys
from dataclasses import asdict
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))

from oracle import oracle as O  # noqa: E402
from tests.cases import OPTIONS, discharges, domain, noflux_masks  # noqa: E402

STEPS = 3
# name: (grid, option set, extra params, reference?, NoFlux masks?, discharges?, cell fluxes?)
CASES = {
    "implicit_xx_coast": ("coast", "implicit_xx", {}, False, False, False, False),
    "implicit_yy_tvd_zlevel": ("zlevel", "implicit_yy_tvd", {}, False, False, False, False),
    "implicit_xx_layer1": ("layer1", "implicit_xx_central", {}, False, False, False, False),
    "nullgradient_open": ("open", "tvd_minmod", dict(BoundaryCondition=4), True, False, False, False),
    "massconsnullgrad_open": ("open", "upwind1", dict(BoundaryCondition=7), True, False, False, False),
    "cyclic_nsopen": ("nsopen", "tvd_superbee", dict(BoundaryCondition=8), True, False, False, False),
    "noflux_zlevel": ("zlevel", "tvd_superbee", dict(NoAdvFlux=1, NoDifFlux=1), False, True, False, False),
    "discharges_coast": ("coast", "theta_difv", {}, False, False, True, False),
    "cellfluxes_zlevel": ("zlevel", "explicit_v_tvd", dict(CellFluxes=1), False, False, False, True),
}


def case_inputs(name):
    """The inputs of a case, from the seeded generators."""
    grid, opt, extra, with_ref, with_nf, with_disch, _ = CASES[name]
    d = domain(grid)
    P0 = d.tracer(3, 2.0, 0.5, seed=23)
    ref = d.reference(2.5, 0.3, seed=24) if with_ref else None
    nf = noflux_masks(d, seed=25) if with_nf else None
    ds = discharges(d, seed=26) if with_disch else None
    pd = dict(DTProp=30.0, **OPTIONS[opt], **extra)
    return d, P0, ref, nf, ds, pd


def main():
    O.build()
    out = {}
    for name, (grid, _, _, _, _, _, cflux) in CASES.items():
        d, P0, ref, nf, ds, pd = case_inputs(name)
        for k, v in asdict(d.spec).items():
            out[f"{name}/spec/{k}"] = np.array(v)
        for n, a in d.arrays.items():
            out[f"{name}/{n}"] = a
        out[f"{name}/P0"] = P0
        if ref is not None:
            out[f"{name}/Ref"] = ref
        if nf is not None:
            for n, m in zip(("NoFluxU", "NoFluxV", "NoFluxW"), nf):
                out[f"{name}/{n}"] = m
        if ds is not None:
            for n, a in ds.items():
                out[f"{name}/disch/{n}"] = a
        for k, v in pd.items():
            out[f"{name}/param/{k}"] = np.array(v)
        P = P0.copy()
        work = O.Work(d)
        for _ in range(STEPS):
            assert O.step(d, P, O.params(**pd), ReferenceProp=ref, work=work, NoFlux=nf, Disch=ds) == 0
        out[f"{name}/P{STEPS}"] = P
        if cflux:
            for n, a in O.cell_fluxes(d, work).items():
                out[f"{name}/flux/{n}"] = a
    np.savez_compressed(HERE / "features.npz", **out)
    print(f"wrote {HERE / 'features.npz'}: {len(CASES)} cases, {STEPS} steps")


if __name__ == "__main__":
    main()
