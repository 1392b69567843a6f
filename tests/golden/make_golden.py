"""Write tests/golden/small_cases.npz: regression fixtures of the transport step.

No golden vectors of the reference exist for this path (its Fortran cannot be
built here), so these fixtures pin the oracle and the FP64 drop-in against
themselves across machines and revisions: the domain arrays themselves (not the
generator's seeds, whose transcendental functions may round differently on
another libm), the initial tracer, optional reference concentrations, and the
oracle's field after three steps, for a few grids and option sets.  The
oracle's step uses only IEEE +, -, *, / and min/max, so the outputs must be
reproduced bit for bit on any machine.

    python tests/golden/make_golden.py          # rewrites the fixture
"""
from __future__ import annotations

import sys
from dataclasses import asdict
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))

from oracle import oracle as O  # noqa: E402
from tests.cases import OPTIONS, domain  # noqa: E402

GRIDS = ["coast", "zlevel", "open"]
OPTS = ["upwind1", "tvd_superbee", "tvd_minmod", "upwind3", "explicit_v_tvd", "nulldif"]
STEPS = 3


def main():
    O.build()
    out = {}
    for g in GRIDS:
        d = domain(g)
        for k, v in asdict(d.spec).items():
            out[f"{g}/spec/{k}"] = np.array(v)
        for n, a in d.arrays.items():
            out[f"{g}/{n}"] = a
        P0 = d.tracer(3, 2.0, 0.5, seed=17)
        out[f"{g}/P0"] = P0
        ref = d.reference(2.5, 0.3, seed=18) if d.spec.open_sides else None
        if ref is not None:
            out[f"{g}/Ref"] = ref
        for o in OPTS:
            pd = dict(DTProp=30.0, **OPTIONS[o])
            if ref is not None:
                pd.update(BoundaryCondition=1, DecayTime=0.0)
            P = P0.copy()
            work = O.Work(d)
            for _ in range(STEPS):
                assert O.step(d, P, O.params(**pd), ReferenceProp=ref, work=work) == 0
            out[f"{g}/{o}/P{STEPS}"] = P
    np.savez_compressed(HERE / "small_cases.npz", **out)
    print(f"wrote {HERE / 'small_cases.npz'}: {len(GRIDS)} grids x {len(OPTS)} option sets, {STEPS} steps")


if __name__ == "__main__":
    main()
