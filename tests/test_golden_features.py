"""Regression fixtures of the step's options (tests/golden/features.npz,
written by tests/golden/make_features.py): implicit horizontal advection,
NullGradient / MassConservNullGrad / Cyclic boundaries, NoFlux masks,
discharges and cell fluxes.  The oracle and the FP64 drop-in must reproduce
the stored fields (and fluxes) bit for bit on any machine."""
from pathlib import Path

import numpy as np
import pytest

from mohid_gb300 import synth
from oracle import oracle as O

FIX = Path(__file__).resolve().parent / "golden" / "features.npz"
STEPS = 3
FLUXES = ("AdvFluxX", "AdvFluxY", "AdvFluxZ", "DifFluxX", "DifFluxY", "DifFluxZ")


def _load():
    z = np.load(FIX)
    names = sorted({k.split("/")[0] for k in z.files})
    cases = {}
    for c in names:
        spec = {k.split("/")[-1]: z[k].item() for k in z.files if k.startswith(f"{c}/spec/")}
        arrays = {n: z[f"{c}/{n}"] for n in synth.F3 + synth.I3 + synth.F2 + synth.I2}
        d = synth.Domain(spec=synth.GenSpec(**spec), arrays=arrays)
        pd = {k.split("/")[-1]: z[k].item() for k in z.files if k.startswith(f"{c}/param/")}
        ref = z[f"{c}/Ref"] if f"{c}/Ref" in z.files else None
        nf = tuple(z[f"{c}/{n}"] for n in ("NoFluxU", "NoFluxV", "NoFluxW")) if f"{c}/NoFluxU" in z.files else None
        ds = {k.split("/")[-1]: z[k] for k in z.files if k.startswith(f"{c}/disch/")} or None
        flux = {n: z[f"{c}/flux/{n}"] for n in FLUXES} if f"{c}/flux/AdvFluxX" in z.files else None
        cases[c] = (d, z[f"{c}/P0"], pd, ref, nf, ds, z[f"{c}/P{STEPS}"], flux)
    return cases


CASES = sorted({k.split("/")[0] for k in np.load(FIX).files})


@pytest.fixture(scope="module")
def cases():
    return _load()


@pytest.mark.parametrize("case", CASES)
def test_oracle_reproduces_feature_fixture(built, cases, case):
    d, P0, pd, ref, nf, ds, want, flux = cases[case]
    P = P0.copy()
    work = O.Work(d)
    for _ in range(STEPS):
        assert O.step(d, P, O.params(**pd), ReferenceProp=ref, work=work, NoFlux=nf, Disch=ds) == 0
    assert np.array_equal(P, want)
    if flux is not None:
        got = O.cell_fluxes(d, work)
        for n in FLUXES:
            assert np.array_equal(got[n], flux[n]), n


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES)
def test_plain_f64_reproduces_feature_fixture(gpu, cases, case):
    from mohid_gb300 import advdiff
    d, P0, pd, ref, nf, ds, want, flux = cases[case]
    ad = advdiff.AdvectionDiffusion(d)
    ad.set_hydro()
    if nf is not None:
        ad.set_noflux(nf)
    if ds is not None:
        ad.set_discharges(ds)
    P = P0.copy()
    for _ in range(STEPS):
        ad.step(P, advdiff.params(**pd), ref)
    assert np.array_equal(P, want)
    if flux is not None:
        got = ad.cell_fluxes()
        for n in FLUXES:
            assert np.array_equal(got[n], flux[n]), n
    ad.kill()
