"""Batched FP32 multi-tracer form on the GPU against the FP64 oracle.

Tolerance (FP32 arithmetic, FP64 volume difference): relative L2 over water
cells <= 1e-5 after the stated number of steps; a single step is expected to
agree to ~1e-6.  With FP16-stored transports the oracle is run on the same
FP16-rounded transports, so the bar measures the arithmetic alone.
"""
import numpy as np
import pytest

from mohid_gb300 import advdiff, batched, configs, synth
from oracle import oracle as O
from tests.cases import domain, fp16_round_fields

pytestmark = pytest.mark.gpu
TOL = 1e-5

BATCH_OPTIONS = {
    "upwind1": dict(),
    "tvd_superbee": dict(AdvMethodH=4, TVDLimitationH=4, Upwind2H=1),
    "tvd_minmod": dict(AdvMethodH=4, TVDLimitationH=1, Upwind2H=1),
    "tvd_vanleer": dict(AdvMethodH=4, TVDLimitationH=2, Upwind2H=1),
    "tvd_muscl": dict(AdvMethodH=4, TVDLimitationH=3, Upwind2H=1),
    "tvd_pdm": dict(AdvMethodH=4, TVDLimitationH=5, Upwind2H=1),
    "nulldif": dict(NullDif=1),
    "xzflow": dict(XZFlow=1),
    "vertical1d": dict(Vertical1D=1),
    "background": dict(SchmidtBackground_V=1e-3, schmidt_H=0.7, SchmidtCoef_V=2.0),
}


def rel_l2(d, a, b):
    wp = d.water_mask()
    return float(np.linalg.norm(a[wp] - b[wp]) / np.linalg.norm(b[wp]))


def run_pair(d, tracers, pd, steps, storage=batched.FP32, refs=None, graph=False):
    """(oracle results, batched results) after `steps` steps."""
    ad = advdiff.AdvectionDiffusion(d)
    ad.set_hydro()
    b = batched.Batch(ad, len(tracers), storage)
    for t, P in enumerate(tracers):
        b.set_tracer(t, P)
        if refs is not None:
            b.set_reference(t, refs[t])
    b.step(advdiff.params(**pd), nsteps=steps, graph=graph)
    b.sync()
    got = [b.get_tracer(t) for t in range(len(tracers))]
    b.destroy()
    ad.kill()
    want = []
    work = O.Work(d)
    for t, P in enumerate(tracers):
        Q = P.copy()
        for _ in range(steps):
            assert O.step(d, Q, O.params(**pd), ReferenceProp=None if refs is None else refs[t],
                          work=work) == 0
        want.append(Q)
    return want, got


@pytest.mark.parametrize("grid", ["coast", "zlevel", "layer1", "column"])
@pytest.mark.parametrize("opt", sorted(BATCH_OPTIONS))
@pytest.mark.parametrize("nt", [1, 3])
def test_batched_one_step(gpu, grid, opt, nt):
    d = domain(grid)
    tr = [d.tracer(3, 1.0 + t, 0.7, seed=9 + t) for t in range(nt)]
    want, got = run_pair(d, tr, dict(DTProp=30.0, **BATCH_OPTIONS[opt]), 1)
    wp = d.water_mask()
    for w, g in zip(want, got):
        assert rel_l2(d, g, w) <= 1e-6
        # land, null and halo cells exactly as the reference leaves them
        assert np.array_equal(g[~wp], w[~wp])


@pytest.mark.parametrize("grid", ["open", "nsopen"])
@pytest.mark.parametrize("opt", ["upwind1", "tvd_minmod", "tvd_superbee"])
@pytest.mark.parametrize("decay", [0.0, 600.0])
def test_batched_open_boundaries(gpu, grid, opt, decay):
    d = domain(grid)
    tr = [d.tracer(3, 1.0, 0.5, seed=1), d.tracer(1, 5.0, 20.0, seed=4)]
    refs = [d.reference(2.0, 0.3, seed=2), d.reference(12.0, 0.2, seed=3)]
    pd = dict(DTProp=30.0, BoundaryCondition=1, DecayTime=decay, **BATCH_OPTIONS[opt])
    want, got = run_pair(d, tr, pd, 5, refs=refs)
    for w, g in zip(want, got):
        assert rel_l2(d, g, w) <= TOL


@pytest.mark.parametrize("grid", ["open", "nsopen", "allopen"])
@pytest.mark.parametrize("opt", ["upwind1", "tvd_superbee"])
@pytest.mark.parametrize("bc,decay", [(2, 0.0), (2, 300.0), (5, 0.0), (7, 0.0), (4, 0.0), (8, 0.0)])
def test_batched_other_open_boundaries(gpu, grid, opt, bc, decay):
    # ImposedValue, SubModel (identity rows with the interior mean decayed
    # towards the reference), MassConservNullGrad (inflow rows take the
    # neighbours' mean), NullGradient (the sweep after the solve) and Cyclic
    # (references, then the copies across the domain after the solve), one
    # step and five steps against the oracle
    if grid == "allopen":
        d = synth.generate(synth.GenSpec(ni=40, nj=33, nk=6, land_frac=0.1, land_kind=1, seed=11, open_sides=15,
                                         bathy_kind=1, dt=30.0))
    else:
        d = domain(grid)
    tr = [d.tracer(3, 1.0, 0.5, seed=1), d.tracer(1, 5.0, 20.0, seed=4)]
    refs = [d.reference(2.0, 0.3, seed=2), d.reference(12.0, 0.2, seed=3)]
    pd = dict(DTProp=30.0, BoundaryCondition=bc, DecayTime=decay, **BATCH_OPTIONS[opt])
    for steps, tol in ((1, 1e-6), (5, TOL)):
        want, got = run_pair(d, tr, pd, steps, refs=refs)
        for w, g in zip(want, got):
            assert rel_l2(d, g, w) <= tol


@pytest.mark.parametrize("grid", ["nsopen", "allopen"])
def test_batched_null_gradient_without_reference(gpu, grid):
    # ImposeNullGradient runs after the solve whether or not a reference is given (AD:1874-1880)
    if grid == "allopen":
        d = synth.generate(synth.GenSpec(ni=40, nj=33, nk=6, land_frac=0.1, land_kind=1, seed=11, open_sides=15,
                                         bathy_kind=1, dt=30.0))
    else:
        d = domain(grid)
    tr = [d.tracer(3, 1.0, 0.5, seed=1), d.tracer(1, 5.0, 20.0, seed=4)]
    pd = dict(DTProp=30.0, BoundaryCondition=4, **BATCH_OPTIONS["tvd_superbee"])
    want, got = run_pair(d, tr, pd, 5)
    for w, g in zip(want, got):
        assert rel_l2(d, g, w) <= TOL


@pytest.mark.parametrize("grid", ["coast", "zlevel", "open"])
@pytest.mark.parametrize("opt", ["upwind1", "tvd_superbee"])
@pytest.mark.parametrize("seed", [0, 1])
def test_batched_discharges(gpu, grid, opt, seed):
    # SetDischarges with each tracer's concentrations: point and uniform
    # discharges, inflows, withdrawals (DischConcMF), a bypass and an ignored
    # discharge, with MassConservation boundaries where the grid is open; one
    # step at 1e-6 and five at 1e-5 against the oracle
    from tests.cases import discharges
    d = domain(grid)
    tr = [d.tracer(3, 1.0, 0.5, seed=2), d.tracer(1, 5.0, 20.0, seed=4)]
    refs = [d.reference(2.0, 0.3, seed=3), d.reference(12.0, 0.2, seed=5)] if d.spec.open_sides else None
    ds = discharges(d, seed=seed)
    concs = [ds["Conc"], ds["Conc"] * 3.0 + 10.0]
    pd = dict(DTProp=30.0, **BATCH_OPTIONS[opt])
    for steps, tol in ((1, 1e-6), (5, TOL)):
        ad = advdiff.AdvectionDiffusion(d)
        ad.set_hydro()
        ad.set_discharges(ds)
        b = batched.Batch(ad, len(tr))
        for t, P in enumerate(tr):
            b.set_tracer(t, P)
            b.set_discharge_conc(t, concs[t])
            if refs:
                b.set_reference(t, refs[t])
        b.step(advdiff.params(**pd), nsteps=steps, graph=steps > 1)
        b.sync()
        got = [b.get_tracer(t) for t in range(len(tr))]
        b.destroy()
        ad.kill()
        for t, P in enumerate(tr):
            Q = P.copy()
            for _ in range(steps):
                assert O.step(d, Q, O.params(**pd), ReferenceProp=refs[t] if refs else None,
                              Disch=dict(ds, Conc=concs[t])) == 0
            assert rel_l2(d, got[t], Q) <= tol


def test_batched_discharges_need_every_concentration(gpu):
    from tests.cases import discharges
    d = domain("coast")
    ad = advdiff.AdvectionDiffusion(d)
    ad.set_hydro()
    ad.set_discharges(discharges(d, seed=0))
    b = batched.Batch(ad, 2)
    b.set_tracer(0, d.tracer(3, 1.0, 0.5, seed=2))
    b.set_tracer(1, d.tracer(3, 1.0, 0.5, seed=3))
    b.set_discharge_conc(0, discharges(d, seed=0)["Conc"])
    with pytest.raises(advdiff.N.MohidAdError) as ei:
        b.step(advdiff.params(DTProp=30.0))
    assert ei.value.code == 3
    b.destroy()
    ad.kill()


@pytest.mark.parametrize("grid", ["coast", "zlevel", "layer1"])
@pytest.mark.parametrize("opt", ["upwind1", "tvd_superbee"])
@pytest.mark.parametrize("flags", [dict(NoAdvFlux=1), dict(NoDifFlux=1), dict(NoAdvFlux=1, NoDifFlux=1)])
def test_batched_noflux_masks(gpu, grid, opt, flags):
    # NoAdvFlux / NoDifFlux with the instance's NoFluxU/V/W masks: one step at
    # 1e-6, then four more alternating with and without the options (the
    # flags are formed again each time) at 1e-5, against the oracle
    from tests.cases import noflux_masks
    d = domain(grid)
    nf = noflux_masks(d, seed=5)
    tr = [d.tracer(3, 1.0, 0.5, seed=2), d.tracer(1, 5.0, 20.0, seed=4)]
    base = dict(DTProp=30.0, **BATCH_OPTIONS[opt])
    seq = [dict(base, **flags), base, dict(base, **flags), dict(base, **flags), base]
    ad = advdiff.AdvectionDiffusion(d)
    ad.set_hydro()
    b = batched.Batch(ad, len(tr))
    for t, P in enumerate(tr):
        b.set_tracer(t, P)
    with pytest.raises(advdiff.N.MohidAdError) as ei:        # the masks are required
        b.step(advdiff.params(**seq[0]))
    assert ei.value.code == 9
    ad.set_noflux(nf)
    want = [P.copy() for P in tr]
    work = O.Work(d)
    for n, pd in enumerate(seq):
        b.step(advdiff.params(**pd), nsteps=1)
        b.sync()
        for Q in want:
            assert O.step(d, Q, O.params(**pd), work=work, NoFlux=nf) == 0
        for t, Q in enumerate(want):
            assert rel_l2(d, b.get_tracer(t), Q) <= (1e-6 if n == 0 else TOL)
    b.destroy()
    ad.kill()


def _batched_fluxes(d, tr, refs, pd, steps, nf=None):
    """(per tracer: oracle fluxes, batched fluxes) of the last of `steps` steps."""
    ad = advdiff.AdvectionDiffusion(d)
    ad.set_hydro()
    if nf is not None:
        ad.set_noflux(nf)
    b = batched.Batch(ad, len(tr))
    for t, P in enumerate(tr):
        b.set_tracer(t, P)
        if refs:
            b.set_reference(t, refs[t])
    b.step(advdiff.params(**pd), nsteps=steps, graph=steps > 1)
    b.sync()
    got = [b.cell_fluxes(t) for t in range(len(tr))]
    b.destroy()
    ad.kill()
    out = []
    for t, P in enumerate(tr):
        Q = P.copy()
        work = O.Work(d)
        for _ in range(steps):
            assert O.step(d, Q, O.params(**pd), ReferenceProp=refs[t] if refs else None, work=work,
                          NoFlux=nf) == 0
        out.append((O.cell_fluxes(d, work), got[t]))
    return out


# FP32 fluxes against FP64 ones: relative L2 per array.  The explicit
# horizontal fluxes of a first step see the loaded field (rounded once to
# FP32); the others see a field after FP32 steps, and the diffusive ones are
# differences of neighbouring values, which the field's error enters relative
# to the difference.
FLUX_TOL = {1: 1e-5, 3: 2e-5}


@pytest.mark.parametrize("grid", ["coast", "zlevel", "open"])
@pytest.mark.parametrize("opt", ["upwind1", "tvd_superbee", "tvd_pdm", "nulldif", "xzflow", "vertical1d",
                                 "background"])
def test_batched_cell_fluxes(gpu, grid, opt):
    # GetAdvFlux / GetDifFlux of the batched form against the oracle's, after
    # one step and after three (the last step's fluxes); arrays the oracle
    # leaves zero are zero
    d = domain(grid)
    tr = [d.tracer(3, 1.0, 0.5, seed=2), d.tracer(1, 5.0, 20.0, seed=4)]
    refs = [d.reference(2.0, 0.3, seed=3), d.reference(12.0, 0.2, seed=5)] if d.spec.open_sides else None
    pd = dict(DTProp=30.0, CellFluxes=1, **BATCH_OPTIONS[opt])
    for steps in (1, 3):
        for want, got in _batched_fluxes(d, tr, refs, pd, steps):
            for n in O.FLUX_NAMES:
                w, g = want[n], got[n]
                nw = float(np.linalg.norm(w))
                if nw == 0.0:
                    assert not g.any(), n
                else:
                    assert float(np.linalg.norm(g - w)) <= FLUX_TOL[steps] * nw, (n, steps)


@pytest.mark.parametrize("flags", [dict(NoAdvFlux=1), dict(NoDifFlux=1)])
def test_batched_cell_fluxes_noflux(gpu, flags):
    # masked faces carry no flux, except DifFluxZ, which the reference forms
    # from the unmasked diffusivity
    from tests.cases import noflux_masks
    d = domain("coast")
    nf = noflux_masks(d, seed=5)
    tr = [d.tracer(3, 1.0, 0.5, seed=2)]
    pd = dict(DTProp=30.0, CellFluxes=1, **flags, **BATCH_OPTIONS["tvd_superbee"])
    for want, got in _batched_fluxes(d, tr, None, pd, 1, nf=nf):
        for n in O.FLUX_NAMES:
            w, g = want[n], got[n]
            assert float(np.linalg.norm(g - w)) <= FLUX_TOL[1] * float(np.linalg.norm(w)), n


def test_batched_cell_fluxes_need_the_option(gpu):
    d = domain("coast")
    ad = advdiff.AdvectionDiffusion(d)
    ad.set_hydro()
    b = batched.Batch(ad, 1)
    b.set_tracer(0, d.tracer(3, 1.0, 0.5, seed=2))
    b.step(advdiff.params(DTProp=30.0))
    with pytest.raises(advdiff.N.MohidAdError) as ei:
        b.cell_fluxes(0)
    assert ei.value.code == 3
    b.step(advdiff.params(DTProp=30.0, CellFluxes=1))
    b.cell_fluxes(0)
    b.set_tracer(0, d.tracer(3, 1.0, 0.5, seed=3))       # the buffers no longer hold that step
    with pytest.raises(advdiff.N.MohidAdError) as ei:
        b.cell_fluxes(0)
    assert ei.value.code == 3
    b.destroy()
    ad.kill()


def test_batched_noflux_rejected_with_references(gpu):
    from tests.cases import noflux_masks
    d = domain("open")
    ad = advdiff.AdvectionDiffusion(d)
    ad.set_hydro()
    ad.set_noflux(noflux_masks(d, seed=5))
    b = batched.Batch(ad, 1)
    b.set_tracer(0, d.tracer(3, 1.0, 0.5, seed=2))
    b.set_reference(0, d.reference(2.0, 0.3, seed=3))
    with pytest.raises(advdiff.N.MohidAdError) as ei:
        b.step(advdiff.params(DTProp=30.0, NoAdvFlux=1))
    assert ei.value.code == 4
    b.destroy()
    ad.kill()


def test_batched_rejects_boundary_conditions_like_the_plain_form(gpu):
    # Orlanski stays with the plain form (MOHID_AD_ERR_UNSUPPORTED); codes
    # the reference rejects give MOHID_AD_ERR_OPTION as there
    d = domain("open")
    ad = advdiff.AdvectionDiffusion(d)
    ad.set_hydro()
    b = batched.Batch(ad, 1)
    b.set_tracer(0, d.tracer(3, 1.0, 0.5, seed=1))
    for bc, code in ((8, 3),):                       # cyclic without a reference
        with pytest.raises(advdiff.N.MohidAdError) as ei:
            b.step(advdiff.params(DTProp=30.0, BoundaryCondition=bc))
        assert ei.value.code == code
    b.set_reference(0, d.reference(2.0, 0.3, seed=2))
    for bc, code in ((6, 4), (3, 3)):
        with pytest.raises(advdiff.N.MohidAdError) as ei:
            b.step(advdiff.params(DTProp=30.0, BoundaryCondition=bc))
        assert ei.value.code == code
    b.destroy()
    ad.kill()


def test_batched_cfg1_100_steps(gpu):
    w = configs.cfg1()
    d = synth.generate(w.spec)
    tr = [d.tracer(*w.tracers[0], seed=11)]
    want, got = run_pair(d, tr, w.params(), w.steps)
    assert rel_l2(d, got[0], want[0]) <= TOL


def test_batched_cfg2_grid_300_steps(gpu):
    """Config 2 options (P2_TVD SuperBee, T and S) on a 128x128x40 cut, 300 steps."""
    w = configs.cfg2().scaled(ni=128, nj=128)
    d = synth.generate(w.spec)
    tr = [d.tracer(k, a, b, seed=100 + t) for t, (k, a, b) in enumerate(w.tracers)]
    want, got = run_pair(d, tr, w.params(), 300, graph=True)
    for a_, b_ in zip(got, want):
        assert rel_l2(d, a_, b_) <= TOL


def test_batched_graph_equals_direct(gpu):
    d = domain("coast")
    tr = [d.tracer(3, 1.0, 0.7, seed=9), d.tracer(1, 3.0, 9.0, seed=2)]
    pd = dict(DTProp=30.0, AdvMethodH=4, TVDLimitationH=4, Upwind2H=1)
    _, direct = run_pair(d, tr, pd, 7, graph=False)
    _, graphed = run_pair(d, tr, pd, 7, graph=True)
    for a_, b_ in zip(direct, graphed):
        assert np.array_equal(a_, b_)


@pytest.mark.parametrize("storage", [batched.FP16_Q, batched.FP16_QK])
def test_batched_fp16_storage(gpu, storage):
    """FP16-stored transports (and diffusivities): oracle on the same rounded inputs."""
    import torch
    w = configs.cfg3().scaled(ni=96, nj=64, nk=20)
    d = synth.generate(w.spec)
    fp16_round_fields(d, storage)      # the same per-field scaling the library applies
    tr = [d.tracer(k, a_, b_, seed=7 + t) for t, (k, a_, b_) in enumerate(w.tracers[:4])]
    want, got = run_pair(d, tr, w.params(), 20, storage=storage)
    for g_, w_ in zip(got, want):
        assert rel_l2(d, g_, w_) <= TOL


def test_batched_mass_budget_matches_oracle_sum(gpu):
    d = domain("zlevel")
    P = d.tracer(3, 2.0, 0.5, seed=5)
    ad = advdiff.AdvectionDiffusion(d)
    ad.set_hydro()
    b = batched.Batch(ad, 1)
    b.set_tracer(0, P)
    b.step(advdiff.params(DTProp=30.0), nsteps=3)
    m = b.mass(0)
    Pg = b.get_tracer(0)
    b.destroy(); ad.kill()
    # the stored anomaly plus its constant, summed in FP64 by the oracle
    assert abs(m - O.mass(d, Pg)) <= 1e-14 * abs(m)


@pytest.mark.parametrize("bad", [dict(AdvMethodH=5), dict(AdvMethodV=4, TVDLimitationV=4, Upwind2V=1),
                                 dict(ImpExp_DifV=0.5), dict(Docycle_method=2), dict(ImpExp_AdvV=0.0)])
def test_batched_rejects_unsupported(gpu, bad):
    d = domain("coast")
    ad = advdiff.AdvectionDiffusion(d)
    ad.set_hydro()
    b = batched.Batch(ad, 1)
    b.set_tracer(0, d.tracer(4, 1.0, 0.0, seed=1))
    with pytest.raises(advdiff.N.MohidAdError) as ei:
        b.step(advdiff.params(DTProp=30.0, **bad))
    assert ei.value.code == 4
    b.destroy(); ad.kill()


@pytest.mark.parametrize("storage", [0, 1, 2])
def test_graph_rebuilt_after_new_hydrodynamics(gpu, storage):
    """A graph captured under one hydrodynamic state is not reused under the
    next (its arguments hold the FP16 scales and the tile count): graph and
    direct stepping agree bit for bit across a change of state."""
    from mohid_gb300 import synth
    d = domain("coast")
    arrays = dict(d.arrays)
    for n in ("Wflux_X", "Wflux_Y", "Wflux_Z"):
        arrays[n] = d.arrays[n] * 0.5                    # divergence-free still
    d2 = synth.Domain(spec=d.spec, arrays=arrays)
    P = d.tracer(3, 1.0, 0.5, seed=1)
    pd = advdiff.params(DTProp=30.0, AdvMethodH=4, TVDLimitationH=4, Upwind2H=1)
    out = {}
    for graph in (True, False):
        ad = advdiff.AdvectionDiffusion(d)
        ad.set_hydro()
        b = batched.Batch(ad, 1, storage)
        b.set_tracer(0, P)
        b.step(pd, nsteps=4, graph=graph)
        ad.set_hydro(d2)
        b.step(pd, nsteps=4, graph=graph)
        ad.set_hydro(d)
        b.step(pd, nsteps=4, graph=graph)
        b.sync()
        out[graph] = b.get_tracer(0)
        b.destroy()
        ad.kill()
    assert np.array_equal(out[True], out[False])
