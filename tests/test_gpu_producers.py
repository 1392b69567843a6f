"""Device producers of the step's inputs against the oracle, bit for bit.

mohid_ad_geometry_dev (ModuleGeometry: StoreVolumeZOld, ComputeDistances,
ComputeVolumes, ComputeAreas) and mohid_ad_vertical_flux (ModuleHydrodynamic:
WaterFlux_Z_VarGrid / _FixGrid) work in place on an instance's device arrays;
the oracle restates the same routines on the same starting arrays.  A transport
step made with the produced fields then equals the oracle's step on them.
"""
import dataclasses

import numpy as np
import pytest

from mohid_gb300 import advdiff, batched, synth
from oracle import oracle as O
from tests.cases import domain
from tests.test_oracle_producers import grid_lengths, szz_from

pytestmark = pytest.mark.gpu


def new_level(d, seed):
    """Layer interfaces of a new water level: every column's thicknesses scaled
    by a seeded factor within 2 %, its floor kept."""
    rng = np.random.default_rng(seed)
    f = 1.0 + 0.02 * (rng.random(d.shape2) - 0.5)
    szz = szz_from(d)
    bottom = szz[0].copy()
    dwz = d.arrays["DWZ"] * f[None]
    out = np.zeros(d.shape3)
    out[0] = bottom
    for k in range(1, d.nk + 1):
        out[k] = out[k - 1] - dwz[k]
    out[d.nk + 1] = out[d.nk]
    return out


def oracle_geometry(d, szz, state, faces_option):
    dxx, dyy = grid_lengths(d)
    O.geometry(d.ni, d.nj, d.nk, szz, d.arrays["WaterPoints3D"], d.arrays["DUX"], d.arrays["DVY"], dxx, dyy,
               faces_option, True, state)


@pytest.mark.parametrize("grid", ["coast", "zlevel", "open"])
@pytest.mark.parametrize("faces_option", [3, 2])
def test_geometry_and_vertical_flux_match_oracle(gpu, grid, faces_option):
    import torch
    d = domain(grid)
    a = d.arrays
    ad = advdiff.AdvectionDiffusion(d)
    ad.set_hydro()
    dxx, dyy = grid_lengths(d)
    DXX, DYY = torch.from_numpy(dxx).cuda(), torch.from_numpy(dyy).cuda()
    state = {n: a[n].copy() for n in ("DWZ", "DZZ", "VolumeZ", "VolumeZOld", "AreaU", "AreaV")}
    state["DUZ"] = np.zeros(d.shape3)
    state["DVZ"] = np.zeros(d.shape3)
    qz = a["Wflux_Z"].copy()
    for call in range(2):                           # two new levels: the arrays persist between calls
        szz = new_level(d, seed=call)
        ad.geometry(torch.from_numpy(szz).cuda(), DXX, DYY, faces_option, store_old=True)
        ad.vertical_flux(d.spec.dt, var_grid=call == 0)
        got = ad.get_fields()
        oracle_geometry(d, szz, state, faces_option)
        dn = synth.Domain(spec=d.spec, arrays=dict(a, VolumeZ=state["VolumeZ"], VolumeZOld=state["VolumeZOld"]))
        O.vertical_flux(dn, qz, d.spec.dt, call == 0)
        for n in ("DWZ", "DZZ", "VolumeZ", "VolumeZOld", "AreaU", "AreaV"):
            assert np.array_equal(got[n], state[n]), (call, n)
        assert np.array_equal(got["Wflux_Z"], qz), call
    ad.kill()


def test_step_with_produced_fields_matches_oracle(gpu):
    """Geometry and vertical flux made on the device, then one plain FP64 step
    and two batched FP32 steps, against the oracle on the produced fields."""
    import torch
    d = domain("open")
    a = d.arrays
    ad = advdiff.AdvectionDiffusion(d)
    ad.set_hydro()
    dxx, dyy = grid_lengths(d)
    szz = new_level(d, seed=7)
    ad.geometry(torch.from_numpy(szz).cuda(), torch.from_numpy(dxx).cuda(), torch.from_numpy(dyy).cuda(), 3, True)
    ad.vertical_flux(d.spec.dt, True)
    prod = ad.get_fields()
    dn = synth.Domain(spec=d.spec, arrays=dict(a, **{n: prod[n] for n in synth.F3}))
    pd = dict(DTProp=d.spec.dt, AdvMethodH=4, TVDLimitationH=4, Upwind2H=1)
    P = d.tracer(3, 2.0, 0.5, seed=3)
    ref = d.reference(2.0, 0.2, seed=4)
    Pg = P.copy()
    ad.step(Pg, advdiff.params(BoundaryCondition=1, **pd), ReferenceProp=ref)
    Po = P.copy()
    assert O.step(dn, Po, O.params(BoundaryCondition=1, **pd), ReferenceProp=ref) == 0
    assert np.array_equal(Pg, Po)
    # the batched form repacks the produced state (a new hydrodynamic version)
    b = batched.Batch(ad, 1)
    b.set_tracer(0, P)
    b.set_reference(0, ref)
    b.step(advdiff.params(BoundaryCondition=1, **pd), nsteps=2)
    b.sync()
    g = b.get_tracer(0)
    b.destroy()
    ad.kill()
    Q = P.copy()
    for _ in range(2):
        assert O.step(dn, Q, O.params(BoundaryCondition=1, **pd), ReferenceProp=ref) == 0
    wp = d.water_mask()
    assert np.linalg.norm(g[wp] - Q[wp]) / np.linalg.norm(Q[wp]) <= 1e-6


def test_partial_update_keeps_the_rest(gpu):
    """set_hydro with NULL arrays keeps the instance's copies and the masks."""
    d = domain("coast")
    ad = advdiff.AdvectionDiffusion(d)
    ad.set_hydro()
    qx = d.arrays["Wflux_X"] * 0.5
    ad.set_fields({"Wflux_X": qx})
    got = ad.get_fields()
    assert np.array_equal(got["Wflux_X"], qx)
    for n in synth.F3:
        if n != "Wflux_X":
            assert np.array_equal(got[n], d.arrays[n]), n
    # a step with the kept masks equals the oracle on the updated field
    dn = synth.Domain(spec=d.spec, arrays=dict(d.arrays, Wflux_X=qx))
    P = d.tracer(3, 1.0, 0.5, seed=2)
    Pg, Po = P.copy(), P.copy()
    ad.step(Pg, advdiff.params(DTProp=30.0))
    assert O.step(dn, Po, O.params(DTProp=30.0)) == 0
    assert np.array_equal(Pg, Po)
    ad.kill()


def test_producers_reject_bad_arguments(gpu):
    import torch
    d = domain("coast")
    ad = advdiff.AdvectionDiffusion(d)
    ad.set_hydro()
    z = torch.zeros(d.shape3, dtype=torch.float64, device="cuda")
    z2 = torch.zeros(d.shape2, dtype=torch.float64, device="cuda")
    with pytest.raises(advdiff.N.MohidAdError) as e:
        ad.geometry(z, z2, z2, faces_option=1)
    assert e.value.code == 3
    with pytest.raises(advdiff.N.MohidAdError) as e:
        ad.vertical_flux(0.0, var_grid=True)
    assert e.value.code == 3
    ad.kill()


def test_cfg2_cut_producers_match_oracle(gpu):
    """A 96x80x40 cut of the 512x512x40 workload (average face thickness)."""
    import torch
    from mohid_gb300 import configs
    w = configs.cfg2().scaled(ni=96, nj=80)
    d = synth.generate(dataclasses.replace(w.spec))
    a = d.arrays
    ad = advdiff.AdvectionDiffusion(d)
    ad.set_hydro()
    dxx, dyy = grid_lengths(d)
    szz = new_level(d, seed=11)
    ad.geometry(torch.from_numpy(szz).cuda(), torch.from_numpy(dxx).cuda(), torch.from_numpy(dyy).cuda(), 2, True)
    ad.vertical_flux(w.spec.dt, True)
    got = ad.get_fields()
    ad.kill()
    state = {n: a[n].copy() for n in ("DWZ", "DZZ", "VolumeZ", "VolumeZOld", "AreaU", "AreaV")}
    state["DUZ"] = np.zeros(d.shape3)
    state["DVZ"] = np.zeros(d.shape3)
    oracle_geometry(d, szz, state, 2)
    qz = a["Wflux_Z"].copy()
    dn = synth.Domain(spec=d.spec, arrays=dict(a, VolumeZ=state["VolumeZ"], VolumeZOld=state["VolumeZOld"]))
    O.vertical_flux(dn, qz, w.spec.dt, True)
    for n in ("DWZ", "DZZ", "VolumeZ", "VolumeZOld", "AreaU", "AreaV"):
        assert np.array_equal(got[n], state[n]), n
    assert np.array_equal(got["Wflux_Z"], qz)


def test_bound_device_arrays(gpu):
    """mohid_ad_bind_hydro_dev: the instance reads the caller's device arrays in
    place (no copy), the producers write into them, a new bind after a change
    marks a new state for the batched form, and a later copy upload returns
    the field to the instance's own storage."""
    import torch
    d = domain("open")
    a = d.arrays
    ad = advdiff.AdvectionDiffusion(d)
    ad.set_hydro()
    dev = {n: torch.from_numpy(a[n].copy()).cuda() for n in synth.F3}
    ad.set_fields(dev, bind=True)
    pd = dict(DTProp=d.spec.dt, AdvMethodH=4, TVDLimitationH=4, Upwind2H=1)
    P = d.tracer(3, 2.0, 0.5, seed=3)
    ref = d.reference(2.0, 0.2, seed=4)
    Pg, Po = P.copy(), P.copy()
    ad.step(Pg, advdiff.params(BoundaryCondition=1, **pd), ReferenceProp=ref)
    assert O.step(d, Po, O.params(BoundaryCondition=1, **pd), ReferenceProp=ref) == 0
    assert np.array_equal(Pg, Po)
    # the producers write the bound arrays
    dxx, dyy = grid_lengths(d)
    szz = new_level(d, seed=7)
    ad.geometry(torch.from_numpy(szz).cuda(), torch.from_numpy(dxx).cuda(), torch.from_numpy(dyy).cuda(), 3, True)
    ad.vertical_flux(d.spec.dt, True)
    torch.cuda.synchronize()
    prod = ad.get_fields()
    for n in ("VolumeZ", "VolumeZOld", "Wflux_Z"):
        assert np.array_equal(dev[n].cpu().numpy(), prod[n]), n
    # the caller changes a bound array in place and binds again: the batched
    # form sees the new state
    b = batched.Batch(ad, 1)
    b.set_tracer(0, P)
    b.set_reference(0, ref)
    b.step(advdiff.params(BoundaryCondition=1, **pd), nsteps=1)
    dev["Wflux_X"].mul_(0.5)
    ad.set_fields({"Wflux_X": dev["Wflux_X"]}, bind=True)
    b.step(advdiff.params(BoundaryCondition=1, **pd), nsteps=1)
    b.sync()
    g = b.get_tracer(0)
    b.destroy()
    dn1 = synth.Domain(spec=d.spec, arrays=dict(a, **{n: prod[n] for n in synth.F3}))
    dn2 = synth.Domain(spec=d.spec, arrays=dict(dn1.arrays, Wflux_X=prod["Wflux_X"] * 0.5))
    Q = P.copy()
    assert O.step(dn1, Q, O.params(BoundaryCondition=1, **pd), ReferenceProp=ref) == 0
    assert O.step(dn2, Q, O.params(BoundaryCondition=1, **pd), ReferenceProp=ref) == 0
    wp = d.water_mask()
    assert np.linalg.norm(g[wp] - Q[wp]) / np.linalg.norm(Q[wp]) <= 1e-6
    # a copy upload of one field stops borrowing it; the others stay bound
    qx = a["Wflux_X"] * 0.25
    ad.set_fields({"Wflux_X": qx})
    dev["Wflux_X"].zero_()
    got = ad.get_fields()
    assert np.array_equal(got["Wflux_X"], qx)
    assert np.array_equal(got["VolumeZ"], dev["VolumeZ"].cpu().numpy())
    ad.kill()
    del dev
