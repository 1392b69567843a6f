"""The allocation-free mass budget against the existing (allocating) budget.

mohid_ad_mass_f64_noalloc serves callers that cannot allocate device memory
when they need a budget (their memory belongs to another allocator, or they
must not synchronise inside a time step); its scratch is a fixed device array.
Its result must equal the batched form's budget (mohid_ad_batched_mass) of the
same field within the budget tolerance of the other tests (1e-14 relative),
on two calls in a row sharing that scratch.  This file is collected last.
"""
import ctypes as C

import numpy as np
import pytest

from mohid_gb300 import _native as N, advdiff, batched
from tests.cases import domain

pytestmark = pytest.mark.gpu
RTOL = 1e-14


def _noalloc(d, P_dev, V_dev, WP_dev, out_dev):
    size = N.T_Size3D(0, d.ni + 1, 0, d.nj + 1, 0, d.nk + 1)
    st = C.c_int(-1)
    rc = N.ad_lib().mohid_ad_mass_f64_noalloc(C.byref(size), C.c_void_p(P_dev.data_ptr()),
                                              C.c_void_p(V_dev.data_ptr()), C.c_void_p(WP_dev.data_ptr()),
                                              C.c_void_p(out_dev.data_ptr()), None, C.byref(st))
    return rc, st.value


@pytest.mark.parametrize("grid", ["zlevel", "coast"])
def test_noalloc_mass_matches_existing_budget_twice(gpu, grid):
    import torch
    d = domain(grid)
    ad = advdiff.AdvectionDiffusion(d)
    ad.set_hydro()
    b = batched.Batch(ad, 1)
    b.set_tracer(0, d.tracer(3, 2.0, 0.5, seed=5))
    b.step(advdiff.params(DTProp=30.0), nsteps=3)
    want = b.mass(0)                                   # existing entry point
    P = torch.from_numpy(b.get_tracer(0)).cuda()
    V = torch.from_numpy(d.arrays["VolumeZ"]).cuda()
    WP = torch.from_numpy(d.arrays["WaterPoints3D"]).cuda()
    b.destroy()
    ad.kill()
    outs = [torch.full((1,), float("nan"), dtype=torch.float64, device="cuda") for _ in range(2)]
    torch.cuda.synchronize()
    lib = N.ad_lib()
    st0 = C.c_int(0)
    for call in range(2):                              # two calls sharing the scratch
        if call == 1:
            # the first (warm-up) call loaded the module holding the scratch;
            # the second must allocate nothing: every allocation of this
            # library fails from here on, and the device's free memory must
            # not change across the call
            N.check(lib.mohid_ad_debug_fail_alloc(C.byref(C.c_int(1)), C.byref(st0)), "fail_alloc")
            free0 = torch.cuda.mem_get_info()[0]
        try:
            rc, st = _noalloc(d, P, V, WP, outs[call])
            assert rc == 0 and st == 0
            torch.cuda.synchronize()
            if call == 1:
                assert torch.cuda.mem_get_info()[0] == free0
        finally:
            if call == 1:
                N.check(lib.mohid_ad_debug_fail_alloc(C.byref(C.c_int(0)), C.byref(st0)), "fail_alloc")
        got = float(outs[call].item())
        assert abs(got - want) <= RTOL * abs(want), (call, got, want)


def test_noalloc_rejects_grids_beyond_its_scratch(gpu):
    import torch
    nj = 8193                                          # one row more than the scratch holds
    size = N.T_Size3D(0, 3, 0, nj + 1, 0, 3)
    dummy = torch.zeros(1, dtype=torch.float64, device="cuda")
    st = C.c_int(-1)
    rc = N.ad_lib().mohid_ad_mass_f64_noalloc(C.byref(size), C.c_void_p(dummy.data_ptr()),
                                              C.c_void_p(dummy.data_ptr()), C.c_void_p(dummy.data_ptr()),
                                              C.c_void_p(dummy.data_ptr()), None, C.byref(st))
    assert rc == 1 and st.value == 1                   # MOHID_AD_ERR_BOUNDS, nothing launched
    assert b"8192" in N.ad_lib().mohid_ad_last_error()
