"""Failure detection through the C-ABI, injected on the host (no GPU fault).

* non-finite input: the step's device status word reports it
  (MOHID_AD_ERR_NONFINITE), in the plain and the batched form;
* allocation failure: the test hook fails the n-th device allocation; every
  allocating entry point returns MOHID_AD_ERR_ALLOC, releases what it had,
  and works again afterwards;
* bounded waits: the step kernels' stage wait, on a barrier nothing completes,
  gives up and reports MOHID_AD_ERR_TIMEOUT instead of hanging.
"""
import ctypes as C

import numpy as np
import pytest

from mohid_gb300 import _native as N
from mohid_gb300 import advdiff, batched
from oracle import oracle as O
from tests.cases import domain

pytestmark = pytest.mark.gpu
NONFINITE, ALLOC, TIMEOUT = 7, 8, 10


def _fail_alloc(after):
    st = C.c_int(0)
    N.check(N.ad_lib().mohid_ad_debug_fail_alloc(C.byref(C.c_int(after)), C.byref(st)), "fail_alloc")


def test_nonfinite_input_reported_plain(gpu):
    d = domain("coast")
    P = d.tracer(3, 1.0, 0.5, seed=1)
    wp = d.water_mask()
    k, j, i = (int(x[0]) for x in np.nonzero(wp))
    P[k, j, i] = np.nan
    ad = advdiff.AdvectionDiffusion(d)
    ad.set_hydro()
    with pytest.raises(advdiff.N.MohidAdError) as ei:
        ad.step(P, advdiff.params(DTProp=30.0))
    assert ei.value.code == NONFINITE
    # the instance stays usable
    Q = d.tracer(3, 1.0, 0.5, seed=1)
    Qo = Q.copy()
    ad.step(Q, advdiff.params(DTProp=30.0))
    assert O.step(d, Qo, O.params(DTProp=30.0)) == 0
    assert np.array_equal(Q, Qo)
    ad.kill()


def test_nonfinite_input_reported_batched(gpu):
    d = domain("zlevel")
    P = d.tracer(3, 1.0, 0.5, seed=1)
    wp = d.water_mask()
    k, j, i = (int(x[0]) for x in np.nonzero(wp))
    P[k, j, i] = np.inf
    ad = advdiff.AdvectionDiffusion(d)
    ad.set_hydro()
    b = batched.Batch(ad, 1)
    b.set_tracer(0, P)
    b.step(advdiff.params(DTProp=30.0), nsteps=2)
    with pytest.raises(advdiff.N.MohidAdError) as ei:
        b.sync()
    assert ei.value.code == NONFINITE
    b.destroy()
    ad.kill()


@pytest.mark.parametrize("after", [1, 2, 5, 9, 17, 30, 45])
def test_allocation_failure_is_clean(gpu, after):
    d = domain("open")
    # plain instance creation
    _fail_alloc(after)
    try:
        ad = advdiff.AdvectionDiffusion(d)
    except advdiff.N.MohidAdError as e:
        assert e.code == ALLOC
        ad = None
    _fail_alloc(0)
    if ad is None:
        ad = advdiff.AdvectionDiffusion(d)
    ad.set_hydro()
    # batched instance creation
    _fail_alloc(after)
    try:
        b = batched.Batch(ad, 3, storage=1)
    except advdiff.N.MohidAdError as e:
        assert e.code == ALLOC
        b = None
    _fail_alloc(0)
    if b is None:
        b = batched.Batch(ad, 3, storage=1)
    # the instances work after the failure
    P = d.tracer(3, 1.0, 0.5, seed=2)
    for t in range(3):
        b.set_tracer(t, P)
    b.step(advdiff.params(DTProp=30.0), nsteps=2)
    b.sync()
    assert np.all(np.isfinite(b.get_tracer(0)[d.water_mask()]))
    Q, Qo = P.copy(), P.copy()
    ad.step(Q, advdiff.params(DTProp=30.0))
    assert O.step(d, Qo, O.params(DTProp=30.0)) == 0
    assert np.array_equal(Q, Qo)
    b.destroy()
    ad.kill()


def test_allocation_failure_on_first_use(gpu):
    """Buffers allocated on first use (implicit horizontal system, cell fluxes)."""
    d = domain("zlevel")
    ad = advdiff.AdvectionDiffusion(d)
    ad.set_hydro()
    P = d.tracer(3, 1.0, 0.5, seed=3)
    for pd in (dict(ImpExp_AdvXX=1.0), dict(CellFluxes=1)):
        _fail_alloc(1)
        Q = P.copy()
        with pytest.raises(advdiff.N.MohidAdError) as ei:
            ad.step(Q, advdiff.params(DTProp=30.0, **pd))
        assert ei.value.code == ALLOC
        assert np.array_equal(Q, P)
        _fail_alloc(0)
        Q, Qo = P.copy(), P.copy()
        ad.step(Q, advdiff.params(DTProp=30.0, **pd))
        assert O.step(d, Qo, O.params(DTProp=30.0, **pd)) == 0
        assert np.array_equal(Q, Qo)
    ad.kill()


@pytest.mark.parametrize("polls", [1, 4096])
def test_bounded_wait_gives_up(gpu, polls):
    st = C.c_int(0)
    rc = N.ad_lib().mohid_ad_debug_wait_probe(C.byref(C.c_int(polls)), C.byref(st))
    assert rc == TIMEOUT
    # the context is still usable
    d = domain("coast")
    ad = advdiff.AdvectionDiffusion(d)
    ad.set_hydro()
    Q = d.tracer(3, 1.0, 0.5, seed=4)
    Qo = Q.copy()
    ad.step(Q, advdiff.params(DTProp=30.0))
    assert O.step(d, Qo, O.params(DTProp=30.0)) == 0
    assert np.array_equal(Q, Qo)
    ad.kill()
