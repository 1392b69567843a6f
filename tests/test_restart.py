"""Restart files of a batched property group (mohid_gb300.restart), with a
stand-in for the batch: the format needs no GPU."""
import numpy as np
import pytest

from mohid_gb300 import restart


class _Domain:
    shape3 = (4, 5, 6)


class _Ad:
    domain = _Domain()


class _Batch:
    """What restart uses of mohid_gb300.batched.Batch: ad.domain.shape3, nt,
    get_tracer, set_tracer."""

    def __init__(self, nt, seed=0):
        self.ad, self.nt = _Ad(), nt
        rng = np.random.default_rng(seed)
        self.fields = [rng.standard_normal(_Domain.shape3) for _ in range(nt)]

    def get_tracer(self, t):
        return self.fields[t].copy()

    def set_tracer(self, t, P):
        assert P.dtype == np.float64 and P.flags.c_contiguous and P.shape == _Domain.shape3
        self.fields[t] = P.copy()


def test_roundtrip(tmp_path):
    a, b = _Batch(3, seed=1), _Batch(3, seed=2)
    restart.save(a, tmp_path / "wp", step=1234, names=["temperature", "salinity", "age"])
    step, names = restart.load(b, tmp_path / "wp")
    assert step == 1234 and names == ["temperature", "salinity", "age"]
    for x, y in zip(a.fields, b.fields):
        assert np.array_equal(x, y)


def test_rejects_another_batch(tmp_path):
    restart.save(_Batch(2), tmp_path / "wp.npz", step=1)
    with pytest.raises(restart.RestartError):
        restart.load(_Batch(3), tmp_path / "wp.npz")           # tracer count
    other = _Batch(2)
    other.ad = type("A", (), {"domain": type("D", (), {"shape3": (4, 5, 7)})()})()
    with pytest.raises(restart.RestartError):
        restart.load(other, tmp_path / "wp.npz")               # grid
    with pytest.raises(restart.RestartError):
        restart.save(_Batch(2), tmp_path / "x", step=0, names=["one"])
