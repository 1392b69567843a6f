"""Shared fixtures: build the native libraries once per session, seeded domains."""
import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def _has_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if _has_gpu():
        return
    skip = pytest.mark.skip(reason="no CUDA GPU in this environment")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def built():
    from mohid_gb300 import build as B
    from oracle import oracle as O
    B.build()
    O.build()
    return True


@pytest.fixture(scope="session")
def gpu(built):
    import torch
    assert torch.cuda.is_available()
    torch.cuda.init()
    return torch.device("cuda:0")
