import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (run on the GB300 box)")
    config.addinivalue_line("markers", "slow: takes more than a few seconds on the CPU")


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:  # pragma: no cover
        return False


HAS_GPU = _has_gpu()


@pytest.fixture(scope="session")
def lib():
    from ctbangbang_gb300 import lib as _lib
    from ctbangbang_gb300 import build
    build.build()
    return _lib.load()


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import oracle as _o
    return _o.oracle()


@pytest.fixture(scope="session")
def ref_lib():
    from oracle import oracle as _o
    r = _o.reference()
    if r is None:
        pytest.skip("reference CPU build (oracle/_ref) not available on this machine")
    return r


@pytest.fixture
def gpu_required():
    if not HAS_GPU:
        pytest.skip("no CUDA device")
