import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def gpu_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def native_lib():
    from pyvr_gb300 import _native
    return _native.load()


@pytest.fixture(scope="session", autouse=True)
def exact_arithmetic():
    """The GPU tests compare renders with the oracle bit for bit, so they run
    the exact arithmetic; tests of the fast arithmetic (the library's default)
    switch to it with ``pyvr_gb300.batch.arithmetic("fast")``."""
    try:
        from pyvr_gb300.batch import set_arithmetic
        set_arithmetic("exact")
    except Exception:  # no library (CPU-only checks that do not need it)
        pass
    yield
