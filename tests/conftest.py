import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")


@pytest.fixture(scope="session")
def built():
    """Build libpfdtd.so and the oracle once per session."""
    import __graft_entry__ as g
    g.build()
    return True


@pytest.fixture(scope="session")
def lib(built):
    from parallelfdtd_gb300 import _lib
    return _lib.load()


@pytest.fixture(scope="session")
def gpu(lib):
    """The GPU tests run on a CUDA box; elsewhere they fail loudly rather than
    fall back to a CPU path."""
    import ctypes
    n = ctypes.c_int()
    lib.pfdtd_device_count(ctypes.byref(n))
    if n.value < 1:
        pytest.fail("no CUDA device visible: -m gpu tests need the GPU")
    return n.value
