import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs through libsphgpu.so)")
    config.addinivalue_line("markers", "slow: long-running parity case")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.lib()
    return O


@pytest.fixture(scope="session")
def sphlib():
    """The in-tree CUDA library (built on demand; never a fallback)."""
    from sphugo_gb300 import build
    from sphugo_gb300 import _lib as L
    build.build()
    return L.load()


@pytest.fixture(scope="session")
def gpu(sphlib):
    import ctypes as C
    n = C.c_int32(0)
    rc = sphlib.sph_device_count(C.byref(n))
    if rc != 0 or n.value < 1:
        pytest.fail("no CUDA device visible to libsphgpu.so: the gpu tests need one")
    return sphlib
