import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

# Tests choose the kernel tier they exercise (fnJitCompile / fnSetJitEnabled); automatic
# background specialisation stays off unless a test turns it on (tests/test_jit.py does).
os.environ.setdefault("FASTNOISE_AUTO_SPECIALISE", "0")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (runs on the GB300 box)")


@pytest.fixture(scope="session")
def native():
    """The product library, built in-tree if needed (CPU-only calls are fine without a GPU)."""
    from fastnoise2_gb300 import build as b
    b.build()
    import fastnoise2_gb300 as fn
    return fn


@pytest.fixture(scope="session")
def gpu(native):
    import ctypes
    try:
        rt = ctypes.CDLL("libcudart.so")
        n = ctypes.c_int(0)
        if rt.cudaGetDeviceCount(ctypes.byref(n)) != 0 or n.value == 0:
            pytest.fail("no CUDA device: GPU tests must run on a GPU host")
    except OSError:
        pytest.fail("libcudart not loadable")
    return native
