"""Host-side failure handling that needs no GPU (CPU only).

Without a CUDA device every generation entry point must fail loudly -- NaN
output, a status from fnGetLastError -- never compute on the CPU.
"""
import numpy as np
import pytest

from tests import trees


def no_cuda_device():
    import ctypes
    try:
        rt = ctypes.CDLL("libcudart.so")
        n = ctypes.c_int(0)
        return rt.cudaGetDeviceCount(ctypes.byref(n)) != 0 or n.value == 0
    except OSError:
        return True


needs_no_gpu = pytest.mark.skipif(not no_cuda_device(), reason="checks the no-device path")


@needs_no_gpu
def test_generation_without_device_fails_loudly(native):
    node = trees.to_product(trees.simplex_c0())
    with pytest.raises(native.FastNoiseError) as e:
        node.gen_uniform_grid((0, 0, 0), (4, 4, 4), (1, 1, 1), 1)
    assert e.value.code == -3
    out = np.zeros(8, np.float32)
    mm = np.zeros(2, np.float32)
    L = native.lib()
    L.fnGenUniformGrid2D(node.handle, out.ctypes.data_as(native._FP), 0, 0, 4, 2, 1, 1, 1, mm.ctypes.data_as(native._FP))
    assert np.isnan(out).all() and np.isnan(mm).all()
    assert L.fnGetLastError() != 0


@needs_no_gpu
def test_server_without_device_reports_error(native):
    with pytest.raises(native.FastNoiseError):
        native.Server(pool_bytes=1 << 20)


def test_invalid_arguments(native):
    L = native.lib()
    out = np.zeros(4, np.float32)
    L.fnGenUniformGrid2D(None, out.ctypes.data_as(native._FP), 0, 0, 2, 2, 1, 1, 1, None)
    assert L.fnGetLastError() == -1 and np.isnan(out).all()
    assert L.fnGenBatchDevice(None, 3, None, 0) == -1
    assert L.fnServerSubmit(None, None, None) == -1
    assert L.fnServerPoll(None, 1) == -1
