"""fnGenUniformGrid3DDeviceNoAlloc: the allocation-free 3D grid entry point.

Its results must equal fnGenUniformGrid3DDevice's bit for bit, also when two
calls run back to back on one stream and the second finds the first call's
program and workspace still in the shared static scratch.  The file is named
so that pytest collects it last: it must pass after the other tests (the
scratch then already holds older contents) and alone in a fresh process (the
first call then does the per-device set-up).
"""
import ctypes

import numpy as np
import pytest

from oracle.tree import N
from tests import trees

FN_ERR_CAPACITY = -4


def _call(fn, entry, node, out_ptr, offset, count, step, seed, mm_ptr, stream=0):
    f = getattr(fn.lib(), entry)
    return f(node._h, ctypes.c_void_p(out_ptr), *map(float, offset), *map(int, count), *map(float, step),
             int(np.int32(seed)), ctypes.c_void_p(mm_ptr), ctypes.c_void_p(stream) if stream else None)


def _deep_chain(links):
    """A tree whose program exceeds the 16 KiB static program area: a chain of Add nodes."""
    node = N("Perlin")
    for i in range(links):
        node = N("Add", LHS=node, RHS=N("Perlin", Seed_Offset=i + 1))
    return node


def test_no_alloc_rejects_oversized_tree(native):
    """Oversized programs are refused before any CUDA call (runs without a GPU)."""
    fn = native
    node = trees.to_product(_deep_chain(400))
    rc = _call(fn, "fnGenUniformGrid3DDeviceNoAlloc", node, 0x1000, (0, 0, 0), (4, 4, 4), (1, 1, 1), 1, 0)
    assert rc == FN_ERR_CAPACITY
    assert "16384" in fn.lib().fnGetLastErrorString().decode()


@pytest.mark.gpu
def test_no_alloc_matches_device_entry_point_twice(gpu):
    torch = pytest.importorskip("torch")
    fn = gpu
    cases = [
        (trees.to_product(trees.terrain_c2()), (-3.5, 7.25, 1.0), (37, 29, 23), (0.75, 1.0, 1.25), 1337),
        (trees.to_product(trees.fbm_perlin_c1()), (100.0, -20.0, 5.5), (64, 48, 40), (1.0, 1.0, 1.0), -77),
    ]
    refs, gots = [], []
    for node, off, cnt, st, seed in cases:
        n = int(np.prod(cnt))
        ref = torch.full((n,), float("nan"), device="cuda")
        ref_mm = torch.zeros(2, device="cuda")
        assert _call(fn, "fnGenUniformGrid3DDevice", node, ref.data_ptr(), off, cnt, st, seed, ref_mm.data_ptr()) == 0
        refs.append((ref, ref_mm))
    torch.cuda.synchronize()
    # two calls in a row on the same (default) stream, no synchronisation between them
    for node, off, cnt, st, seed in cases:
        n = int(np.prod(cnt))
        out = torch.full((n,), float("nan"), device="cuda")
        mm = torch.zeros(2, device="cuda")
        gots.append((out, mm))
    for (node, off, cnt, st, seed), (out, mm) in zip(cases, gots):
        rc = _call(fn, "fnGenUniformGrid3DDeviceNoAlloc", node, out.data_ptr(), off, cnt, st, seed, mm.data_ptr())
        assert rc == 0, fn.lib().fnGetLastErrorString()
    torch.cuda.synchronize()
    for (ref, ref_mm), (out, mm) in zip(refs, gots):
        assert torch.equal(out.view(torch.int32), ref.view(torch.int32))
        assert torch.equal(mm.view(torch.int32), ref_mm.view(torch.int32))


@pytest.mark.gpu
def test_no_alloc_back_to_back_on_a_non_blocking_stream(gpu):
    """Two calls queued on a non-blocking stream with nothing between them: the second call's
    copies into the shared array must wait for the first call's kernel by stream order alone
    (no implicit synchronisation of the legacy default stream helps here)."""
    torch = pytest.importorskip("torch")
    fn = gpu
    cases = [
        (trees.to_product(trees.fbm_perlin_c1()), (-40.0, 12.5, 3.0), (96, 80, 72), (1.0, 1.0, 1.0), 42),
        (trees.to_product(trees.cellular_lookup_tree()), (7.0, -9.0, 100.0), (33, 65, 17), (0.5, 2.0, 1.0), -5),
    ]
    refs = []
    for node, off, cnt, st, seed in cases:
        ref = torch.full((int(np.prod(cnt)),), float("nan"), device="cuda")
        ref_mm = torch.zeros(2, device="cuda")
        assert _call(fn, "fnGenUniformGrid3DDevice", node, ref.data_ptr(), off, cnt, st, seed, ref_mm.data_ptr()) == 0
        refs.append((ref, ref_mm))
    gots = [(torch.full((int(np.prod(c[2])),), float("nan"), device="cuda"), torch.zeros(2, device="cuda")) for c in cases]
    torch.cuda.synchronize()
    stream = torch.cuda.Stream()                     # created with cudaStreamNonBlocking
    for (node, off, cnt, st, seed), (out, mm) in zip(cases, gots):
        rc = _call(fn, "fnGenUniformGrid3DDeviceNoAlloc", node, out.data_ptr(), off, cnt, st, seed, mm.data_ptr(),
                   stream.cuda_stream)
        assert rc == 0, fn.lib().fnGetLastErrorString()
    stream.synchronize()
    for (ref, ref_mm), (out, mm) in zip(refs, gots):
        assert torch.equal(out.view(torch.int32), ref.view(torch.int32))
        assert torch.equal(mm.view(torch.int32), ref_mm.view(torch.int32))
