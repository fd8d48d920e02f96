"""Large grids into host memory are generated slab by slab along the outermost axis (each slab's
copy to the host overlapping the next slab's generation).  The output and OutputMinMax must be
those of one launch over the whole grid: positions come from each point's index in the whole
grid, and the slabs' min/max are combined in slab order."""
import numpy as np
import pytest

from oracle.oracle import OracleTree
from tests import trees

pytestmark = pytest.mark.gpu


def device_grid(fn, torch, node, offset, count, step, seed):
    L = fn.lib()
    n = int(np.prod(count))
    out = torch.empty(n, dtype=torch.float32, device="cuda")
    mm = torch.empty(2, dtype=torch.float32, device="cuda")
    f = {3: L.fnGenUniformGrid3DDevice, 4: L.fnGenUniformGrid4DDevice}[len(count)]
    rc = f(node.handle, out.data_ptr(), *map(float, offset), *map(int, count), *map(float, step), int(seed), mm.data_ptr(), None)
    assert rc == 0
    torch.cuda.synchronize()
    return out.cpu().numpy(), tuple(float(v) for v in mm.cpu().numpy())


@pytest.mark.parametrize("jit", [True, False])
@pytest.mark.parametrize("case", [
    ((-100.0, 20.5, -7.0), (200, 160, 300), (1.0, 0.5, 2.0)),           # 9.6 M points, two slabs
    ((3.0, -2.0, 11.0), (257, 129, 300), (0.75, 1.25, 1.0)),            # odd row length: slabs start unaligned
    ((0.0, 0.0, 0.0, 5.0), (64, 48, 40, 70), (1.0, 1.0, 1.0, 1.0)),     # 4D, 8.6 M points
])
def test_slabbed_host_grid_equals_one_launch(gpu, case, jit):
    torch = pytest.importorskip("torch")
    fn = gpu
    offset, count, step = case
    root = trees.fbm_perlin_c1()
    node = trees.to_product(root)
    if jit:
        fn.jit_compile([(node, len(count))])
    old = fn.set_jit_enabled(jit)
    try:
        host, hmm = node.gen_uniform_grid(offset, count, step, 42)
        dev, dmm = device_grid(fn, torch, node, offset, count, step, 42)
    finally:
        fn.set_jit_enabled(old)
    assert np.array_equal(host.view(np.uint32), dev.view(np.uint32))
    assert hmm == dmm
    # spot check against the oracle: the first and last planes of the outermost axis, as
    # one-plane grids at that plane's position (fma(r, step, offset), exact in float64 here)
    plane = int(np.prod(count[:-1]))
    for r in (0, count[-1] - 1):
        pos = float(np.float32(float(r) * float(np.float32(step[-1])) + float(np.float32(offset[-1]))))
        o, _ = OracleTree(root).grid(tuple(offset[:-1]) + (pos,), tuple(count[:-1]) + (1,), step, 42)
        assert np.array_equal(host[r * plane:(r + 1) * plane].view(np.uint32), np.asarray(o, np.float32).view(np.uint32)), r


@pytest.mark.parametrize("jit", [True, False])
def test_host_calls_into_page_locked_memory(gpu, jit):
    """Host outputs the device can store into are written by the kernel directly (no device
    buffer, no copy, no slabs): page-locked memory, and pageable memory whose pages are
    resident where the device reads host page tables.  Outputs and OutputMinMax equal those of
    the same calls into fresh (untouched, so staged) pageable arrays, for grids below and above
    the slab size, tileable images and position arrays, and an application buffer registered
    in part (the call whose output runs past the registered bytes does not store into it as
    page-locked memory)."""
    torch = pytest.importorskip("torch")
    fn = gpu
    root = trees.terrain_c2()
    node = trees.to_product(root)
    if jit:
        fn.jit_compile([(node, d) for d in (2, 3, 4)])
    old = fn.set_jit_enabled(jit)
    try:
        for offset, count, step in [((1.0, 2.0), (300, 200), (1.0, 1.0)), ((-3.0, 4.0, 5.0), (64, 48, 40), (1.0, 0.5, 2.0)),
                                    ((-100.0, 20.5, -7.0), (200, 160, 300), (1.0, 0.5, 2.0)),
                                    ((0.0, 0.0, 0.0, 5.0), (16, 12, 10, 7), (1.0, 1.0, 1.0, 1.0))]:
            n = int(np.prod(count))
            pinned = torch.empty(n, dtype=torch.float32, pin_memory=True).numpy()
            pinned[:] = np.nan
            a, amm = node.gen_uniform_grid(offset, count, step, 42, out=pinned)
            b, bmm = node.gen_uniform_grid(offset, count, step, 42)
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32)) and amm == bmm, count
            touched = np.full(n, np.nan, np.float32)
            c, cmm = node.gen_uniform_grid(offset, count, step, 42, out=touched)
            assert np.array_equal(c.view(np.uint32), b.view(np.uint32)) and cmm == bmm, count
        pinned = torch.empty(96 * 80, dtype=torch.float32, pin_memory=True).numpy()
        a, amm = node.gen_tileable_2d((96, 80), (1.0, 1.0), 7, out=pinned)
        b, bmm = node.gen_tileable_2d((96, 80), (1.0, 1.0), 7)
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)) and amm == bmm
        rng = np.random.default_rng(5)
        xyz = [rng.uniform(-1e4, 1e4, 5000).astype(np.float32) for _ in range(3)]
        pinned = torch.empty(5000, dtype=torch.float32, pin_memory=True).numpy()
        a, amm = node.gen_position_array(xyz, (0.5, 0.25, -1.0), 2024, out=pinned)
        b, bmm = node.gen_position_array(xyz, (0.5, 0.25, -1.0), 2024)
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)) and amm == bmm
        # an application buffer registered in part: inside the registered bytes, and past them
        cudart = torch.cuda.cudart()
        count = (64, 48, 40)
        n = int(np.prod(count))
        buf = np.empty(2 * n + 1024, np.float32)
        assert int(cudart.cudaHostRegister(buf.ctypes.data, (n + 512) * 4, 0)) == 0
        try:
            ref, rmm = node.gen_uniform_grid((-3.0, 4.0, 5.0), count, (1.0, 0.5, 2.0), 42)
            for start in (0, 512, n // 2):
                out = buf[start:start + n]
                out[:] = np.nan
                got, gmm = node.gen_uniform_grid((-3.0, 4.0, 5.0), count, (1.0, 0.5, 2.0), 42, out=out)
                assert np.array_equal(got.view(np.uint32), ref.view(np.uint32)) and gmm == rmm, start
        finally:
            cudart.cudaHostUnregister(buf.ctypes.data)
    finally:
        fn.set_jit_enabled(old)


_STAGED_CHILD = r"""
import sys, numpy as np
sys.path.insert(0, sys.argv[1])
import fastnoise2_gb300 as fn
from tests import trees
node = trees.to_product(trees.terrain_c2())
out = np.full(64 * 48 * 40, np.nan, np.float32)
got, mm = node.gen_uniform_grid((-3.0, 4.0, 5.0), (64, 48, 40), (1.0, 0.5, 2.0), 42, out=out)
rng = np.random.default_rng(5)
xyz = [rng.uniform(-1e4, 1e4, 5000).astype(np.float32) for _ in range(3)]
pos, pmm = node.gen_position_array(xyz, (0.5, 0.25, -1.0), 2024, out=np.full(5000, np.nan, np.float32))
batch = np.full(2 * 32 ** 3, np.nan, np.float32)              # one ordinary array, two requests
bmm = np.zeros(4, np.float32)
fn.gen_batch_host([fn.make_request(node, fn.KIND_GRID3D, batch.ctypes.data + 4 * k * 32 ** 3, 5 + k, (32, 32, 32),
                                   (float(k), 1.0, 2.0), (1, 1, 1), minmax=bmm[2 * k:2 * k + 2]) for k in range(2)])
np.save(sys.argv[2], np.concatenate([got, np.array(mm, np.float32), pos, np.array(pmm, np.float32), batch, bmm]))
"""


def test_host_direct_stores_can_be_turned_off(gpu, tmp_path):
    """FASTNOISE_HOST_DIRECT=0 stages every host output in device memory and copies it (and
    copies position arrays to the device), for the per-call host calls and fnGenBatchHost; the
    results equal the direct stores and in-place position reads of this process."""
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    path = tmp_path / "staged.npy"
    env = dict(os.environ, FASTNOISE_HOST_DIRECT="0")
    r = subprocess.run([sys.executable, "-c", _STAGED_CHILD, root, str(path)], capture_output=True, text=True, timeout=600,
                       cwd=root, env=env)
    assert r.returncode == 0, r.stderr
    staged = np.load(path)
    node = trees.to_product(trees.terrain_c2())
    out = np.full(64 * 48 * 40, np.nan, np.float32)
    got, mm = node.gen_uniform_grid((-3.0, 4.0, 5.0), (64, 48, 40), (1.0, 0.5, 2.0), 42, out=out)
    rng = np.random.default_rng(5)
    xyz = [rng.uniform(-1e4, 1e4, 5000).astype(np.float32) for _ in range(3)]      # resident: read in place
    pos, pmm = node.gen_position_array(xyz, (0.5, 0.25, -1.0), 2024, out=np.full(5000, np.nan, np.float32))
    batch = np.full(2 * 32 ** 3, np.nan, np.float32)          # resident: the batch kernels store into it
    bmm = np.zeros(4, np.float32)
    fn = gpu
    fn.gen_batch_host([fn.make_request(node, fn.KIND_GRID3D, batch.ctypes.data + 4 * k * 32 ** 3, 5 + k, (32, 32, 32),
                                       (float(k), 1.0, 2.0), (1, 1, 1), minmax=bmm[2 * k:2 * k + 2]) for k in range(2)])
    n = got.size
    assert np.array_equal(staged[:n].view(np.uint32), got.view(np.uint32))
    assert (float(staged[n]), float(staged[n + 1])) == mm
    assert np.array_equal(staged[n + 2:n + 2 + 5000].view(np.uint32), pos.view(np.uint32))
    assert (float(staged[n + 5002]), float(staged[n + 5003])) == pmm
    tail = staged[n + 5004:]
    assert np.array_equal(tail[:batch.size].view(np.uint32), batch.view(np.uint32))
    assert np.array_equal(tail[batch.size:].view(np.uint32), bmm.view(np.uint32))
