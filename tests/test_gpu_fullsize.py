"""Parity at the full sizes the benchmark times, on the paths it times.

Every workload of the benchmark is generated here at its full size through the C-ABI with the
tree's specialised kernels (fnJitCompile, the path bench.py measures), and compared with the
CPU oracle bit for bit, with OutputMinMax equal:

  * FractalFBm(Perlin) 256^3 from (-128, -128, -128), seed 42: device call, host call (the
    slabbed drop-in path) and the interpreter kernel;
  * the terrain tree as GenTileable2D 1024^2 and GenUniformGrid3D 128^3, seed 7;
  * GenUniformGrid4D 32^4 and GenPositionArray3D over 1 M positions uniform in [-1e4, 1e4]^3,
    for each of the eight chunk-mix trees (the serving workload's extra requests);
  * all 4096 requests of the chunk mix in one fnGenBatchDevice launch, and its first 512
    requests through the request server.

Reference drivers: Generator.inl:129-186 (GenUniformGrid3D), :188-254 (4D), :286-316
(GenPositionArray3D), :370-433 (GenTileable2D); OutputMinMax Generator.h:85-105.
Tolerance: bit-exact (tests/parity.py states the 1e-5 absolute fallback, never needed).
"""
import numpy as np
import pytest

from oracle import oracle
from oracle.oracle import OracleTree
from tests import chunkmix, trees
from tests.parity import assert_parity, minmax_equal

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    return torch


@pytest.fixture(scope="module")
def specialised(gpu):
    """Product nodes of every tree used below, with their specialised kernels built."""
    fn = gpu
    nodes = {m.__name__: trees.to_product(m()) for m in trees.MIX_TREES}
    fn.jit_compile([(n, d) for n in nodes.values() for d in (2, 3, 4)])
    fn.set_jit_enabled(True)
    yield fn, nodes
    fn.set_jit_enabled(True)


def device_grid(torch, node, offset, count, step, seed):
    pts = int(np.prod(count))
    out = torch.empty(pts, dtype=torch.float32, device="cuda")
    mm = torch.empty(2, dtype=torch.float32, device="cuda")
    node.gen_uniform_grid_device(out.data_ptr(), offset, count, step, seed, mm.data_ptr())
    torch.cuda.synchronize()
    m = mm.cpu().numpy()
    return out.cpu().numpy(), (float(m[0]), float(m[1]))


def device_array(ptr, n):
    """Copy n floats from a raw device pointer into a numpy array."""
    import ctypes
    host = np.empty(n, np.float32)
    rt = ctypes.CDLL("libcudart.so")
    rt.cudaMemcpy.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
    assert rt.cudaMemcpy(host.ctypes.data, ptr, n * 4, 2) == 0   # cudaMemcpyDeviceToHost
    return host


_ORACLE = {}


def oracle_grid(name, offset, count, step, seed):
    key = ("grid", name, tuple(offset), tuple(count), tuple(step), seed)
    if key not in _ORACLE:
        _ORACLE[key] = OracleTree(getattr(trees, name)()).grid(offset, count, step, seed)
    return _ORACLE[key]


FBM = ("fbm_perlin_c1", (-128.0, -128.0, -128.0), (256, 256, 256), (1.0, 1.0, 1.0), 42)


def test_fbm_perlin_256_device(specialised, torch_cuda):
    fn, nodes = specialised
    name, off, cnt, st, seed = FBM
    assert fn.is_specialised(nodes[name], 3)
    g, gmm = device_grid(torch_cuda, nodes[name], off, cnt, st, seed)
    o, omm = oracle_grid(name, off, cnt, st, seed)
    assert_parity(g, gmm, o, omm, label="FBm(Perlin) 256^3 device, specialised")


def test_fbm_perlin_256_host(specialised):
    """fnGenUniformGrid3D, the drop-in host call (slabs copied while later slabs generate)."""
    fn, nodes = specialised
    name, off, cnt, st, seed = FBM
    g, gmm = nodes[name].gen_uniform_grid(off, cnt, st, seed)
    o, omm = oracle_grid(name, off, cnt, st, seed)
    assert_parity(g, gmm, o, omm, label="FBm(Perlin) 256^3 host, specialised")


def test_fbm_perlin_256_interpreter(specialised, torch_cuda):
    fn, nodes = specialised
    name, off, cnt, st, seed = FBM
    fn.set_jit_enabled(False)
    try:
        g, gmm = device_grid(torch_cuda, nodes[name], off, cnt, st, seed)
    finally:
        fn.set_jit_enabled(True)
    o, omm = oracle_grid(name, off, cnt, st, seed)
    assert_parity(g, gmm, o, omm, label="FBm(Perlin) 256^3 device, interpreter")


def test_terrain_tileable_1024(specialised, torch_cuda):
    fn, nodes = specialised
    node = nodes["terrain_c2"]
    assert fn.is_specialised(node, 4)
    torch = torch_cuda
    out = torch.empty(1024 * 1024, dtype=torch.float32, device="cuda")
    mm = torch.empty(2, dtype=torch.float32, device="cuda")
    node.gen_tileable_2d_device(out.data_ptr(), (1024, 1024), (1.0, 1.0), 7, mm.data_ptr())
    torch.cuda.synchronize()
    m = mm.cpu().numpy()
    o, omm = OracleTree(trees.terrain_c2()).tileable(1024, 1024, 1.0, 1.0, 7)
    assert_parity(out.cpu().numpy(), (float(m[0]), float(m[1])), o, omm, label="terrain tileable 1024^2")
    # the host call (reference signature) gives the same image
    h, hmm = node.gen_tileable_2d((1024, 1024), (1.0, 1.0), 7)
    assert_parity(h, hmm, o, omm, label="terrain tileable 1024^2 host")


def test_terrain_128(specialised, torch_cuda):
    fn, nodes = specialised
    args = ((0.0, 0.0, 0.0), (128, 128, 128), (1.0, 1.0, 1.0), 7)
    g, gmm = device_grid(torch_cuda, nodes["terrain_c2"], *args)
    o, omm = oracle_grid("terrain_c2", *args)
    assert_parity(g, gmm, o, omm, label="terrain 128^3")


MIX_NAMES = [m.__name__ for m in trees.MIX_TREES]


@pytest.mark.parametrize("name", MIX_NAMES)
def test_grid4d_32(specialised, torch_cuda, name):
    """GenUniformGrid4D 32^4 (1,048,576 points), the serving workload's 4D request."""
    fn, nodes = specialised
    args = ((-16.0, 48.0, -80.0, 5.0), (32, 32, 32, 32), (1.0, 1.0, 1.0, 1.0), 20261203)
    g, gmm = device_grid(torch_cuda, nodes[name], *args)
    o, omm = oracle_grid(name, *args)
    assert_parity(g, gmm, o, omm, label=f"{name} 32^4")


@pytest.fixture(scope="module")
def million_positions():
    rng = np.random.default_rng(20261203)
    return [rng.uniform(-1e4, 1e4, 1 << 20).astype(np.float32) for _ in range(3)]


@pytest.mark.parametrize("name", MIX_NAMES)
def test_positions_1m(specialised, torch_cuda, million_positions, name):
    """GenPositionArray3D over 1 M positions uniform in [-1e4, 1e4]^3, device arrays."""
    fn, nodes = specialised
    torch = torch_cuda
    pos = million_positions
    dpos = [torch.from_numpy(p).cuda() for p in pos]
    out = torch.empty(1 << 20, dtype=torch.float32, device="cuda")
    mm = torch.empty(2, dtype=torch.float32, device="cuda")
    nodes[name].gen_position_array_device(out.data_ptr(), 1 << 20, [p.data_ptr() for p in dpos], (0.5, -3.0, 7.25), 99,
                                          mm.data_ptr())
    torch.cuda.synchronize()
    m = mm.cpu().numpy()
    o, omm = OracleTree(getattr(trees, name)()).positions(pos, (0.5, -3.0, 7.25), 99)
    assert_parity(out.cpu().numpy(), (float(m[0]), float(m[1])), o, omm, label=f"{name} 1M positions")


@pytest.fixture(scope="module")
def mix_oracle():
    """The whole 4096-request chunk mix on the oracle: one contiguous output, per-request min/max."""
    chunks = chunkmix.make_mix(4096)
    otrees = [OracleTree(m()) for m in trees.MIX_TREES]
    pts = sum(c.points for c in chunks)
    out = np.empty(pts, np.float32)
    mm = np.zeros((len(chunks), 2), np.float32)
    reqs, off = [], 0
    for k, c in enumerate(chunks):
        kind = oracle.KIND_GRID3D if len(c.count) == 3 else oracle.KIND_GRID2D
        reqs.append(oracle.request(otrees[c.tree], kind, out[off:off + c.points], mm[k], c.seed, c.count, c.offset,
                                   (1.0,) * len(c.count)))
        off += c.points
    oracle.gen_requests(reqs)
    return chunks, out, mm


def mix_requests(fn, torch, chunks, nodes, base, minmax):
    """Requests whose outputs lie back to back from device address `base`; base None = every
    output NULL (the request server then carves it from its pool)."""
    reqs, off = [], 0
    for k, c in enumerate(chunks):
        kind = fn.KIND_GRID3D if len(c.count) == 3 else fn.KIND_GRID2D
        out = 0 if base is None else base + 4 * off
        reqs.append(fn.make_request(nodes[MIX_NAMES[c.tree]], kind, out, c.seed, c.count, c.offset,
                                    (1, 1, 1, 1), minmax=None if minmax is None else minmax[k]))
        off += c.points
    return reqs


def compare_mix(chunks, got, gmm, ref, rmm, label):
    same = got.view(np.uint32) == ref.view(np.uint32)
    if not same.all():
        # name the first request that differs
        off = 0
        for k, c in enumerate(chunks):
            seg = slice(off, off + c.points)
            if not same[seg].all():
                assert_parity(got[seg], tuple(gmm[k]), ref[seg], tuple(rmm[k]), label=f"{label}: request {k} {c}")
            off += c.points
    for k in range(len(chunks)):
        assert minmax_equal(tuple(map(float, gmm[k])), tuple(map(float, rmm[k]))), (label, k, gmm[k], rmm[k])


def test_chunk_mix_4096_batched(specialised, torch_cuda, mix_oracle):
    """All 4096 requests (394 M points) in one fnGenBatchDevice launch, as the benchmark runs them."""
    fn, nodes = specialised
    torch = torch_cuda
    chunks, ref, rmm = mix_oracle
    pts = len(ref)
    out = torch.empty(pts, dtype=torch.float32, device="cuda")
    gmm = np.zeros((len(chunks), 2), np.float32)
    reqs = mix_requests(fn, torch, chunks, nodes, out.data_ptr(), gmm)
    arr = fn.request_array(reqs)
    fn.gen_batch(arr, sync=True)
    info = fn.batch_info()
    assert info["requests"] == 4096 and info["specialised"] == 1 and info["points"] == pts
    compare_mix(chunks, out.cpu().numpy(), gmm, ref, rmm, "chunk mix batched")


def test_chunk_mix_512_served(specialised, torch_cuda, mix_oracle):
    """The first 512 requests of the mix through the request server (outputs from its pool)."""
    fn, nodes = specialised
    torch = torch_cuda
    chunks, ref, rmm = mix_oracle
    n = 512
    chunks = chunks[:n]
    pts = sum(c.points for c in chunks)
    srv = fn.Server(pool_bytes=4 * pts + (64 << 20), streams=3, max_batch_requests=128)
    try:
        reqs = mix_requests(fn, torch, chunks, nodes, None, None)
        assert all(r.out is None for r in reqs)
        tickets = srv.submit_many(reqs)
        got = np.empty(pts, np.float32)
        gmm = np.zeros((n, 2), np.float32)
        off = 0
        for k, (c, t) in enumerate(zip(chunks, tickets)):
            mn, mx, ptr = srv.wait(t, timeout_ms=60000)   # ptr: the output's block of the server's pool
            gmm[k] = (mn, mx)
            got[off:off + c.points] = device_array(ptr, c.points)
            srv.release(t)
            off += c.points
        assert srv.stats()["completed"] == n
    finally:
        srv.close()
    compare_mix(chunks, got, gmm, ref[:pts], rmm[:n], "chunk mix served")
