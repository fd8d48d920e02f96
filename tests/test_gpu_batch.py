"""Batched persistent launch (fnGenBatchDevice): each request's output and min/max
equal the per-call path's, alone and inside a mix of trees, kinds and sizes."""
import numpy as np
import pytest

from oracle.oracle import OracleTree
from tests import chunkmix, trees
from tests.parity import assert_parity

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    return torch


def requests_for(fn, torch, chunks, nodes):
    reqs, outs, mms = [], [], []
    for c in chunks:
        out = torch.empty(c.points, dtype=torch.float32, device="cuda")
        mm = np.zeros(2, np.float32)
        kind = fn.KIND_GRID3D if len(c.count) == 3 else fn.KIND_GRID2D
        reqs.append(fn.make_request(nodes[c.tree], kind, out.data_ptr(), c.seed, c.count, c.offset, (1, 1, 1, 1), minmax=mm))
        outs.append(out)
        mms.append(mm)
    return reqs, outs, mms


@pytest.mark.parametrize("graph", [True, False])
def test_batch_matches_per_call(gpu, torch_cuda, graph):
    fn, torch = gpu, torch_cuda
    sizes = [(16, 16, 16), (9, 7, 5), (32, 32), (50, 3), (1, 1, 1), (0, 4, 4)]
    chunks = chunkmix.make_mix(48, seed=7, sizes=sizes)
    nodes = [trees.to_product(m()) for m in trees.MIX_TREES]
    reqs, outs, mms = requests_for(fn, torch, chunks, nodes)
    fn.gen_batch(reqs, sync=True, graph=graph)
    for c, out, mm in zip(chunks, outs, mms):
        ref, rmm = nodes[c.tree].gen_uniform_grid(c.offset, c.count, (1,) * len(c.count), c.seed)
        got = out.cpu().numpy()
        assert np.array_equal(got.view(np.uint32), ref.view(np.uint32)), c
        assert (mm[0], mm[1]) == rmm, (c, mm, rmm)


def test_batch_against_oracle(gpu, torch_cuda):
    fn, torch = gpu, torch_cuda
    chunks = chunkmix.make_mix(16, seed=11, sizes=[(12, 10, 8), (40, 24)])
    nodes = [trees.to_product(m()) for m in trees.MIX_TREES]
    reqs, outs, mms = requests_for(fn, torch, chunks, nodes)
    fn.gen_batch(reqs, sync=True)
    for c, out, mm in zip(chunks, outs, mms):
        o, omm = OracleTree(trees.MIX_TREES[c.tree]()).grid(c.offset, c.count, (1,) * len(c.count), c.seed)
        assert_parity(out.cpu().numpy(), (float(mm[0]), float(mm[1])), o, omm, label=str(c))


def test_batch_mixed_kinds(gpu, torch_cuda):
    """Tileable and position-array requests ride in the same launch as grids."""
    fn, torch = gpu, torch_cuda
    terrain = trees.to_product(trees.terrain_c2())
    fbm = trees.to_product(trees.fbm_perlin_c1())
    rng = np.random.default_rng(5)
    pos = [torch.tensor(rng.uniform(-1e4, 1e4, 5000).astype(np.float32), device="cuda") for _ in range(3)]
    o1 = torch.empty(64 * 48, device="cuda")
    o2 = torch.empty(5000, device="cuda")
    o3 = torch.empty(20 * 20 * 20, device="cuda")
    m1, m2, m3 = (np.zeros(2, np.float32) for _ in range(3))
    reqs = [fn.make_request(terrain, fn.KIND_TILEABLE2D, o1.data_ptr(), 7, (64, 48), step=(1.0, 1.0), minmax=m1),
            fn.make_request(fbm, fn.KIND_POSITIONS3D, o2.data_ptr(), 42, (5000,), offset=(1.0, 2.0, 3.0),
                            positions=[p.data_ptr() for p in pos], minmax=m2),
            fn.make_request(fbm, fn.KIND_GRID3D, o3.data_ptr(), 3, (20, 20, 20), offset=(-5, -5, -5), minmax=m3)]
    fn.gen_batch(reqs, sync=True)
    t, tmm = terrain.gen_tileable_2d((64, 48), (1.0, 1.0), 7)
    p, pmm = fbm.gen_position_array([x.cpu().numpy() for x in pos], (1.0, 2.0, 3.0), 42)
    g, gmm = fbm.gen_uniform_grid((-5, -5, -5), (20, 20, 20), (1, 1, 1), 3)
    for got, ref, mm, rmm in ((o1, t, m1, tmm), (o2, p, m2, pmm), (o3, g, m3, gmm)):
        assert np.array_equal(got.cpu().numpy().view(np.uint32), ref.view(np.uint32))
        assert (mm[0], mm[1]) == rmm


def test_autotune_and_reuse(gpu, torch_cuda, tmp_path):
    fn, torch = gpu, torch_cuda
    chunks = chunkmix.make_mix(24, seed=3, sizes=[(16, 16, 16), (64, 64)])
    nodes = [trees.to_product(m()) for m in trees.MIX_TREES]
    reqs, outs, mms = requests_for(fn, torch, chunks, nodes)
    fn.autotune_batch(reqs)
    first = [o.clone() for o in outs]
    fn.gen_batch(reqs, sync=True)
    for a, b in zip(first, outs):
        assert torch.equal(a, b)
    path = str(tmp_path / "tune.txt")
    assert fn.lib().fnAutotuneSave(path.encode()) == 0
    assert fn.lib().fnAutotuneLoad(path.encode()) == 0


def test_bad_request_fails_loudly(gpu, torch_cuda):
    fn = gpu
    node = trees.to_product(trees.unsupported_tree())         # rejected by the GPU compiler
    out = torch_cuda.empty(16, device="cuda")
    with pytest.raises(fn.FastNoiseError):
        fn.gen_batch([fn.make_request(node, fn.KIND_GRID2D, out.data_ptr(), 1, (4, 4))])


@pytest.mark.parametrize("mode", ["pinned", "pageable", "pinned-and-pageable", "pageable-written", "block-written"])
def test_batch_host_outputs_match_device_batch(gpu, torch_cuda, mode):
    """fnGenBatchHost: outputs in one page-locked block (contiguous runs copied together),
    separate fresh pageable arrays, or one request outside the page-locked block (all staged:
    slices across both staging buffers, the mix being larger than one 2^25-point slice); and
    separate or contiguous pageable arrays already written (stored into directly by the batch
    kernels where the device reads host page tables); a request larger than a slice and empty
    requests; outputs and min/max equal the device batch's."""
    fn, torch = gpu, torch_cuda
    chunks = chunkmix.make_mix(40, seed=19, sizes=[(128, 128, 64), (96, 80, 70), (0, 5, 5), (17, 3)])
    chunks.append(chunkmix.Chunk(tree=1, count=(384, 320, 300), offset=(-5.0, 7.0, 3.0), seed=77))   # 36.9 M points
    nodes = [trees.to_product(m()) for m in trees.MIX_TREES]
    dreqs, douts, dmms = requests_for(fn, torch, chunks, nodes)
    fn.gen_batch(dreqs, sync=True)
    total = sum(c.points for c in chunks)
    if mode == "block-written":
        block = np.full(max(total, 1), np.nan, np.float32)
    else:
        block = torch.empty(max(total, 1), dtype=torch.float32, pin_memory=True).numpy()
        block[:] = np.nan
    hreqs, houts, hmms, off = [], [], [], 0
    for k, c in enumerate(chunks):
        in_block = mode in ("pinned", "block-written") or (mode == "pinned-and-pageable" and k != 7)
        if in_block:
            out = block[off:off + c.points]
        elif mode == "pageable-written":
            out = np.full(c.points, np.nan, np.float32)
        else:
            out = np.empty(c.points, np.float32)
        off += c.points
        mm = np.zeros(2, np.float32)
        kind = fn.KIND_GRID3D if len(c.count) == 3 else fn.KIND_GRID2D
        hreqs.append(fn.make_request(nodes[c.tree], kind, out.ctypes.data, c.seed, c.count, c.offset, (1, 1, 1, 1), minmax=mm))
        houts.append(out)
        hmms.append(mm)
    fn.gen_batch_host(hreqs)
    info = fn.batch_info()
    assert info["requests"] == len(chunks) and info["points"] == total
    for c, dout, dmm, hout, hmm in zip(chunks, douts, dmms, houts, hmms):
        assert np.array_equal(hout.view(np.uint32), dout.cpu().numpy().view(np.uint32)), c
        assert (hmm[0], hmm[1]) == (dmm[0], dmm[1]), c


def test_batch_host_outputs_across_a_registered_range(gpu, torch_cuda):
    """Host outputs in an application buffer page-locked in part by cudaHostRegister: inside the
    registered bytes, and starting inside them but running past their end (the copy is cut at
    the end of the registered range; the rest goes to pageable memory)."""
    fn, torch = gpu, torch_cuda
    cudart = torch.cuda.cudart()
    node = trees.to_product(trees.MIX_TREES[2]())
    n = 96 * 80 * 70
    buf = np.empty(2 * n + 1024, np.float32)
    assert int(cudart.cudaHostRegister(buf.ctypes.data, (n + 512) * 4, 0)) == 0
    try:
        ref, rmm = node.gen_uniform_grid((1.0, 2.0, 3.0), (96, 80, 70), (1, 1, 1), 5)
        for start in (0, 512, n // 2, n + 1024):    # inside; inside; running past the registered end; pageable
            out = buf[start:start + n]
            out[:] = np.nan
            mm = np.zeros(2, np.float32)
            fn.gen_batch_host([fn.make_request(node, fn.KIND_GRID3D, out.ctypes.data, 5, (96, 80, 70), (1.0, 2.0, 3.0),
                                               (1, 1, 1, 1), minmax=mm)])
            assert np.array_equal(out.view(np.uint32), ref.view(np.uint32)) and (float(mm[0]), float(mm[1])) == rmm
    finally:
        cudart.cudaHostUnregister(buf.ctypes.data)


def test_autotune_picks_a_batch_kernel_variant_per_tree(gpu, torch_cuda, tmp_path):
    """fnAutotuneBatch times every variant of each specialised tree's batch kernel (block size,
    register bound, points in flight per thread) and keeps one per tree; fnAutotuneSave lists the
    choices as "tree" lines.  Every variant gives the same outputs: with a table that forces
    variant v for every tree, the batch equals the per-call results bit for bit."""
    fn, torch = gpu, torch_cuda
    nodes = [trees.to_product(m()) for m in trees.MIX_TREES]
    fn.jit_compile([(n, d) for n in nodes for d in (2, 3)])
    chunks = chunkmix.make_mix(64, seed=13, sizes=[(16, 16, 16), (32, 32, 32), (64, 64), (128, 128)])
    reqs, outs, mms = requests_for(fn, torch, chunks, nodes)
    refs = [nodes[c.tree].gen_uniform_grid(c.offset, c.count, (1,) * len(c.count), c.seed) for c in chunks]
    fn.autotune_batch(reqs)
    path = tmp_path / "tune.txt"
    fn.autotune_save(path)
    lines = path.read_text().splitlines()
    tree_lines = [ln.split() for ln in lines if ln.startswith("tree ")]
    assert len(tree_lines) == len({(c.tree, len(c.count)) for c in chunks})   # one per tree and dimensionality
    n_variants = 5
    for variant in range(n_variants):
        forced = [ln for ln in lines if not ln.startswith("tree ")]
        forced += [f"tree {t[1]} {variant} 0 0 0 1.0" for t in tree_lines]
        path.write_text("\n".join(forced) + "\n")
        fn.autotune_load(path)
        for o in outs:
            o.fill_(float("nan"))
        fn.gen_batch(reqs, sync=True)
        for c, o, mm, (ref, rmm) in zip(chunks, outs, mms, refs):
            assert np.array_equal(o.cpu().numpy().view(np.uint32), ref.view(np.uint32)), (variant, c)
            assert (mm[0], mm[1]) == rmm, (variant, c)
