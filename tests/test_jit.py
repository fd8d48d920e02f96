"""Run-time specialised kernels (fnJitCompile): the generated straight-line CUDA
compiles for sm_103a for every node kind in 2D/3D/4D (NVRTC runs on the host, so
that part needs no GPU), and on the GPU its results equal the interpreter's bit
for bit on every driver, alone and in batches."""
import numpy as np
import pytest

from oracle.oracle import OracleTree
from oracle.tree import N
from tests import chunkmix, trees
from tests.parity import assert_parity
from tests.test_gpu_parity import COMPOSITE, GRID, SINGLE

ALL = {**SINGLE, **COMPOSITE}


@pytest.mark.parametrize("dim", [2, 3, 4])
def test_every_node_kind_compiles(native, dim):
    fn = native
    pairs = [(trees.to_product(m()), dim) for m in ALL.values()]
    assert fn.jit_check(pairs) > 0


def test_batch_kernel_variants_compile(native):
    """The other variants of the per-tree batch kernels (block size, register bound, points in
    flight per thread), which the autotuner builds and times, compile for sm_103a."""
    fn = native
    pairs = [(trees.to_product(m()), 3) for m in trees.MIX_TREES] + [(trees.to_product(trees.terrain_c2()), 4),
                                                                       (trees.to_product(trees.cellular_value_tree()), 2)]
    assert fn.jit_check_batch_variants(pairs) > 0


def test_jit_rejects_bad_arguments(native):
    fn = native
    with pytest.raises(fn.FastNoiseError):
        fn.jit_check([(trees.to_product(trees.simplex_c0()), 5)])


@pytest.fixture(scope="module")
def jit_all(gpu):
    """Every test tree specialised in 2D/3D/4D (one module per dimensionality)."""
    fn = gpu
    nodes = {name: trees.to_product(m()) for name, m in ALL.items()}
    for dim in (2, 3, 4):
        fn.jit_compile([(n, dim) for n in nodes.values()])
    yield fn, nodes
    fn.set_jit_enabled(True)


def _both(fn, call):
    """Run `call` with the specialised kernels, then with the interpreter only."""
    fn.set_jit_enabled(True)
    a = call()
    fn.set_jit_enabled(False)
    try:
        b = call()
    finally:
        fn.set_jit_enabled(True)
    return a, b


def _same(a, b, label):
    (ga, ma), (gb, mb) = a, b
    assert np.array_equal(np.asarray(ga).view(np.uint32), np.asarray(gb).view(np.uint32)), label
    assert np.array_equal(np.asarray(ma, np.float32).view(np.uint32), np.asarray(mb, np.float32).view(np.uint32)), label


@pytest.mark.gpu
@pytest.mark.parametrize("dim", [2, 3, 4])
@pytest.mark.parametrize("name", sorted(ALL))
def test_jit_grid_matches_interpreter(jit_all, name, dim):
    fn, nodes = jit_all
    off, cnt, st = GRID[dim]
    a, b = _both(fn, lambda: nodes[name].gen_uniform_grid(off, cnt, st, 1337))
    _same(a, b, f"{name} {dim}D")


@pytest.mark.gpu
@pytest.mark.parametrize("dim", [2, 3, 4])
def test_jit_positions_match_interpreter(jit_all, dim):
    fn, nodes = jit_all
    rng = np.random.default_rng(dim)
    pos = [rng.uniform(-1e4, 1e4, 3001).astype(np.float32) for _ in range(dim)]
    for name in ("Simplex", "CellularDistanceSub", "Terrain", "WarpProgressive", "DomainRotate"):
        a, b = _both(fn, lambda: nodes[name].gen_position_array(pos, (0.5,) * dim, -9))
        _same(a, b, f"{name} {dim}D positions")
    big = [rng.uniform(-1e4, 1e4, 700001).astype(np.float32) for _ in range(dim)]
    a, b = _both(fn, lambda: nodes["Simplex"].gen_position_array(big, (0.5,) * dim, 3))
    _same(a, b, f"Simplex {dim}D 700001 positions")


@pytest.mark.gpu
def test_jit_tileable_matches_oracle(jit_all):
    from oracle.oracle import OracleTree
    fn, nodes = jit_all
    root = trees.terrain_c2()
    g, gmm = nodes["Terrain"].gen_tileable_2d((96, 80), (1.0, 1.0), 7)
    o, omm = OracleTree(root).tileable(96, 80, 1.0, 1.0, 7)
    assert_parity(g, gmm, o, omm, label="terrain tileable (specialised)")


@pytest.mark.gpu
@pytest.mark.parametrize("cnt", [(1, 1, 1), (5, 3, 2), (129, 1, 1), (16, 16, 16), (33, 17, 9), (97, 89, 73)])
def test_jit_ragged_grids(jit_all, cnt):
    """Chunk tails: sizes that are not multiples of the warp chunk (32 points per
    warp for small calls, 128 with float4 stores from about 0.6 M points on)."""
    fn, nodes = jit_all
    a, b = _both(fn, lambda: nodes["FBm"].gen_uniform_grid((-3.0, 2.0, 1.0), cnt, (1.0, 1.0, 1.0), 42))
    _same(a, b, str(cnt))


@pytest.mark.gpu
def test_jit_batch_matches_interpreter(gpu):
    torch = pytest.importorskip("torch")
    fn = gpu
    nodes = [trees.to_product(m()) for m in trees.MIX_TREES]
    fn.jit_compile([(n, d) for n in nodes for d in (2, 3)])
    chunks = chunkmix.make_mix(64, seed=5, sizes=[(16, 16, 16), (9, 7, 5), (32, 32), (50, 3), (0, 4, 4)])

    def run():
        outs, reqs, mms = [], [], []
        for c in chunks:
            out = torch.empty(max(c.points, 1), dtype=torch.float32, device="cuda")
            mm = np.zeros(2, np.float32)
            kind = fn.KIND_GRID3D if len(c.count) == 3 else fn.KIND_GRID2D
            reqs.append(fn.make_request(nodes[c.tree], kind, out.data_ptr(), c.seed, c.count, c.offset, (1, 1, 1, 1), minmax=mm))
            outs.append(out)
            mms.append(mm)
        fn.autotune_batch(reqs)                      # several launches of one signature: graph updates
        for _ in range(3):
            fn.gen_batch(reqs, sync=True)
        fn.gen_batch(reqs, sync=True, graph=False)   # the same work as plain stream launches
        return [o.cpu().numpy()[:c.points] for o, c in zip(outs, chunks)], mms

    (ja, jm), (ia, im) = _both(fn, run)
    run()
    info = fn.batch_info()
    assert info["specialised"] == 1 and info["requests"] == len(chunks) and info["ctas"] > 0
    for c, x, y, mx, my in zip(chunks, ja, ia, jm, im):
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32)), c
        assert np.array_equal(mx.view(np.uint32), my.view(np.uint32)), c


@pytest.mark.gpu
@pytest.mark.parametrize("i0, i1", [(0, 0), (0, 3), (2, 1), (3, 3), (1, 2)])
@pytest.mark.parametrize("dim", [2, 3])
def test_specialised_cellular_distance_slots(gpu, i0, i1, dim):
    """The specialised kernels keep only the sorted distance slots up to max(i0, i1); every
    index pair must still match the oracle."""
    fn = gpu
    root = N("CellularDistance", Feature_Scale=7.0, Return_Type="Index0Sub1")
    root.set("Distance Index 0", i0)
    root.set("Distance Index 1", i1)
    root.set("Distance Function", "Euclidean Squared")
    node = trees.to_product(root)
    fn.jit_compile([(node, dim)])
    count = (40, 24, 9)[:dim]
    offset = (-13.0, 5.5, 2.0)[:dim]
    g, gmm = node.gen_uniform_grid(offset, count, (1.0,) * dim, 99)
    o, omm = OracleTree(root).grid(offset, count, (1.0,) * dim, 99)
    assert_parity(g, gmm, o, omm, label=f"{dim}D indices {i0},{i1}")


@pytest.mark.gpu
def test_automatic_specialisation(gpu):
    """A tree used repeatedly on the interpreter is specialised in the background; its calls
    then run the specialised kernels with the same results."""
    fn = gpu
    root = N("FractalRidged", Source=N("Value", Feature_Scale=23.0), Octaves=3)   # a tree no other test specialises
    node = trees.to_product(root)
    off, cnt, st = (3.0, -7.0, 11.0), (48, 40, 36), (1.0, 1.0, 1.0)
    old = fn.set_auto_specialise(3)
    try:
        assert not fn.is_specialised(node, 3)
        first, fmm = node.gen_uniform_grid(off, cnt, st, 5)
        for _ in range(3):
            node.gen_uniform_grid(off, cnt, st, 5)
        assert fn.auto_specialise_wait(120000)
        assert fn.is_specialised(node, 3)
        again, amm = node.gen_uniform_grid(off, cnt, st, 5)
        assert np.array_equal(first.view(np.uint32), again.view(np.uint32)) and fmm == amm
        o, omm = OracleTree(root).grid(off, cnt, st, 5)
        assert_parity(again, amm, o, omm, label="auto-specialised")
    finally:
        fn.set_auto_specialise(old)


def test_module_cache(native, tmp_path):
    """The on-disk cache of specialised modules: a compile writes each module (batch and
    per-call) once; the same sources later load from the cache; a damaged file is ignored
    and rewritten; with the cache off nothing is read."""
    fn = native
    pairs = [(trees.to_product(N("FractalFBm", Source=N("Perlin", Feature_Scale=31.0), Octaves=2)), 3)]
    fn.jit_set_cache_dir(tmp_path)
    try:
        assert fn.jit_cache_info()["dir"] == str(tmp_path)
        i0 = fn.jit_cache_info()
        size = fn.jit_check(pairs)
        i1 = fn.jit_cache_info()
        assert (i1["misses"] - i0["misses"], i1["hits"] - i0["hits"]) == (2, 0)
        files = sorted(tmp_path.glob("*.cubin"))
        assert len(files) == 2 and not list(tmp_path.glob("*.tmp*"))
        assert fn.jit_check(pairs) == size
        i2 = fn.jit_cache_info()
        assert (i2["misses"] - i1["misses"], i2["hits"] - i1["hits"]) == (0, 2)
        whole = files[0].read_bytes()
        files[0].write_bytes(whole[: len(whole) // 2])
        assert fn.jit_check(pairs) == size
        i3 = fn.jit_cache_info()
        assert (i3["misses"] - i2["misses"], i3["hits"] - i2["hits"]) == (1, 1)
        assert files[0].read_bytes() == whole
        fn.jit_set_cache_dir(None)
        assert fn.jit_cache_info()["dir"] == ""
        fn.jit_check(pairs)
        i4 = fn.jit_cache_info()
        assert (i4["misses"] - i3["misses"], i4["hits"] - i3["hits"]) == (2, 0)
    finally:
        fn.jit_set_cache_dir(None)


_CACHE_CHILD = r"""
import sys, numpy as np
sys.path.insert(0, sys.argv[1])
import fastnoise2_gb300 as fn
from oracle.tree import N
from tests import trees
fn.jit_set_cache_dir(sys.argv[2])
import torch
node = trees.to_product(N("FractalRidged", Source=N("Simplex", Feature_Scale=17.0), Octaves=3))
other = trees.to_product(N("CellularDistance", Feature_Scale=13.0))
args = ((2.0, -5.0, 9.0), (40, 36, 30), (1.0, 1.0, 1.0), 11)
out = torch.empty(40 * 36 * 30, dtype=torch.float32, device="cuda")
batch = [fn.make_request(other, fn.KIND_GRID3D, out.data_ptr(), 12, args[1], args[0], (1, 1, 1))]
if sys.argv[3] == "warm":                      # specialise in the background, which writes the cache
    fn.set_auto_specialise(1)
    node.gen_uniform_grid(*args)
    fn.gen_batch(batch, sync=True)
    assert fn.auto_specialise_wait(120000) and fn.is_specialised(node, 3) and fn.is_specialised(other, 3)
else:                                          # a fresh process: specialised from the first call
    fn.set_auto_specialise(0)
    assert not fn.is_specialised(node, 3) and not fn.is_specialised(other, 3)
    first, fmm = node.gen_uniform_grid(*args)
    assert fn.is_specialised(node, 3), "per-call: not loaded from the cache"
    fn.gen_batch(batch, sync=True)
    assert fn.batch_info()["specialised"] == 1, "batch: not loaded from the cache"
    assert fn.jit_cache_info()["hits"] == 4
    got = out.cpu().numpy().copy()
    fn.set_jit_enabled(False)
    ref, rmm = node.gen_uniform_grid(*args)
    assert np.array_equal(first.view(np.uint32), ref.view(np.uint32)) and fmm == rmm
    fn.gen_batch(batch, sync=True)
    assert fn.batch_info()["specialised"] == 0
    assert np.array_equal(got.view(np.uint32), out.cpu().numpy().view(np.uint32))
print("ok")
"""


@pytest.mark.gpu
def test_cached_modules_specialise_the_first_call(gpu, tmp_path):
    """Trees specialised by one process run their specialised kernels from the first call
    (per-call and batch) in the next process that uses the same cache directory, with the
    interpreter's results."""
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    for phase in ("warm", "cold"):
        r = subprocess.run([sys.executable, "-c", _CACHE_CHILD, root, str(tmp_path), phase], capture_output=True, text=True,
                           timeout=600, cwd=root)
        assert r.returncode == 0 and r.stdout.strip().endswith("ok"), (phase, r.stdout, r.stderr)


def test_automatic_specialisation_controls(native):
    fn = native
    old = fn.set_auto_specialise(0)
    assert fn.set_auto_specialise(7) == 0
    assert fn.set_auto_specialise(old) == 7
    assert fn.auto_specialise_wait(0)
