"""Live trees on the GPU: trees sent over the Node Editor's channel are decoded, compiled and
swapped in (fnLiveTree*), generation with the acquired tree matches the oracle for that tree,
and server requests submitted before a swap finish with the tree they were submitted with."""
import time

import numpy as np
import pytest

from oracle.oracle import OracleTree
from oracle.tree import N, encode
from tests import trees
from tests.parity import assert_parity

pytestmark = pytest.mark.gpu

OFFSET, COUNT, STEP, SEED = (-8.0, 3.0, 17.0), (16, 12, 10), (1.0, 1.0, 1.0), 1337


def tree_a():
    return N("FractalFBm", Source=N("Simplex", Feature_Scale=30.0), Octaves=3)


def tree_b():
    return N("CellularDistance", Feature_Scale=12.0, Return_Type="Index0Sub1")


def tree_c():
    return trees.fbm_perlin_c1()


def check_node(node, root):
    g, gmm = node.gen_uniform_grid(OFFSET, COUNT, STEP, SEED)
    o, omm = OracleTree(root).grid(OFFSET, COUNT, STEP, SEED)
    assert_parity(g, gmm, o, omm, label=encode(root))


@pytest.fixture
def channels(gpu):
    fn = gpu
    editor, app = fn.EditorChannel(), fn.EditorChannel()
    yield editor, app
    app.close()
    editor.close()


def test_update_swaps_and_rejects(gpu, channels):
    fn = gpu
    editor, app = channels
    live = fn.LiveTree(app, encode(tree_a()), dims=(3, 2), poll_ms=0)
    node, v = live.acquire()
    assert v == 1 and node.encode() == encode(tree_a())
    check_node(node, tree_a())
    assert live.update() == 0
    editor.send_selected(encode(tree_b()))
    assert live.update() == 1
    node_b, v = live.acquire()
    assert v == 2 and node_b.encode() == encode(tree_b())
    check_node(node_b, tree_b())
    check_node(node, tree_a())                      # the old tree still works for its holders
    editor.send_selected("@@@ not a tree")
    assert live.update() == -1
    assert live.acquire()[1] == 2 and live.info()["rejected"] == 1
    live.close()


def test_background_polling(gpu, channels):
    fn = gpu
    editor, app = channels
    live = fn.LiveTree(app, encode(tree_a()), dims=(3,), poll_ms=2)
    editor.send_selected(encode(tree_c()))
    deadline = time.time() + 60.0                  # includes NVRTC specialisation of the new tree
    while live.acquire()[1] < 2 and time.time() < deadline:
        time.sleep(0.01)
    node, v = live.acquire()
    assert v == 2, live.info()
    check_node(node, tree_c())
    live.close()


def test_server_requests_keep_their_tree_across_a_swap(gpu, channels):
    fn = gpu
    editor, app = channels
    live = fn.LiveTree(app, encode(tree_a()), dims=(3,), poll_ms=0)
    srv = fn.Server(pool_bytes=64 << 20, streams=2, max_batch_requests=8)
    import ctypes
    rt = ctypes.CDLL("libcudart.so")
    rt.cudaMemcpy.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
    submitted = []
    for round_ in range(3):
        node, v = live.acquire()
        for k in range(6):
            req = fn.make_request(node, fn.KIND_GRID3D, 0, SEED + k, COUNT, OFFSET, (1, 1, 1, 1))
            submitted.append((srv.submit(req), v, SEED + k))
        del node                                      # the server holds its own reference
        editor.send_selected(encode([tree_b, tree_c][round_ % 2]()))
        assert live.update() == 1
    roots = {1: tree_a(), 2: tree_b(), 3: tree_c()}
    n = COUNT[0] * COUNT[1] * COUNT[2]
    for ticket, version, seed in submitted:
        mn, mx, ptr = srv.wait(ticket, timeout_ms=60000)
        got = np.empty(n, np.float32)
        assert rt.cudaMemcpy(got.ctypes.data, ptr, n * 4, 2) == 0
        o, omm = OracleTree(roots[version]).grid(OFFSET, COUNT, STEP, seed)
        assert np.array_equal(got.view(np.uint32), o.view(np.uint32)), (version, seed)
        assert (mn, mx) == (float(omm[0]), float(omm[1]))
        assert srv.release(ticket) == 0
    srv.close()
    live.close()
