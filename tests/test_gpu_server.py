"""Request server: continuous batching over a device pool.

Each result must be bit-identical whether the request is generated alone
(per-call fnGenUniformGrid*) or inside a mix that is admitted while other
batches are still on the GPU.  Failure paths are host-side: pool exhaustion
(admission waits), a request larger than the pool (rejected), cancellation
and bounded waits -- none of them faults or stalls the GPU.
"""
import time

import numpy as np
import pytest

from tests import chunkmix, trees

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    return torch


def device_array(torch, ptr, n):
    """Copy n floats from a raw device pointer into a numpy array."""
    import ctypes
    host = np.empty(n, np.float32)
    rt = ctypes.CDLL("libcudart.so")
    rt.cudaMemcpy.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
    assert rt.cudaMemcpy(host.ctypes.data, ptr, n * 4, 2) == 0   # cudaMemcpyDeviceToHost
    return host


def request(fn, node, c, out_ptr=0):
    kind = fn.KIND_GRID3D if len(c.count) == 3 else fn.KIND_GRID2D
    return fn.make_request(node, kind, out_ptr, c.seed, c.count, c.offset, (1, 1, 1, 1))


def test_results_same_alone_and_in_the_mix(gpu, torch_cuda):
    fn = gpu
    nodes = [trees.to_product(m()) for m in trees.MIX_TREES]
    chunks = chunkmix.make_mix(96, seed=21, sizes=[(16, 16, 16), (24, 20, 12), (32, 32), (128, 64)])
    srv = fn.Server(pool_bytes=64 << 20, streams=3, max_batch_requests=16)
    tickets = []
    for i, c in enumerate(chunks):                # arrive in waves while earlier batches run
        tickets.append(srv.submit(request(fn, nodes[c.tree], c)))
        if i % 24 == 23:
            time.sleep(0.002)
    for t, c in zip(tickets, chunks):
        mn, mx, ptr = srv.wait(t, timeout_ms=30000)
        got = device_array(torch_cuda, ptr, c.points)
        ref, rmm = nodes[c.tree].gen_uniform_grid(c.offset, c.count, (1,) * len(c.count), c.seed)
        assert np.array_equal(got.view(np.uint32), ref.view(np.uint32)), c
        assert (mn, mx) == rmm
        assert srv.release(t) == 0
    st = srv.stats()
    assert st["completed"] == len(chunks) and st["failed"] == 0
    assert st["batches"] >= 2 and st["p99Micros"] >= st["p50Micros"] > 0
    assert st["poolUsed"] == 0
    srv.close()


def test_submit_many_and_wait_many(gpu, torch_cuda):
    fn = gpu
    nodes = [trees.to_product(m()) for m in trees.MIX_TREES]
    chunks = chunkmix.make_mix(64, seed=33, sizes=[(16, 16, 16), (9, 7, 5), (32, 32), (50, 3)])
    srv = fn.Server(pool_bytes=64 << 20, streams=2, max_batch_requests=24)
    tickets = srv.submit_many([request(fn, nodes[c.tree], c) for c in chunks])
    assert len(set(tickets)) == len(chunks)
    srv.wait_many(tickets, timeout_ms=30000)
    for t, c in zip(tickets, chunks):
        assert srv.poll(t) == 1
        mn, mx, ptr = srv.wait(t, timeout_ms=0)
        got = device_array(torch_cuda, ptr, c.points)
        ref, rmm = nodes[c.tree].gen_uniform_grid(c.offset, c.count, (1,) * len(c.count), c.seed)
        assert np.array_equal(got.view(np.uint32), ref.view(np.uint32)), c
        assert (mn, mx) == rmm
        assert srv.release(t) == 0
    # a prebuilt request array and the tickets as a ctypes array (no per-call list conversion)
    arr = fn.request_array([request(fn, nodes[c.tree], c) for c in chunks])
    tarr = srv.submit_many(arr, as_array=True)
    srv.wait_many(tarr, timeout_ms=30000)
    for t, c in zip(tarr, chunks):
        mn, mx, ptr = srv.wait(t, timeout_ms=0)
        got = device_array(torch_cuda, ptr, c.points)
        ref, rmm = nodes[c.tree].gen_uniform_grid(c.offset, c.count, (1,) * len(c.count), c.seed)
        assert np.array_equal(got.view(np.uint32), ref.view(np.uint32)), c
        assert srv.release(t) == 0
    # all or nothing: one bad request rejects the whole list
    unsupported = trees.to_product(trees.unsupported_tree())      # keep the node alive while requests point to it
    bad = [request(fn, nodes[0], chunks[0]), request(fn, unsupported, chunks[1])]
    before = srv.stats()["submitted"]
    with pytest.raises(fn.FastNoiseError) as e:
        srv.submit_many(bad)
    assert e.value.code == -2 and srv.stats()["submitted"] == before
    srv.close()


def test_user_owned_outputs(gpu, torch_cuda):
    fn, torch = gpu, torch_cuda
    node = trees.to_product(trees.fbm_perlin_c1())
    srv = fn.Server(pool_bytes=1 << 20)
    out = torch.empty(32 * 32 * 32, device="cuda")
    c = chunkmix.Chunk(0, (32, 32, 32), (64.0, -32.0, 0.0), 9)
    t = srv.submit(request(fn, node, c, out.data_ptr()))
    mn, mx, ptr = srv.wait(t, 30000)
    assert ptr == out.data_ptr()
    ref, rmm = node.gen_uniform_grid(c.offset, c.count, (1, 1, 1), c.seed)
    assert np.array_equal(out.cpu().numpy().view(np.uint32), ref.view(np.uint32)) and (mn, mx) == rmm
    srv.close()


def test_pool_pressure_defers_admission(gpu, torch_cuda):
    fn = gpu
    node = trees.to_product(trees.simplex_c0())
    srv = fn.Server(pool_bytes=3 * 64 * 64 * 64 * 4, streams=2, max_batch_requests=4)   # room for 3 outputs
    c = chunkmix.Chunk(0, (64, 64, 64), (0.0, 0.0, 0.0), 1337)
    tickets = [srv.submit(request(fn, node, c)) for _ in range(8)]
    done = 0
    for t in tickets:                            # releasing results lets the rest be admitted
        srv.wait(t, 60000)
        assert srv.release(t) == 0
        done += 1
    assert done == 8 and srv.stats()["poolUsed"] == 0
    srv.close()


def test_request_larger_than_pool_is_rejected(gpu):
    fn = gpu
    node = trees.to_product(trees.simplex_c0())
    srv = fn.Server(pool_bytes=1 << 20)
    c = chunkmix.Chunk(0, (128, 128, 128), (0.0, 0.0, 0.0), 1)
    with pytest.raises(fn.FastNoiseError) as e:
        srv.submit(request(fn, node, c))
    assert e.value.code == -4
    srv.close()


def test_compile_errors_surface_at_submit(gpu):
    fn = gpu
    srv = fn.Server(pool_bytes=1 << 20)
    node = trees.to_product(trees.unsupported_tree())
    with pytest.raises(fn.FastNoiseError) as e:
        srv.submit(fn.make_request(node, fn.KIND_GRID2D, 0, 1, (8, 8)))
    assert e.value.code == -2
    srv.close()


def test_cancel_timeout_and_unknown_ticket(gpu):
    fn = gpu
    node = trees.to_product(trees.terrain_c2())
    srv = fn.Server(pool_bytes=256 << 20, streams=1, max_batch_requests=1)
    c = chunkmix.Chunk(2, (128, 128, 64), (0.0, 0.0, 0.0), 7)
    tickets = [srv.submit(request(fn, node, c)) for _ in range(6)]
    last = tickets[-1]
    rc = srv.cancel(last)
    assert rc in (0, -6)
    if rc == 0:
        with pytest.raises(fn.FastNoiseError) as e:
            srv.wait(last, 1000)
        assert e.value.code == -6
    with pytest.raises(fn.FastNoiseError) as e:
        srv.wait(tickets[-2], 0)                 # still queued behind a single stream
    assert e.value.code in (-5,)
    for t in tickets[:-1]:
        srv.wait(t, 60000)
        srv.release(t)
    assert srv.poll(123456789) < 0
    srv.close()


def test_batches_overlap_on_the_gpu(gpu, torch_cuda):
    """Continuous batching: requests submitted in waves are admitted while earlier batches run,
    and batches execute on the GPU at the same time.  The kernels stamp each request's
    completion with the device clock; two batches whose spans of completions intersect were
    both executing then (server statistic overlappedBatches).  Every result is the same as the
    request generated alone."""
    fn = gpu
    nodes = [trees.to_product(m()) for m in trees.MIX_TREES]
    chunks = chunkmix.make_mix(240, seed=5, sizes=[(32, 32, 32), (64, 64, 64), (128, 128), (512, 512)])
    srv = fn.Server(pool_bytes=2 << 30, streams=3, max_batch_requests=8)
    tickets = []
    for i in range(0, len(chunks), 40):                 # waves of 40 while earlier waves run
        tickets += srv.submit_many([request(fn, nodes[c.tree], c) for c in chunks[i:i + 40]])
        time.sleep(0.0005)
    srv.wait_many(tickets, timeout_ms=60000)
    st = srv.stats()
    assert st["completed"] == len(chunks) and st["failed"] == 0
    assert st["maxInflightBatches"] >= 2, st
    assert st["overlappedBatches"] >= 2 and st["maxConcurrentBatches"] >= 2, st
    for t, c in zip(tickets, chunks):
        mn, mx, ptr = srv.wait(t, timeout_ms=0)
        got = device_array(torch_cuda, ptr, c.points)
        ref, rmm = nodes[c.tree].gen_uniform_grid(c.offset, c.count, (1,) * len(c.count), c.seed)
        assert np.array_equal(got.view(np.uint32), ref.view(np.uint32)), c
        assert (mn, mx) == rmm
        assert srv.release(t) == 0
    srv.close()


def test_paced_submission_and_per_call_paced(gpu, torch_cuda):
    """fnServerSubmitPaced queues requests on an arrival schedule and counts latency from the
    arrival; fnGenEachPaced drives the per-call path with the same schedule.  Both return every
    request's result equal to the request generated alone."""
    fn = gpu
    torch = torch_cuda
    nodes = [trees.to_product(m()) for m in trees.MIX_TREES]
    chunks = chunkmix.make_mix(120, seed=9, sizes=[(16, 16, 16), (32, 32, 32), (64, 64), (128, 128)])
    arrivals = np.cumsum(np.random.default_rng(3).exponential(1.0 / 20000.0, len(chunks))) * 1e6
    srv = fn.Server(pool_bytes=256 << 20, streams=3, max_batch_requests=32)
    tickets = srv.submit_paced([request(fn, nodes[c.tree], c) for c in chunks], arrivals)
    srv.wait_many(tickets, timeout_ms=60000)
    st = srv.stats()
    assert st["completed"] == len(chunks) and st["p99Micros"] >= st["p50Micros"] > 0
    refs = []
    for t, c in zip(tickets, chunks):
        mn, mx, ptr = srv.wait(t, timeout_ms=0)
        ref, rmm = nodes[c.tree].gen_uniform_grid(c.offset, c.count, (1,) * len(c.count), c.seed)
        assert np.array_equal(device_array(torch, ptr, c.points).view(np.uint32), ref.view(np.uint32)), c
        assert (mn, mx) == rmm
        refs.append((ref, rmm))
        srv.release(t)
    srv.close()
    outs = [torch.full((c.points,), float("nan"), device="cuda") for c in chunks]
    mms = [np.zeros(2, np.float32) for _ in chunks]
    reqs = [fn.make_request(nodes[c.tree], fn.KIND_GRID3D if len(c.count) == 3 else fn.KIND_GRID2D, o.data_ptr(), c.seed,
                            c.count, c.offset, (1, 1, 1, 1), minmax=m) for c, o, m in zip(chunks, outs, mms)]
    lat = fn.gen_each_paced(reqs, arrivals)
    assert lat.shape == (len(chunks),) and (lat > 0).all()
    for (ref, rmm), o, m in zip(refs, outs, mms):
        assert np.array_equal(o.cpu().numpy().view(np.uint32), ref.view(np.uint32))
        assert (float(m[0]), float(m[1])) == rmm
