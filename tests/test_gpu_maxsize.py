"""Requests past the 32-bit index range: more than 2^31 points in one call and more than 2^32
points in one batch request.

The reference's C interface takes int counts per axis, so such grids are expressible through
it (Generator.inl:129-186 computes the position of point i from its per-axis indices).  Those
paths run on 64-bit point indices: the per-call kernels take them above 2^31 points, the batch
kernels above 2^32.  A full oracle pass over billions of points is out of reach, so the checks
are size-independent: z-slabs of the large grid equal the same slab generated as a small grid
of its own (positions fma(float(i), step, offset) are exact for these integer offsets), one
slab equals the oracle, and OutputMinMax equals the minimum and maximum of the output.
"""
import numpy as np
import pytest

from oracle.oracle import OracleTree
from oracle.tree import N
from tests import trees
from tests.parity import assert_parity

pytestmark = pytest.mark.gpu

NX, NY = 2048, 1024
TREE = lambda: N("Value", Feature_Scale=37.0)          # cheap, so billions of points take a fraction of a second
SLABS = (0, 700, 1024)


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    return torch


@pytest.fixture
def node(gpu):
    fn = gpu
    old = fn.set_auto_specialise(0)
    yield trees.to_product(TREE())
    fn.set_auto_specialise(old)


def slab(torch, node, z, seed):
    out = torch.empty(NX * NY, dtype=torch.float32, device="cuda")
    mm = torch.empty(2, dtype=torch.float32, device="cuda")
    node.gen_uniform_grid_device(out.data_ptr(), (0.0, 0.0, float(z)), (NX, NY, 1), (1.0, 1.0, 1.0), seed, mm.data_ptr())
    torch.cuda.synchronize()
    return out


def check_big(torch, node, big, nz, seed, mm):
    plane = NX * NY
    for z in SLABS:
        if z < nz:
            ref = slab(torch, node, z, seed)
            assert torch.equal(big[z * plane:(z + 1) * plane].view(torch.int32), ref.view(torch.int32)), z
    lo, hi = torch.aminmax(big)
    assert (float(lo), float(hi)) == mm
    o, omm = OracleTree(TREE()).grid((0.0, 0.0, float(SLABS[-1])), (NX, NY, 1), (1.0, 1.0, 1.0), seed)
    last = big[SLABS[-1] * plane:(SLABS[-1] + 1) * plane].cpu().numpy()
    assert_parity(last, (float(last.min()), float(last.max())), o, omm, label="slab vs oracle")


def test_device_grid_beyond_2_31_points(node, torch_cuda):
    torch = torch_cuda
    nz = 1025
    total = NX * NY * nz
    assert total > 2 ** 31
    big = torch.empty(total, dtype=torch.float32, device="cuda")
    mm = torch.empty(2, dtype=torch.float32, device="cuda")
    node.gen_uniform_grid_device(big.data_ptr(), (0.0, 0.0, 0.0), (NX, NY, nz), (1.0, 1.0, 1.0), 91, mm.data_ptr())
    torch.cuda.synchronize()
    m = mm.cpu().numpy()
    check_big(torch, node, big, nz, 91, (float(m[0]), float(m[1])))
    del big
    torch.cuda.empty_cache()


def test_host_grid_beyond_2_31_points(node, torch_cuda):
    """The drop-in host call (fnGenUniformGrid3D) on the same grid."""
    torch = torch_cuda
    nz = 1025
    out, mm = node.gen_uniform_grid((0.0, 0.0, 0.0), (NX, NY, nz), (1.0, 1.0, 1.0), 92)
    assert out.size == NX * NY * nz
    big = torch.from_numpy(out).cuda()
    del out
    check_big(torch, node, big, nz, 92, mm)
    del big
    torch.cuda.empty_cache()


def test_batch_request_beyond_2_32_points(gpu, node, torch_cuda):
    """One batch with a 4.3 G-point request beside a small one (fnGenBatchDevice)."""
    fn, torch = gpu, torch_cuda
    nz = 2049
    total = NX * NY * nz
    assert total > 2 ** 32
    big = torch.empty(total, dtype=torch.float32, device="cuda")
    small = torch.empty(4096, dtype=torch.float32, device="cuda")
    mm_big, mm_small = np.zeros(2, np.float32), np.zeros(2, np.float32)
    reqs = [fn.make_request(node, fn.KIND_GRID3D, big.data_ptr(), 93, (NX, NY, nz), (0.0, 0.0, 0.0), (1, 1, 1), minmax=mm_big),
            fn.make_request(node, fn.KIND_GRID3D, small.data_ptr(), 94, (16, 16, 16), (5.0, 6.0, 7.0), (1, 1, 1),
                            minmax=mm_small)]
    fn.gen_batch(reqs, sync=True)
    check_big(torch, node, big, nz, 93, (float(mm_big[0]), float(mm_big[1])))
    ref, rmm = node.gen_uniform_grid((5.0, 6.0, 7.0), (16, 16, 16), (1.0, 1.0, 1.0), 94)
    assert np.array_equal(small.cpu().numpy().view(np.uint32), ref.view(np.uint32))
    assert (float(mm_small[0]), float(mm_small[1])) == rmm
    del big
    torch.cuda.empty_cache()
