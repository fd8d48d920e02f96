"""Chunk meshing on the GPU (fnBuildChunkMeshBloxel / Dmc / Heightmap) against the CPU
restatement of the Node Editor's meshers (oracle/mesh.py): the same vertices, indices, heights
and OutputMinMax, bit for bit.  Each 3D case runs on both kernel tiers: the interpreter, which
writes the chunk's density array, and the tree's specialised kernels, with which the meshers
work from the sparse form (the densities' classification bitmasks, and values evaluated again
only at the voxels the light and vertex passes read)."""
import numpy as np
import pytest

from oracle import mesh as omesh
from oracle.tree import N
from tests import trees

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    return torch


def surface_tree():
    """Densities that cross 0: a vertical gradient plus fractal noise (a terrain surface)."""
    g = N("Gradient")
    g.set("Multiplier", 0.08, 1)
    return N("Add", LHS=N("FractalFBm", Source=N("Simplex", Feature_Scale=18.0), Octaves=3), RHS=g)


def caves_tree():
    return N("CellularDistance", Feature_Scale=9.0, Return_Type="Index0Sub1")


# interpreter: the density array; specialised: the density array from the tree's specialised
# kernel; sparse: the sparse density form (fnSetMeshDensityForm)
TIERS = ["interpreter", "specialised", "sparse"]


@pytest.fixture(autouse=True)
def density_form(request, gpu):
    tier = request.node.callspec.params.get("tier") if hasattr(request.node, "callspec") else None
    prev = gpu.set_mesh_density_form(gpu.MESH_DENSITY_SPARSE if tier == "sparse" else gpu.MESH_DENSITY_ARRAY)
    yield
    gpu.set_mesh_density_form(prev)


def product_node(fn, root, tier):
    node = trees.to_product(root)
    if tier in ("specialised", "sparse"):
        fn.jit_compile([(node, 3)])
    return node


def run_bloxel(fn, torch, root, size, pos, seed, iso, up_z, vcap=None, icap=None, tier="interpreter"):
    node = product_node(fn, root, tier)
    vcap = vcap if vcap is not None else size ** 3 * 24
    icap = icap if icap is not None else size ** 3 * 36
    v = torch.zeros(max(vcap, 1) * 4, dtype=torch.float32, device="cuda")
    i = torch.zeros(max(icap, 1), dtype=torch.int32, device="cuda")
    res = fn.build_chunk_mesh_bloxel(node, size, pos, seed, iso, up_z, v.data_ptr(), vcap, i.data_ptr(), icap)
    return res, v.cpu().numpy().reshape(-1, 4), i.cpu().numpy().view(np.uint32)


def oracle_bloxel(root, size, pos, seed, iso, up_z):
    d, mm = omesh.bloxel_densities(root, size, pos, seed, up_z)
    return (*omesh.bloxel_mesh(d, mm, size, pos, iso), mm)


@pytest.mark.parametrize("case", [
    (surface_tree, 16, (32, -8, 16), 1337, 0.0, False),
    (surface_tree, 20, (-48, 4, -20), 7, 0.1, False),
    (surface_tree, 16, (16, -16, 0), 42, 0.0, True),
    (caves_tree, 12, (-12, 24, 36), -5, -0.8, False),
])
@pytest.mark.parametrize("tier", TIERS)
def test_bloxel_matches_oracle(gpu, torch_cuda, case, tier):
    make, size, pos, seed, iso, up_z = case
    res, gv, gi = run_bloxel(gpu, torch_cuda, make(), size, pos, seed, iso, up_z, tier=tier)
    ov, oi, oair, osolid, omm = oracle_bloxel(make(), size, pos, seed, iso, up_z)
    assert res["fits"] and res["vertexCount"] == len(ov) and res["indexCount"] == len(oi) > 0
    assert np.array_equal(gv[:len(ov)].view(np.uint32), ov.view(np.uint32))
    assert np.array_equal(gi[:len(oi)], oi)
    assert (res["minAirY"], res["maxSolidY"]) == (float(oair), float(osolid))
    assert res["minMax"] == (float(omm[0]), float(omm[1]))


@pytest.mark.parametrize("tier", TIERS)
@pytest.mark.parametrize("value, expect", [(1.0, "air"), (-1.0, "solid")])
def test_bloxel_early_out(gpu, torch_cuda, value, expect, tier):
    """OutputMinMax entirely above / below the iso level: no faces, only the height."""
    res, _, _ = run_bloxel(gpu, torch_cuda, N("Constant", Value=value), 16, (0, 32, 0), 1, 0.0, False, tier=tier)
    assert res["vertexCount"] == 0 and res["indexCount"] == 0
    if expect == "air":
        assert res["minAirY"] == 32.0 and res["maxSolidY"] == float("-inf")
    else:
        assert res["maxSolidY"] == 32.0 - 1.0 + 16 and res["minAirY"] == float("inf")


@pytest.mark.parametrize("tier", TIERS)
def test_bloxel_reports_capacity(gpu, torch_cuda, tier):
    res, _, _ = run_bloxel(gpu, torch_cuda, surface_tree(), 16, (32, -8, 16), 1337, 0.0, False, vcap=8, icap=12, tier=tier)
    ov, oi, _, _, _ = oracle_bloxel(surface_tree(), 16, (32, -8, 16), 1337, 0.0, False)
    assert not res["fits"] and res["vertexCount"] == len(ov) and res["indexCount"] == len(oi)


@pytest.mark.parametrize("size, pos, mul", [(16, (32, 16), 100.0), (24, (-40, 8), 37.5)])
def test_heightmap_matches_oracle(gpu, torch_cuda, size, pos, mul):
    fn, torch = gpu, torch_cuda
    root = N("FractalFBm", Source=N("Perlin", Feature_Scale=30.0), Octaves=4)
    node = trees.to_product(root)
    v = torch.zeros(size * size * 16, dtype=torch.float32, device="cuda")
    i = torch.zeros(size * size * 6, dtype=torch.int32, device="cuda")
    res = fn.build_chunk_mesh_heightmap(node, size, pos, 11, mul, v.data_ptr(), size * size * 4, i.data_ptr(), size * size * 6)
    d, mm = omesh.heightmap_densities(root, size, (pos[0], 0, pos[1]), 11)
    ov, oi = omesh.heightmap_mesh(d, size, (pos[0], 0, pos[1]), mul)
    assert res["fits"] and res["vertexCount"] == len(ov) and res["indexCount"] == len(oi)
    assert np.array_equal(v.cpu().numpy().reshape(-1, 4).view(np.uint32), ov.view(np.uint32))
    assert np.array_equal(i.cpu().numpy().view(np.uint32), oi)
    assert res["minMax"] == (float(mm[0]), float(mm[1]))


def white_tree():
    """Independent random densities per voxel: every marching-cubes case, ambiguous faces included."""
    return N("White", Seed_Offset=5)


def run_dmc(fn, torch, root, size, pos, seed, iso, up_z, vcap=None, icap=None, tier="interpreter"):
    node = product_node(fn, root, tier)
    vcap = vcap if vcap is not None else (size + 1) ** 3 * 4
    icap = icap if icap is not None else size ** 3 * 18
    v = torch.zeros(max(vcap, 1) * 4, dtype=torch.float32, device="cuda")
    i = torch.zeros(max(icap, 1), dtype=torch.int32, device="cuda")
    res = fn.build_chunk_mesh_dmc(node, size, pos, seed, iso, up_z, v.data_ptr(), vcap, i.data_ptr(), icap)
    return res, v.cpu().numpy().reshape(-1, 4), i.cpu().numpy().view(np.uint32)


def oracle_dmc(root, size, pos, seed, iso, up_z):
    d, mm = omesh.dmc_densities(root, size, pos, seed, up_z)
    return (*omesh.dmc_mesh(d, mm, size, pos, iso), mm)


@pytest.mark.parametrize("case", [
    (surface_tree, 16, (32, -8, 16), 1337, 0.0, False),
    (surface_tree, 20, (-48, 4, -20), 7, 0.1, False),
    (surface_tree, 16, (16, -16, 0), 42, 0.0, True),
    (caves_tree, 12, (-12, 24, 36), -5, -0.8, False),
    (white_tree, 10, (100, -3, 7), 99, 0.0, False),
    (white_tree, 9, (0, 0, 0), -1234, 0.3, True),
])
@pytest.mark.parametrize("tier", TIERS)
def test_dmc_matches_oracle(gpu, torch_cuda, case, tier):
    make, size, pos, seed, iso, up_z = case
    res, gv, gi = run_dmc(gpu, torch_cuda, make(), size, pos, seed, iso, up_z, tier=tier)
    ov, oi, oair, osolid, omm = oracle_dmc(make(), size, pos, seed, iso, up_z)
    assert res["fits"] and res["vertexCount"] == len(ov) and res["indexCount"] == len(oi) > 0
    assert np.array_equal(gv[:len(ov)].view(np.uint32), ov.view(np.uint32))
    assert np.array_equal(gi[:len(oi)], oi)
    assert (res["minAirY"], res["maxSolidY"]) == (float(oair), float(osolid))
    assert res["minMax"] == (float(omm[0]), float(omm[1]))


@pytest.mark.parametrize("tier", TIERS)
@pytest.mark.parametrize("value, expect", [(1.0, "air"), (-1.0, "solid")])
def test_dmc_early_out(gpu, torch_cuda, value, expect, tier):
    res, _, _ = run_dmc(gpu, torch_cuda, N("Constant", Value=value), 16, (0, 32, 0), 1, 0.0, False, tier=tier)
    assert res["vertexCount"] == 0 and res["indexCount"] == 0
    if expect == "air":
        assert res["minAirY"] == 32.0 and res["maxSolidY"] == float("-inf")
    else:
        assert res["maxSolidY"] == 32.0 - 1.0 + 16 and res["minAirY"] == float("inf")


@pytest.mark.parametrize("tier", TIERS)
def test_dmc_reports_capacity(gpu, torch_cuda, tier):
    res, _, _ = run_dmc(gpu, torch_cuda, surface_tree(), 16, (32, -8, 16), 1337, 0.0, False, vcap=8, icap=12, tier=tier)
    ov, oi, oair, osolid, _ = oracle_dmc(surface_tree(), 16, (32, -8, 16), 1337, 0.0, False)
    assert not res["fits"] and res["vertexCount"] == len(ov) and res["indexCount"] == len(oi)
    assert (res["minAirY"], res["maxSolidY"]) == (float(oair), float(osolid))


@pytest.mark.parametrize("tier", TIERS)
@pytest.mark.parametrize("kind", ["dmc", "bloxel"])
def test_many_chunks_match_single_calls(gpu, torch_cuda, kind, tier):
    """fnBuildChunkMeshes*: chunks spread over internal streams give each chunk exactly the
    single-call mesh; a chunk with too small buffers reports its counts, the others complete."""
    fn, torch = gpu, torch_cuda
    size = 16
    positions = [(16 * k - 40, -8 + 4 * (k % 3), 16 * (k % 2)) for k in range(7)]
    node = product_node(fn, surface_tree(), tier)
    vcap, icap = (size + 1) ** 3 * 4, size ** 3 * 18
    single = {"dmc": fn.build_chunk_mesh_dmc, "bloxel": fn.build_chunk_mesh_bloxel}[kind]
    bufs, tensors = [], []
    for k in range(len(positions)):
        v = torch.zeros(vcap * 4, dtype=torch.float32, device="cuda")
        i = torch.zeros(icap, dtype=torch.int32, device="cuda")
        small = k == 3
        bufs.append((v.data_ptr(), 8 if small else vcap, i.data_ptr(), 12 if small else icap))
        tensors.append((v, i))
    res = fn.build_chunk_meshes(kind, node, size, positions, 1337, 0.0, False, bufs)
    for k, p in enumerate(positions):
        v1 = torch.zeros(vcap * 4, dtype=torch.float32, device="cuda")
        i1 = torch.zeros(icap, dtype=torch.int32, device="cuda")
        ref = single(node, size, p, 1337, 0.0, False, v1.data_ptr(), vcap, i1.data_ptr(), icap)
        r = res[k]
        assert (r["vertexCount"], r["indexCount"], r["minAirY"], r["maxSolidY"], r["minMax"]) == \
               (ref["vertexCount"], ref["indexCount"], ref["minAirY"], ref["maxSolidY"], ref["minMax"]), k
        if k == 3:
            assert not r["fits"]
            continue
        nv, ni = ref["vertexCount"], ref["indexCount"]
        v, i = tensors[k]
        assert torch.equal(v[:nv * 4].view(torch.int32), v1[:nv * 4].view(torch.int32)), k
        assert torch.equal(i[:ni], i1[:ni]), k


@pytest.mark.parametrize("kind", ["dmc", "bloxel"])
def test_sparse_form_equals_density_array_on_editor_chunks(gpu, torch_cuda, kind):
    """The Node Editor's chunk size (128^3) on a terrain surface: the mesh from the sparse form
    (specialised kernels) equals the mesh from the density array (interpreter) bit for bit."""
    fn, torch = gpu, torch_cuda
    root = N("Add", LHS=N("FractalFBm", Source=N("Simplex", Feature_Scale=60.0), Octaves=4),
             RHS=N("Gradient").set("Multiplier", 0.02, 1))
    run = run_dmc if kind == "dmc" else run_bloxel
    size, vcap, icap = 128, 1 << 20, 3 << 20
    prev = fn.set_mesh_density_form(fn.MESH_DENSITY_SPARSE)
    try:
        got = run(fn, torch, root, size, (-64, -64, 128), 1337, 0.0, False, vcap=vcap, icap=icap, tier="specialised")
    finally:
        fn.set_mesh_density_form(prev)
    fn.set_jit_enabled(False)
    try:
        ref = run(fn, torch, root, size, (-64, -64, 128), 1337, 0.0, False, vcap=vcap, icap=icap, tier="interpreter")
    finally:
        fn.set_jit_enabled(True)
    (r1, v1, i1), (r2, v2, i2) = got, ref
    assert r1 == r2 and r1["fits"] and r1["indexCount"] > 10000
    nv, ni = r1["vertexCount"], r1["indexCount"]
    assert np.array_equal(v1[:nv].view(np.uint32), v2[:nv].view(np.uint32))
    assert np.array_equal(i1[:ni], i2[:ni])
