"""The C++ node API on the GPU: trees built with New<T> and the setters, and the same trees
decoded with NewFromEncodedNodeTree, generate through Generator::GenUniformGrid2D/3D/4D,
GenTileable2D, GenPositionArray3D and GenSingle3D; each result and its OutputMinMax must equal
the C-ABI's and the oracle's bit for bit (reference Generator.h:210-429, Generator.inl).

Also the reference's threading contract (README.md:39-40: one tree used from many threads at
once): eight host threads generate on one shared tree while the library specialises it in the
background, and every result equals the single-thread result.
"""
import os
import subprocess

import numpy as np
import pytest

from oracle.oracle import OracleTree
from tests import trees
from tests.cpp import build_check
from tests.parity import assert_parity

pytestmark = pytest.mark.gpu

TREES = {"simplex_c0": trees.simplex_c0, "fbm_perlin_c1": trees.fbm_perlin_c1, "terrain_c2": trees.terrain_c2,
         "blend_tree": trees.blend_tree}


@pytest.fixture(scope="module")
def generated(gpu, tmp_path_factory):
    exe = build_check.build()
    out = tmp_path_factory.mktemp("cpp_gen")
    r = subprocess.run([exe, "gen", str(out)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    return out


def load(out, name):
    v = np.fromfile(os.path.join(out, name + ".f32"), np.float32)
    mm = np.fromfile(os.path.join(out, name + ".mm"), np.float32)
    return v, (float(mm[0]), float(mm[1]))


def positions():
    i = np.arange(5000, dtype=np.float32)
    return [i * np.float32(0.6), i * np.float32(-1.3), i * np.float32(0.25) + np.float32(7.0)]


CALLS = {
    "grid3d": lambda t: t.grid((-128.0, -128.0, -128.0), (64, 64, 64), (1.0, 1.0, 1.0), 1337),
    "tileable": lambda t: t.tileable(192, 160, 1.0, 1.0, 7),
    "grid2d": lambda t: t.grid((10.5, -3.25), (300, 200), (0.5, 2.0), -42),
    "grid4d": lambda t: t.grid((1.0, 2.0, 3.0, 4.0), (12, 10, 8, 6), (1.0, 1.0, 1.0, 1.0), 99),
    "pos3d": lambda t: t.positions(positions(), (0.5, 0.25, -1.0), 2024),
}


@pytest.mark.parametrize("version", ["setters", "decoded"])
@pytest.mark.parametrize("call", list(CALLS))
@pytest.mark.parametrize("name", list(TREES))
def test_cpp_api_matches_oracle_and_c_abi(generated, name, call, version):
    got, gmm = load(generated, f"{name}_{version}_{call}")
    root = TREES[name]()
    ref, rmm = CALLS[call](OracleTree(root))
    assert_parity(got, gmm, ref, rmm, label=f"C++ API {name} {version} {call}")
    # the C-ABI on the same tree (built with fnNewFromMetadata + fnSet*)
    prod = trees.to_product(root)
    if call == "tileable":
        c, cmm = prod.gen_tileable_2d((192, 160), (1.0, 1.0), 7)
    elif call == "pos3d":
        c, cmm = prod.gen_position_array(positions(), (0.5, 0.25, -1.0), 2024)
    else:
        args = {"grid3d": ((-128.0, -128.0, -128.0), (64, 64, 64), (1.0, 1.0, 1.0), 1337),
                "grid2d": ((10.5, -3.25), (300, 200), (0.5, 2.0), -42),
                "grid4d": ((1.0, 2.0, 3.0, 4.0), (12, 10, 8, 6), (1.0, 1.0, 1.0, 1.0), 99)}[call]
        c, cmm = prod.gen_uniform_grid(*args)
    assert np.array_equal(got.view(np.uint32), c.view(np.uint32)) and gmm == cmm


@pytest.mark.parametrize("name", list(TREES))
def test_cpp_gen_single(generated, name):
    got = np.fromfile(os.path.join(generated, f"{name}_setters_single3d.f32"), np.float32)
    dec = np.fromfile(os.path.join(generated, f"{name}_decoded_single3d.f32"), np.float32)
    ref = OracleTree(TREES[name]()).single((12.5, -7.25, 3.0), 5)
    assert got.view(np.uint32)[0] == np.float32(ref).view(np.uint32) == dec.view(np.uint32)[0]


def test_one_tree_many_threads(gpu):
    """8 host threads share one tree (host calls, per-thread staging, per-thread min/max
    workspaces) while automatic specialisation swaps the tree's kernels in; all results
    bit-identical to the single-thread interpreter result."""
    exe = build_check.build()
    r = subprocess.run([exe, "threads", "8"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "0 mismatches" in r.stdout


def test_drop_in_call_latency(gpu):
    """The C interface called from C++ (tests/cpp/latency_check.cpp): the config-0 grid into
    device, page-locked and std::vector outputs, all bit-identical; the per-call medians are
    printed (pytest -s) beside the round trip of an empty GPU operation."""
    exe = build_check.build("latency_check")
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "0 mismatches" in r.stdout
    print(r.stdout.strip().splitlines()[0])
