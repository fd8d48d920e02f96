"""The C++ node API (include/FastNoise/FastNoise.h, header-only over the C-ABI), CPU checks.

Reference API: FastNoise::New<T> and NewFromEncodedNodeTree (include/FastNoise/FastNoise.h:36-65),
SmartNode with DynamicCast (Utility/SmartNode.h:71-320), the node classes' setters
(Generators/*.h), Metadata and NodeData (Metadata.h).  Generation calls need the GPU and are
checked in test_gpu_cpp_api.py.
"""
import os
import subprocess

import pytest

from oracle import tree as T
from tests import trees
from tests.cpp import build_check

REFERENCE_CPP11_TEST = "/root/reference/tests/FastNoiseCpp11Include.cpp"


@pytest.fixture(scope="module")
def checker(native):
    return build_check.build()


def test_metadata_classes_casts_and_node_data(checker):
    """New<T> for all 47 node classes, DynamicCast, Metadata tables and setters, NodeData
    encode/decode round trips, loop handling with and without fixUp (cpp_api_check meta)."""
    r = subprocess.run([checker, "meta"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr


def test_setters_build_the_same_trees_as_the_metadata_model(checker):
    """Trees built with the typed setters (SetScale, SetOctaveCount, SetReturnType, ...) encode
    to the same strings as the same trees built member by member in the oracle's model of the
    reference's metadata: every setter reaches the member the reference's setter does."""
    r = subprocess.run([checker, "encode"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    got = r.stdout.split()
    want = [T.encode(m()) for m in (trees.simplex_c0, trees.fbm_perlin_c1, trees.terrain_c2, trees.blend_tree)]
    assert got == want


@pytest.mark.skipif(not os.path.exists(REFERENCE_CPP11_TEST), reason="reference sources not present")
@pytest.mark.parametrize("std", ["c++11", "c++17"])
def test_reference_cpp_example_compiles_unchanged(native, tmp_path, std):
    """The reference's own C++ example (tests/FastNoiseCpp11Include.cpp) compiles and links
    against these headers and this library without changes."""
    from fastnoise2_gb300 import build as product
    lib_dir = os.path.dirname(product.build())
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    cmd = ["g++", f"-std={std}", f"-I{root}/include", REFERENCE_CPP11_TEST, "-o", str(tmp_path / "example"),
           f"-L{lib_dir}", "-lfastnoise_gb300", f"-Wl,-rpath,{lib_dir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
