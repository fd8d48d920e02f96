"""The CPU oracle itself (CPU only): regression fixtures, reference invariants,
and the accuracy of the project-written Sin/Cos/Pow kernels.

Parity with the reference is unpinned (no reference golden values exist); these
tests pin the oracle to its committed fixtures and to properties the reference
code guarantees by construction (Generator.inl / Generator.h).
"""
import hashlib
import json
import os

import numpy as np
import pytest

from oracle import oracle as O
from oracle.tree import N, decode
from tests import trees

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "oracle_golden.json")


def load_cases():
    with open(GOLDEN) as f:
        return json.load(f)["cases"]


@pytest.mark.parametrize("case", load_cases(), ids=lambda c: c["name"])
def test_oracle_matches_golden_fixture(case):
    root = decode(case["tree"])
    assert root is not None
    t = O.OracleTree(root)
    if case["kind"] == "grid":
        v, mm = t.grid(*case["args"], case["seed"])
    else:
        v, mm = t.tileable(*case["args"], case["seed"])
    assert hashlib.sha256(np.ascontiguousarray(v, np.float32).tobytes()).hexdigest() == case["sha256"]
    assert mm[0] == case["min"] and mm[1] == case["max"]


def test_sin_cos_accuracy():
    x = np.concatenate([np.linspace(-50, 50, 40001), np.linspace(0, 2 * np.pi, 4096)]).astype(np.float32)
    s = np.array([O.sinf(v) for v in x], np.float32)
    c = np.array([O.cosf(v) for v in x], np.float32)
    ts, tc = np.sin(x.astype(np.float64)), np.cos(x.astype(np.float64))
    assert np.max(np.abs(s - ts)) < 1.5e-7
    assert np.max(np.abs(c - tc)) < 1.5e-7


def test_pow_accuracy():
    rng = np.random.default_rng(3)
    a = rng.uniform(1e-3, 8, 4000).astype(np.float32)
    b = rng.uniform(0.2, 4, 4000).astype(np.float32)
    p = np.array([O.powf(x, y) for x, y in zip(a, b)], np.float64)
    ref = a.astype(np.float64) ** b.astype(np.float64)
    assert np.max(np.abs(p - ref) / ref) < 4e-6
    assert O.powf(0.0, 2.0) == 0.0 and O.powf(5.0, 0.0) == 1.0


def test_output_minmax_is_min_and_max():
    v, mm = O.OracleTree(trees.fbm_perlin_c1()).grid((0, 0, 0), (16, 16, 16), (1, 1, 1), 42)
    assert mm == (float(v.min()), float(v.max()))


def test_single_equals_grid_element():
    t = O.OracleTree(trees.terrain_c2())
    v, _ = t.grid((3, 4, 5), (4, 3, 2), (1, 1, 1), 7)
    assert t.single((6.0, 6.0, 6.0), 7) == v[23]


def test_thread_count_does_not_change_results():
    t = O.OracleTree(trees.fbm_perlin_c1())
    a, ma = t.grid((0, 0, 0), (32, 32, 32), (1, 1, 1), 42, threads=1)
    b, mb = t.grid((0, 0, 0), (32, 32, 32), (1, 1, 1), 42, threads=7)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32)) and ma == mb


def test_request_batch_and_paced_serving_match_single_grids():
    """gen_requests (whole-request batch) and serve_paced (open-loop FIFO) write the same bits
    and min/max as one grid call per request."""
    ts = [O.OracleTree(m()) for m in trees.MIX_TREES[:3]]
    shapes = [(9, 7, 5), (16, 16), (4, 3, 2, 2)]
    kinds = [O.KIND_GRID3D, O.KIND_GRID2D, O.KIND_GRID4D]
    rng = np.random.default_rng(3)
    cases = [(k % 3, k % 3, tuple(rng.uniform(-50, 50, len(shapes[k % 3]))), 11 + k) for k in range(12)]
    for serve in (False, True):
        outs, mms, reqs = [], [], []
        for tree, shape_k, off, seed in cases:
            outs.append(np.empty(int(np.prod(shapes[shape_k])), np.float32))
            mms.append(np.zeros(2, np.float32))
            reqs.append(O.request(ts[tree], kinds[shape_k], outs[-1], mms[-1], seed, shapes[shape_k], off))
        if serve:
            lat = O.serve_paced(reqs, np.arange(len(reqs)) * 50.0, threads=3)
            assert lat.shape == (len(reqs),) and np.all(lat >= 0)
        else:
            O.gen_requests(reqs, threads=3)
        for (tree, shape_k, off, seed), o, mm in zip(cases, outs, mms):
            ref, rmm = ts[tree].grid(off, shapes[shape_k], (1,) * len(shapes[shape_k]), seed)
            assert np.array_equal(ref.view(np.uint32), o.view(np.uint32)) and (float(mm[0]), float(mm[1])) == rmm


def test_noise_outputs_are_normalised():
    """Each coherent noise's bounding constant maps its output into [-1, 1]."""
    for name in ("Simplex", "SuperSimplex", "Perlin", "Value"):
        for cnt in ((200, 200), (48, 48, 48), (14, 14, 14, 14)):
            v, mm = O.OracleTree(N(name, Feature_Scale=3.0)).grid([0.0] * len(cnt), cnt, [1.0] * len(cnt), 1337)
            assert -1.0 <= mm[0] and mm[1] <= 1.0, (name, len(cnt), mm)
            assert mm[1] - mm[0] > 1.0, (name, len(cnt), mm)
