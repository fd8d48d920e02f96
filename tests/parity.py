"""Shared comparison helpers: run a tree through the GPU (product C-ABI) and the
CPU oracle on the same inputs and check the result.

Tolerance: max |gpu - oracle| <= 1e-5 (absolute, the path's stated bound), or
1e-6 relative for values whose magnitude exceeds 10.  Both sides implement the
same IEEE operation sequence, so in practice outputs are bit-identical; the
bit-exact fraction is reported with every comparison.
"""
from __future__ import annotations

import numpy as np

from oracle.oracle import OracleTree
from tests.trees import to_product

ABS_TOL = 1e-5
REL_TOL = 1e-6


def close(gpu: np.ndarray, ref: np.ndarray, nan_equal: bool = True):
    """(ok, max abs err, fraction bit-identical, points failing).  NaN on both sides counts as
    identical when `nan_equal` (the payload of an invalid operation's NaN is the processor's:
    0xFFC00000 on x86, 0x7FFFFFFF from the GPU); outputs that pack integers into float bits
    (ConvertRGBA8) pass nan_equal=False, where every bit pattern is data."""
    gpu = np.asarray(gpu, np.float32)
    ref = np.asarray(ref, np.float32)
    assert gpu.shape == ref.shape
    same_bits = gpu.view(np.uint32) == ref.view(np.uint32)
    if nan_equal:
        same_bits |= np.isnan(gpu) & np.isnan(ref)
    with np.errstate(invalid="ignore"):
        diff = np.abs(gpu.astype(np.float64) - ref.astype(np.float64))
        diff[same_bits] = 0.0
        tol = np.maximum(ABS_TOL, REL_TOL * np.abs(np.nan_to_num(ref.astype(np.float64))))
        bad = ~same_bits & ~(diff <= tol)
    exact = float(np.mean(same_bits)) if gpu.size else 1.0
    finite = diff[~np.isnan(diff)]
    maxerr = float(finite.max()) if finite.size else 0.0
    return (not bad.any()), maxerr, exact, int(bad.sum())


def minmax_equal(a, b):
    def eq(x, y):
        return (np.isnan(x) and np.isnan(y)) or x == y
    return eq(a[0], b[0]) and eq(a[1], b[1])


def run_grid(root, offset, count, step, seed):
    prod = to_product(root)
    g, gmm = prod.gen_uniform_grid(offset, count, step, seed)
    o, omm = OracleTree(root).grid(offset, count, step, seed)
    return g, gmm, o, omm


def run_positions(root, pos, offset, seed):
    prod = to_product(root)
    g, gmm = prod.gen_position_array(pos, offset, seed)
    o, omm = OracleTree(root).positions(pos, offset, seed)
    return g, gmm, o, omm


def run_tileable(root, size, step, seed):
    prod = to_product(root)
    g, gmm = prod.gen_tileable_2d(size, step, seed)
    o, omm = OracleTree(root).tileable(size[0], size[1], step[0], step[1], seed)
    return g, gmm, o, omm


def assert_parity(g, gmm, o, omm, label="", bit_exact=True, nan_equal=True):
    """Tolerance check, plus bit-exactness: the kernels and the oracle perform the
    same IEEE operation sequence (fmaf exactly where FS::FMulAdd is used, the
    same Sin/Cos/Pow polynomials), so any differing bit is a lattice, hash or
    cell-selection divergence and is reported as a failure."""
    ok, maxerr, exact, nbad = close(g, o, nan_equal)
    one_nan = int(np.sum(np.isnan(np.asarray(g, np.float32)) != np.isnan(np.asarray(o, np.float32))))
    assert ok, (f"{label}: {nbad} points beyond tolerance ({one_nan} NaN on one side only), "
                f"max abs err {maxerr:.3e}, bit-exact {exact:.4f}")
    assert minmax_equal(gmm, omm), f"{label}: minmax {gmm} != oracle {omm}"
    if bit_exact:
        assert exact == 1.0, f"{label}: only {exact:.6f} of points bit-identical (max abs err {maxerr:.3e})"
    return maxerr, exact
