"""CPU checks of the mesher restatement (oracle/mesh.py): the dual marching cubes table is
pinned to the reference's kDualPointsList by digest (tests/golden/dmc_table.json, made by
tests/golden/make_dmc_digest.py), and the DMC mesher produces a closed, consistently
oriented surface around an analytic sphere."""
import json
import os
from collections import Counter

import numpy as np

from oracle import mesh as omesh

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "dmc_table.json")


def test_dmc_table_matches_reference_digest():
    table = omesh.dmc_table()
    pinned = json.load(open(GOLDEN))
    assert len(table) == pinned["cases"] == 256
    assert sum(len(row) for row in table) == pinned["dual_points"]
    assert omesh.dmc_table_digest(table) == pinned["sha256"]


def test_dmc_pieces_partition_the_cut_edges():
    for case, row in enumerate(omesh.dmc_table()):
        cut = sum(1 << e for e, (a, b) in enumerate(omesh.DMC_EDGE_CORNERS) if ((case >> a) & 1) != ((case >> b) & 1))
        union = 0
        for piece in row:
            assert piece and not (piece & union)
            union |= piece
        assert union == cut
        # the complementary case cuts the same edges
        comp_union = 0
        for piece in omesh.dmc_dual_points(255 - case):
            comp_union |= piece
        assert comp_union == cut


def sphere_densities(size, centre, radius):
    sg = size + 4
    r = np.arange(sg, dtype=np.float64) - 2
    z, y, x = np.meshgrid(r, r, r, indexing="ij")
    d = np.sqrt((x - centre[0]) ** 2 + (y - centre[1]) ** 2 + (z - centre[2]) ** 2) - radius
    d = d.astype(np.float32).ravel()
    return d, (d.min(), d.max())


def test_dmc_sphere_is_closed_and_oriented():
    size = 12
    d, mm = sphere_densities(size, (5.5, 6.25, 5.75), 3.6)
    verts, idx, min_air, max_solid = omesh.dmc_mesh(d, mm, size, (0, 0, 0), 0.0)
    assert len(idx) % 6 == 0 and len(idx) > 0
    assert idx.max() < len(verts) and len(np.unique(idx)) == len(verts)    # every vertex used
    directed = Counter()
    for t in idx.reshape(-1, 3):
        for k in range(3):
            directed[(int(t[k]), int(t[(k + 1) % 3]))] += 1
    # closed two-manifold with consistent winding: each directed edge once, its reverse once
    for (a, b), n in directed.items():
        assert n == 1 and directed[(b, a)] == 1
    # vertices near the sphere, lights in [0, 1]
    r = np.linalg.norm(verts[:, :3] - np.array([5.5, 6.25, 5.75], np.float32), axis=1)
    assert np.all(np.abs(r - 3.6) < 0.6)
    assert np.all((verts[:, 3] >= 0) & (verts[:, 3] <= 1))
    assert min_air < max_solid


def test_dmc_early_out():
    size = 6
    d = np.full((size + 4) ** 3, 0.5, np.float32)
    v, i, air, solid = omesh.dmc_mesh(d, (0.5, 0.5), size, (3, 16, -2), 0.0)
    assert len(v) == 0 and len(i) == 0 and air == 16.0 and solid == float("-inf")
    v, i, air, solid = omesh.dmc_mesh(-d, (-0.5, -0.5), size, (3, 16, -2), 0.0)
    assert len(v) == 0 and air == float("inf") and solid == 16.0 - 1.0 + size
