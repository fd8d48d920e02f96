"""Generate tests/golden/oracle_golden.json from the CPU oracle.

The reference ships no golden values for this path (its tests are a throughput
harness and an include smoke test), so these fixtures pin the oracle against
its own earlier output: any change to the oracle's arithmetic shows up as a
digest mismatch in tests/test_oracle.py.  Each case stores the tree as an
encoded node-tree string, the call, a SHA-256 of the float32 output bytes,
the OutputMinMax and a few sample values.

Run from the repository root:  python tests/golden/make_golden.py
"""
import hashlib
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle.oracle import OracleTree  # noqa: E402
from oracle.tree import decode, encode  # noqa: E402
from tests import trees  # noqa: E402
from tests.test_gpu_parity import COMPOSITE, GRID, SINGLE  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "oracle_golden.json")


def digest(values: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(values, np.float32).tobytes()).hexdigest()


def case(name, root, kind, args, seed):
    t = OracleTree(root)
    if kind == "grid":
        v, mm = t.grid(*args, seed)
    else:
        v, mm = t.tileable(*args, seed)
    return {"name": name, "tree": encode(root), "kind": kind, "args": args, "seed": seed,
            "sha256": digest(v), "min": mm[0], "max": mm[1],
            "sample": [float(x) for x in v[:: max(1, len(v) // 8)][:8]]}


def main():
    cases = []
    for name, make in sorted({**SINGLE, **COMPOSITE}.items()):
        for dim in (2, 3, 4):
            off, cnt, st = GRID[dim]
            cases.append(case(f"{name}/{dim}D", make(), "grid", [list(off), list(cnt), list(st)], 1337))
    cases.append(case("workload0", trees.simplex_c0(), "grid", [[0, 0, 0], [32, 32, 32], [1, 1, 1]], 1337))
    cases.append(case("workload1", trees.fbm_perlin_c1(), "grid", [[-128, -128, -128], [24, 24, 24], [1, 1, 1]], 42))
    cases.append(case("workload2-tileable", trees.terrain_c2(), "tile", [48, 40, 1.0, 1.0], 7))
    cases.append(case("demo-caves", decode(trees.DEMO_CAVES), "grid", [[-40, 12, 5], [24, 20, 6], [1, 1, 1]], 1337))
    cases.append(case("demo-mountain", decode(trees.DEMO_MOUNTAIN), "grid", [[-60, 25], [48, 40], [1, 1]], 1337))
    for name in ("CellularValue", "CellularDistance", "CellularLookup"):
        for dim in (2, 3, 4):
            off, cnt, st = GRID[dim]
            cases.append(case(f"MinkowskiNode-{name}/{dim}D", trees.minkowski_node_tree(name), "grid",
                              [list(off), list(cnt), list(st)], 1337))
    with open(OUT, "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py", "cases": cases}, f, indent=1)
    print(f"wrote {len(cases)} cases to {OUT}")


if __name__ == "__main__":
    main()
