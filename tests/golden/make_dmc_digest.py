"""Generate tests/golden/dmc_table.json from the reference's dual marching cubes table.

Reads tools/NodeEditor/util/DmcTable.inl of a FastNoise2 checkout (as text), parses
kDualPointsList[256][4] (edge bit sets joined with |), and stores only a SHA-256 of its
canonical form -- per case, the nonzero point codes sorted -- plus the number of cases
and of dual points.  tests/test_mesh_oracle.py checks that oracle/mesh.py's derived
table has the same digest, so the derivation is pinned to the reference's table without
a copy of it in this repository.

Run from the repository root:  python tests/golden/make_dmc_digest.py /path/to/FastNoise2
"""
import json
import os
import re
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle.mesh import dmc_table_digest  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "dmc_table.json")


def parse(path: str):
    src = open(path).read()
    body = src[src.index("kDualPointsList[256][4]"):]
    rows = re.findall(r"\{([^{}]*)\},?\s*//\s*(\d+)", body)
    table = []
    for n, (row, case) in enumerate(rows):
        assert int(case) == n
        codes = []
        for entry in row.split(","):
            entry = entry.strip()
            code = 0
            if entry != "0":
                for term in entry.split("|"):
                    code |= 1 << int(term.strip()[len("EDGE"):])
            codes.append(code)
        table.append(codes)
    assert len(table) == 256
    return table


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_dmc_digest.py /path/to/FastNoise2")
    ref_root = sys.argv[1]
    table = parse(os.path.join(ref_root, "tools", "NodeEditor", "util", "DmcTable.inl"))
    out = {
        "source": "tools/NodeEditor/util/DmcTable.inl kDualPointsList",
        "cases": len(table),
        "dual_points": sum(1 for row in table for c in row if c),
        "sha256": dmc_table_digest(table),
    }
    with open(OUT, "w") as f:
        json.dump(out, f, indent=1)
        f.write("\n")
    print(out)


if __name__ == "__main__":
    main()
