"""Node trees used by the parity tests and the benchmark (test helpers).

Trees are described once with the oracle's tree model (``oracle.tree``) and
handed to the product through its public C-ABI by :func:`to_product`, which
replays the same setter calls a binding would make (fnNewFromMetadata,
fnSetVariable*, fnSetNodeLookup, fnSetHybrid*).
"""
from __future__ import annotations

from typing import Dict, List

from oracle.tree import N, Node, walk


def simplex_c0() -> Node:
    """Workload 0: Simplex with feature scale 50 (frequency 0.02)."""
    return N("Simplex", Feature_Scale=50.0)


def fbm_perlin_c1() -> Node:
    """Workload 1: FractalFBm over Perlin, 5 octaves, gain 0.5, lacunarity 2, weighted strength 0."""
    return N("FractalFBm", Source=N("Perlin"), Octaves=5, Gain=0.5, Lacunarity=2.0, Weighted_Strength=0.0)


def terrain_c2() -> Node:
    """Workload 2: domain-warped ridged SuperSimplex faded with CellularDistance, remapped and terraced."""
    ridged = N("FractalRidged", Source=N("SuperSimplex"), Octaves=4)
    warp = N("DomainWarpGradient", Source=ridged, Warp_Amplitude=30.0)
    warp_fractal = N("DomainWarpFractalProgressive", Domain_Warp_Source=warp, Octaves=3)
    cells = N("CellularDistance")
    cells.set("Distance Function", "Euclidean")
    cells.set("Distance Index 0", 0)
    cells.set("Distance Index 1", 1)
    cells.set("Return Type", "Index0Sub1")
    cells.set("Grid Jitter", 1.0)
    fade = N("Fade", A=warp_fractal, B=cells)
    remap = N("Remap", Source=fade)
    remap.set("From Min", -1.0).set("From Max", 1.0).set("To Min", 0.0).set("To Max", 1.0)
    terrace = N("Terrace", Source=remap, Step_Count=8.0, Smoothness=0.3)
    return terrace


def value_tree() -> Node:
    return N("Value")


def cellular_value_tree() -> Node:
    return N("CellularValue")


def cellular_lookup_tree() -> Node:
    return N("CellularLookup", Lookup=N("Simplex"))


def fbm_simplex_tree() -> Node:
    return N("FractalFBm", Source=N("Simplex"), Octaves=3)


def blend_tree() -> Node:
    return N("Add", LHS=N("Simplex"), RHS=N("Multiply", LHS=N("Perlin"), RHS=N("Value")))


MIX_TREES = [simplex_c0, fbm_perlin_c1, terrain_c2, value_tree, cellular_value_tree, cellular_lookup_tree,
             fbm_simplex_tree, blend_tree]

# Demo trees shipped with the reference (tools/NodeEditor/util/DemoNodeTrees.inl:5-6)
DEMO_MOUNTAIN = "E@BBZEG@BD8JFgIECArXIzwECiQIw/UoPwkuAAE@BJDQAH@BC@AIEAJBw@ABZEED0KV78YZmZmPwQDmpkZPwsAAIA/HAMAAHBCBA=="
DEMO_CAVES = ("FgIcCS4AAQ@BklCQs@BlRBDNzMw9G@AIMAgAw@ADgC@BCiQIzczMPgkJ@BPkIQH4XrPhjNzEw/DBIkCM3MzD4JCQ@ADBCCAE@BQzczMvhg@B/"
              "JAL/BAAL7FE4PgQKFwkNCQg@CQQQDuB4FPwt7FC4/BAOPwnU8DA==")


def unsupported_tree() -> Node:
    """A tree the GPU compiler rejects: a right-deep chain of blends whose pending
    left operands need more than the program's 64 live registers."""
    n = N("Simplex")
    for i in range(70):
        n = N("Add", LHS=N("Value", Seed_Offset=i), RHS=n)
    return n


def minkowski_node_tree(name: str = "CellularDistance") -> Node:
    """A cellular node whose Minkowski P is driven by another node (evaluated at
    every cell's offset vector)."""
    n = N(name, Feature_Scale=3.3, Minkowski_P=N("Value", Feature_Scale=0.8, Output_Min=0.6, Output_Max=3.0))
    n.set("Distance Function", "Minkowski")
    if name == "CellularLookup":
        n.set("Lookup", N("Perlin", Feature_Scale=9.0))
    return n


def to_product(root: Node):
    """Instantiate `root` in the product library through the C-ABI setters."""
    import fastnoise2_gb300 as fn
    L = fn.lib()
    handles: Dict[int, object] = {}
    for node in walk(root):
        h = fn.Node(L.fnNewFromMetadata(node.meta.id, 0))
        for kind, idx, arg in node.ops:
            if kind == "var":
                ok = L.fnSetVariableIntEnum(h.handle, idx, int(arg))
            elif kind == "lookup":
                ok = L.fnSetNodeLookup(h.handle, idx, handles[id(arg)].handle)
            elif kind == "hnode":
                ok = L.fnSetHybridNodeLookup(h.handle, idx, handles[id(arg)].handle)
            else:
                ok = L.fnSetHybridFloat(h.handle, idx, float(arg))
            assert ok, (node.meta.name, kind, idx)
        handles[id(node)] = h
    return handles[id(root)]
