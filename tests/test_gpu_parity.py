"""GPU parity: every node kind, dimensionality and batch driver against the CPU oracle.

Runs through the reference-facing C-ABI (fnGenUniformGrid*/fnGenPositionArray*/
fnGenTileable2D/fnGenSingle*) with host buffers, on seeded inputs small enough
for the oracle to finish in seconds.
"""
import numpy as np
import pytest

from oracle.tree import N, decode
from tests import trees
from tests.parity import assert_parity, run_grid, run_positions, run_tileable

pytestmark = pytest.mark.gpu

GRID = {2: ((-7.5, 3.25), (37, 29), (1.5, 0.75)),
        3: ((-7.5, 3.25, 11.0), (13, 11, 9), (1.5, 0.75, 1.25)),
        4: ((-7.5, 3.25, 11.0, -2.0), (7, 6, 5, 4), (1.5, 0.75, 1.25, 2.0))}


def noise(name, scale=3.7, **kw):
    return N(name, Feature_Scale=scale, **kw)


def cellular(name, df="Euclidean Squared", **kw):
    n = N(name, Feature_Scale=3.1)
    n.set("Distance Function", df)
    for k, v in kw.items():
        n.set(k.replace("_", " "), v)
    return n


def warp_simplex(name, scheme):
    n = N(name, Source=noise("Value", 6.0), Warp_Amplitude=3.5, Feature_Scale=4.5, Seed_Offset=-3)
    n.set("Vectorization Scheme", scheme)
    n.set("Warp Amplitude", noise("Simplex", 30.0))          # node-driven amplitude
    n.set("Amplitude Scaling", 0.75, 0)
    return n


SINGLE = {
    "Constant": lambda: N("Constant", Value=0.625),
    "White": lambda: N("White", Seed_Offset=3),
    "Checkerboard": lambda: noise("Checkerboard", 2.5),
    "SineWave": lambda: noise("SineWave", 5.0),
    "Gradient": lambda: N("Gradient").set("Multiplier", 0.25, 0).set("Multiplier", -0.5, 1).set("Multiplier", 0.125, 2)
                                    .set("Multiplier", 1.0, 3).set("Offset", 3.0, 0),
    "DistanceToPoint": lambda: N("DistanceToPoint").set("Point", 1.5, 0).set("Point", -2.0, 1),
    "Simplex": lambda: noise("Simplex"),
    "SuperSimplex": lambda: noise("SuperSimplex"),
    "Perlin": lambda: noise("Perlin"),
    "Value": lambda: noise("Value"),
    "SimplexRange": lambda: noise("Simplex", Seed_Offset=-17, Output_Min=0.2, Output_Max=3.5),
    "CellularValue": lambda: cellular("CellularValue"),
    "CellularValueIdx2": lambda: cellular("CellularValue", "Manhattan", Value_Index=2),
    "CellularDistance": lambda: cellular("CellularDistance"),
    "CellularDistanceSub": lambda: cellular("CellularDistance", "Euclidean", Return_Type="Index0Sub1"),
    "CellularDistanceHybrid": lambda: cellular("CellularDistance", "Hybrid", Return_Type="Index0Add1", Distance_Index_1=2),
    "CellularDistanceMax": lambda: cellular("CellularDistance", "Max Axis", Return_Type="Index0Mul1"),
    "CellularDistanceDiv": lambda: cellular("CellularDistance", "Euclidean", Return_Type="Index0Div1", Distance_Index_0=1, Distance_Index_1=3),
    "CellularDistanceMinkowski": lambda: cellular("CellularDistance", "Minkowski", Minkowski_P=1.7),
    "CellularJitter": lambda: cellular("CellularDistance", Grid_Jitter=0.6, Size_Jitter=0.4),
    "CellularLookup": lambda: N("CellularLookup", Feature_Scale=4.0, Lookup=noise("Perlin", 9.0)),
    # parameters that change which cells the walk may skip
    "CellularNegJitter": lambda: cellular("CellularValue", "Euclidean", Grid_Jitter=-0.8),
    "CellularSizeShrink": lambda: cellular("CellularValue", "Manhattan", Size_Jitter=-0.5),
    "CellularSizeNegative": lambda: cellular("CellularDistance", "Euclidean", Size_Jitter=-1.5, Return_Type="Index0Add1"),
    "CellularValueHybrid": lambda: cellular("CellularValue", "Hybrid", Value_Index=1, Grid_Jitter=1.3),
    "CellularLookupManhattan": lambda: N("CellularLookup", Feature_Scale=2.9, Lookup=noise("Simplex", 9.0))
                                       .set("Distance Function", "Manhattan").set("Size Jitter", 0.3),
    "CellularJitterNode": lambda: N("CellularLookup", Feature_Scale=3.3, Lookup=noise("Value", 5.0),
                                    Grid_Jitter=noise("Simplex", 9.0)),
}

COMPOSITE = {
    "FBm": lambda: N("FractalFBm", Source=noise("Simplex"), Octaves=4, Lacunarity=1.87, Gain=0.6, Weighted_Strength=0.3),
    "Ridged": lambda: N("FractalRidged", Source=noise("Perlin"), Octaves=3, Weighted_Strength=0.7),
    "FBmGainNode": lambda: N("FractalFBm", Source=noise("Value"), Gain=noise("Simplex", 20.0)),
    "PingPong": lambda: N("PingPong", Source=noise("Simplex"), Ping_Pong_Strength=2.7),
    "WarpGradient": lambda: N("DomainWarpGradient", Source=noise("Simplex"), Warp_Amplitude=4.0, Feature_Scale=6.0, Seed_Offset=5),
    "WarpProgressive": lambda: N("DomainWarpFractalProgressive",
                                 Domain_Warp_Source=N("DomainWarpGradient", Source=noise("Perlin"), Warp_Amplitude=3.0, Feature_Scale=7.0),
                                 Octaves=3, Weighted_Strength=0.4),
    "WarpSimplexOGM": lambda: warp_simplex("DomainWarpSimplex", "Orthogonal Gradient Matrix"),
    "WarpSimplexGOP": lambda: warp_simplex("DomainWarpSimplex", "Gradient Outer Product"),
    "WarpSuperOGM": lambda: warp_simplex("DomainWarpSuperSimplex", "Orthogonal Gradient Matrix"),
    "WarpSuperGOP": lambda: warp_simplex("DomainWarpSuperSimplex", "Gradient Outer Product"),
    "WarpProgressiveSuper": lambda: N("DomainWarpFractalProgressive",
                                      Domain_Warp_Source=warp_simplex("DomainWarpSuperSimplex", "Gradient Outer Product"),
                                      Octaves=3, Gain=0.6),
    "WarpIndependentSimplex": lambda: N("DomainWarpFractalIndependent",
                                        Domain_Warp_Source=warp_simplex("DomainWarpSimplex", "Orthogonal Gradient Matrix"),
                                        Octaves=3, Weighted_Strength=0.5),
    "WarpIndependent": lambda: N("DomainWarpFractalIndependent",
                                 Domain_Warp_Source=N("DomainWarpGradient", Source=noise("Value"), Warp_Amplitude=2.0, Feature_Scale=5.0),
                                 Octaves=4, Gain=0.7),
    "Add": lambda: N("Add", LHS=noise("Simplex"), RHS=noise("Perlin")),
    "Subtract": lambda: N("Subtract", LHS=noise("Simplex"), RHS=0.25),
    "Multiply": lambda: N("Multiply", LHS=noise("Simplex"), RHS=noise("Value")),
    "Divide": lambda: N("Divide", LHS=noise("Simplex"), RHS=1.7),
    "Modulus": lambda: N("Modulus", LHS=noise("Simplex", 9.0), RHS=0.3),
    "Min": lambda: N("Min", LHS=noise("Simplex"), RHS=noise("Perlin")),
    "Max": lambda: N("Max", LHS=noise("Simplex"), RHS=0.1),
    "MinSmooth": lambda: N("MinSmooth", LHS=noise("Simplex"), RHS=noise("Perlin"), Smoothness=0.35),
    "MaxSmooth": lambda: N("MaxSmooth", LHS=noise("Simplex"), RHS=noise("Value"), Smoothness=0.2),
    "Abs": lambda: N("Abs", Source=noise("Simplex")),
    "SignedSquareRoot": lambda: N("SignedSquareRoot", Source=noise("Perlin")),
    "PowFloat": lambda: N("PowFloat", Value=noise("Simplex"), Pow=1.6),
    "PowInt": lambda: N("PowInt", Value=noise("Simplex"), Pow=5),
    "DomainScale": lambda: N("DomainScale", Source=noise("Simplex"), Scaling=1.37),
    "DomainOffset": lambda: N("DomainOffset", Source=noise("Simplex")).set("Offset", 2.5, 0).set("Offset", noise("Perlin", 8.0), 1),
    "DomainRotate": lambda: N("DomainRotate", Source=noise("Simplex"), Yaw=0.7, Pitch=0.3, Roll=-0.4),
    "DomainRotateYaw": lambda: N("DomainRotate", Source=noise("Simplex"), Yaw=1.1),
    "DomainAxisScale": lambda: N("DomainAxisScale", Source=noise("Simplex")).set("Scaling", 0.5, 0).set("Scaling", 2.0, 2),
    "SeedOffset": lambda: N("SeedOffset", Source=noise("Simplex"), Seed_Offset=99),
    "ConvertRGBA8": lambda: N("ConvertRGBA8", Source=noise("Simplex")),
    "GeneratorCache": lambda: N("GeneratorCache", Source=noise("Simplex")),
    "Fade": lambda: N("Fade", A=noise("Simplex"), B=noise("Perlin"), Fade=noise("Value", 11.0), Interpolation="Quintic"),
    "FadeConst": lambda: N("Fade", A=noise("Simplex"), B=noise("Perlin"), Fade=0.25, Interpolation="Hermite"),
    "Remap": lambda: N("Remap", Source=noise("Simplex"), From_Min=-0.5, To_Max=4.0, Clamp_Output="True"),
    "Terrace": lambda: N("Terrace", Source=noise("Simplex"), Step_Count=5.0, Smoothness=0.45),
    "TerraceDynamic": lambda: N("Terrace", Source=noise("Simplex"), Step_Count=3.0, Smoothness=noise("Perlin", 13.0)),
    "AddDimension": lambda: N("AddDimension", Source=noise("Simplex"), New_Dimension_Position=noise("Value", 5.0)),
    "RemoveDimension": lambda: N("RemoveDimension", Source=noise("Simplex"), Remove_Dimension="X"),
    "DomainRotatePlane": lambda: N("DomainRotatePlane", Source=noise("Simplex"), Rotation_Type="Improve XZ Planes"),
    "Terrain": trees.terrain_c2,
}


@pytest.mark.parametrize("dim", [2, 3, 4])
@pytest.mark.parametrize("name", sorted(SINGLE))
def test_single_node_grid(gpu, name, dim):
    off, cnt, st = GRID[dim]
    assert_parity(*run_grid(SINGLE[name](), off, cnt, st, 1337), label=f"{name}/{dim}D")


@pytest.mark.parametrize("dim", [2, 3, 4])
@pytest.mark.parametrize("name", sorted(COMPOSITE))
def test_composite_grid(gpu, name, dim):
    off, cnt, st = GRID[dim]
    assert_parity(*run_grid(COMPOSITE[name](), off, cnt, st, -42), label=f"{name}/{dim}D",
                  nan_equal=name != "ConvertRGBA8")


TIE_GRID = {2: ((-3.0, -2.5), (29, 27), (0.25, 0.25)),
            3: ((-3.0, -2.5, -1.75), (15, 13, 11), (0.25, 0.25, 0.25)),
            4: ((-3.0, -2.5, -1.75, -1.0), (9, 7, 7, 5), (0.25, 0.25, 0.25, 0.25))}


@pytest.mark.parametrize("dim", [2, 3, 4])
@pytest.mark.parametrize("kind,df,extra", [
    ("CellularValue", "Euclidean Squared", {}),
    ("CellularValue", "Manhattan", {"Value Index": 1}),
    ("CellularValue", "Max Axis", {}),
    ("CellularLookup", "Euclidean", {}),
    ("CellularLookup", "Max Axis", {}),
    ("CellularDistance", "Manhattan", {"Return Type": "Index0Sub1"}),
])
def test_cellular_ties(gpu, kind, df, extra, dim):
    """Grid jitter 0 puts every cell point on its lattice point; positions on a quarter grid at
    frequency 1 are then often equidistant from several cells, and the cell the reference visits
    first must win the tie whatever order the walk visits them in."""
    n = N(kind, Feature_Scale=1.0, Grid_Jitter=0.0) if kind != "CellularLookup" else \
        N(kind, Feature_Scale=1.0, Grid_Jitter=0.0, Lookup=noise("Value", 0.7))
    n.set("Distance Function", df)
    for k, v in extra.items():
        n.set(k, v)
    off, cnt, st = TIE_GRID[dim]
    assert_parity(*run_grid(n, off, cnt, st, 77), label=f"{kind}/{df}/{dim}D ties")


@pytest.mark.parametrize("seed", [0, 1337, -1, 2**31 - 1, -(2**31)])
def test_seeds(gpu, seed):
    assert_parity(*run_grid(COMPOSITE["Terrain"](), (0, 0, 0), (9, 8, 7), (3.0, 3.0, 3.0), seed), label=f"seed {seed}")


def test_workload0_simplex_64cubed(gpu):
    """Simplex, scale 50, 64^3 from the origin, seed 1337 (the reference's config-0 case)."""
    assert_parity(*run_grid(trees.simplex_c0(), (0, 0, 0), (64, 64, 64), (1, 1, 1), 1337), label="c0")


def test_workload1_fbm_perlin_reduced(gpu):
    assert_parity(*run_grid(trees.fbm_perlin_c1(), (-128, -128, -128), (40, 36, 32), (1, 1, 1), 42), label="c1")


def test_workload2_terrain_tileable_reduced(gpu):
    assert_parity(*run_tileable(trees.terrain_c2(), (96, 80), (1.0, 1.0), 7), label="c2 tileable")


def test_workload2_terrain_grid_reduced(gpu):
    assert_parity(*run_grid(trees.terrain_c2(), (0, 0, 0), (24, 24, 24), (1, 1, 1), 7), label="c2 3D")


def test_demo_caves_tree(gpu):
    root = decode(trees.DEMO_CAVES)
    assert_parity(*run_grid(root, (-40, 12, 5), (48, 40, 12), (1, 1, 1), 1337), label="caves")


@pytest.mark.parametrize("dim", [2, 3])
def test_demo_mountain_tree(gpu, dim):
    """The Node Editor's mountain demo (DomainWarpSimplex inside a fractal warp)."""
    root = decode(trees.DEMO_MOUNTAIN)
    off, cnt = ((-60, 25), (96, 80)) if dim == 2 else ((-60, 25, 3), (40, 36, 12))
    assert_parity(*run_grid(root, off, cnt, (1,) * dim, 1337), label=f"mountain {dim}D")


@pytest.mark.parametrize("dim", [2, 3, 4])
def test_position_arrays(gpu, dim):
    rng = np.random.default_rng(20261203 + dim)
    count = 3001
    pos = [rng.uniform(-1e4, 1e4, count).astype(np.float32) for _ in range(dim)]
    off = [0.5, -3.0, 7.25, 1.0][:dim]
    assert_parity(*run_positions(COMPOSITE["FBm"](), pos, off, 77), label=f"positions {dim}D")


def test_position_array_matches_grid(gpu):
    """GenPositionArray3D over the grid's own positions reproduces GenUniformGrid3D."""
    from tests.trees import to_product
    root = trees.fbm_perlin_c1()
    prod = to_product(root)
    g, gmm = prod.gen_uniform_grid((0, 0, 0), (16, 8, 4), (1, 1, 1), 5)
    z, y, x = np.meshgrid(np.arange(4), np.arange(8), np.arange(16), indexing="ij")
    p, pmm = prod.gen_position_array([x.ravel().astype(np.float32), y.ravel().astype(np.float32),
                                      z.ravel().astype(np.float32)], (0, 0, 0), 5)
    assert np.array_equal(g.view(np.uint32), p.view(np.uint32))
    assert gmm == pmm


def test_single_matches_grid(gpu):
    from tests.trees import to_product
    prod = to_product(trees.terrain_c2())
    g, _ = prod.gen_uniform_grid((3, 4, 5), (4, 3, 2), (1, 1, 1), 7)
    idx = 1 * 12 + 2 * 4 + 3        # z=1, y=2, x=3
    assert prod.gen_single((6.0, 6.0, 6.0), 7) == g[idx]


@pytest.mark.parametrize("cnt", [(1, 1), (1, 7), (33, 1), (257, 3), (0, 5)])
def test_ragged_and_empty_2d(gpu, cnt):
    g, gmm, o, omm = run_grid(N("Simplex", Feature_Scale=2.0), (0.5, 0.25), cnt, (1, 1), 3)
    if cnt[0] * cnt[1] == 0:
        assert g.size == 0 and gmm == (float("inf"), float("-inf"))
    else:
        assert_parity(g, gmm, o, omm, label=str(cnt))


def test_large_coordinates(gpu):
    assert_parity(*run_grid(COMPOSITE["Terrain"](), (-1.0e6, 2.5e6, 7.0e5), (9, 9, 9), (97.0, 31.0, 11.0), 11), label="far")


def test_unfused_oracle_mode_is_close(gpu):
    """The scalar-build (unfused) reading of FS::FMulAdd stays within the tolerance of the fused one."""
    from oracle.oracle import OracleTree
    root = trees.fbm_perlin_c1()
    a, _ = OracleTree(root).grid((0, 0, 0), (16, 16, 16), (1, 1, 1), 42)
    b, _ = OracleTree(root, unfused=True).grid((0, 0, 0), (16, 16, 16), (1, 1, 1), 42)
    assert np.max(np.abs(a - b)) < 1e-5


@pytest.mark.parametrize("dim", [2, 3, 4])
@pytest.mark.parametrize("name", ["CellularValue", "CellularDistance", "CellularLookup"])
def test_node_driven_minkowski(gpu, name, dim):
    """Minkowski P from a node, sampled at each cell's offset vector: the tree is
    specialised automatically on first use (the interpreter cannot run it)."""
    off, cnt, st = GRID[dim]
    assert_parity(*run_grid(trees.minkowski_node_tree(name), off, cnt, st, 1337), label=f"{name} {dim}D")


def test_node_driven_minkowski_needs_specialisation(gpu):
    import fastnoise2_gb300 as fn
    node = trees.to_product(trees.minkowski_node_tree())
    was = fn.set_jit_enabled(False)
    try:
        with pytest.raises(fn.FastNoiseError) as e:
            node.gen_uniform_grid((0, 0), (8, 8), (1, 1), 1)
        assert e.value.code == -2
    finally:
        fn.set_jit_enabled(was)


@pytest.mark.parametrize("name", ["Perlin", "Value", "Simplex", "SuperSimplex", "CellularDistance", "CellularValue"])
@pytest.mark.parametrize("dim", [2, 3])
def test_out_of_range_lattice_coordinates(gpu, name, dim):
    """Coordinates at and beyond +-2^31: the lattice index conversion must give INT_MIN out of
    range (x86 cvtps2dq) exactly as the oracle does."""
    vals = np.array([0.5, 1e10, -1e10, 2147483648.0, -2147483904.0, 2147483520.0, -2147483648.0,
                     3.0e9, -3.0e9, 123.25], np.float32)
    rng = np.random.default_rng(3)
    pos = [rng.permutation(np.tile(vals, 4)).astype(np.float32) for _ in range(dim)]
    root = N(name, Feature_Scale=1.0)
    g, gmm, o, omm = run_positions(root, pos, (0.0,) * dim, 1337)
    assert_parity(g, gmm, o, omm, label=f"{name} {dim}D out of range")
