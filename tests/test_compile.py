"""Host-side tree compiler (CPU only): every tested tree flattens into a device program."""
import pytest

from oracle.tree import N, decode
from tests import trees
from tests.test_gpu_parity import COMPOSITE, SINGLE


@pytest.mark.parametrize("dim", [2, 3, 4])
@pytest.mark.parametrize("name", sorted({**SINGLE, **COMPOSITE}))
def test_tree_compiles(native, name, dim):
    prod = trees.to_product({**SINGLE, **COMPOSITE}[name]())
    n_instr, n_regs = prod.compile_info(dim)
    assert 1 <= n_instr and 1 <= n_regs <= 64


def test_workload_trees_compile(native):
    for make in trees.MIX_TREES:
        for dim in (2, 3, 4):
            trees.to_product(make()).compile_info(dim)
    trees.to_product(decode(trees.DEMO_CAVES)).compile_info(3)


def test_unsupported_nodes_report_compile_error(native):
    node = trees.to_product(trees.unsupported_tree())
    with pytest.raises(native.FastNoiseError) as e:
        node.compile_info(2)
    assert e.value.code == -2 and "registers" in e.value.message


@pytest.mark.parametrize("name", ["CellularValue", "CellularDistance", "CellularLookup"])
def test_node_driven_minkowski_compiles_and_specialises(native, name):
    """Minkowski P driven by a node becomes a per-cell sub-program; the specialised
    kernels (NVRTC, no GPU needed to compile) evaluate it."""
    node = trees.to_product(trees.minkowski_node_tree(name))
    for dim in (2, 3, 4):
        n_instr, _ = node.compile_info(dim)
        assert n_instr > 0
        assert native.jit_check([(node, dim)]) > 0


def test_demo_trees_compile(native):
    for enc in (trees.DEMO_MOUNTAIN, trees.DEMO_CAVES):
        node = native.Node.from_encoded(enc)
        for dim in (2, 3, 4):
            n_instr, n_regs = node.compile_info(dim)
            assert 0 < n_instr and 0 < n_regs <= 64


def test_missing_source_is_a_compile_error(native):
    with pytest.raises(native.FastNoiseError):
        native.Node.new("FractalFBm").compile_info(3)


def test_octave_count_scales_program(native):
    short = trees.to_product(N("FractalFBm", Source=N("Perlin"), Octaves=2)).compile_info(3)[0]
    long = trees.to_product(N("FractalFBm", Source=N("Perlin"), Octaves=9)).compile_info(3)[0]
    assert long > short
