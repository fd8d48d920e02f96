"""Encoded node trees and metadata (CPU only; no generation calls).

Pins: the reference's two demo trees (tools/NodeEditor/util/DemoNodeTrees.inl:5-6)
decode and re-encode byte-identically, in the oracle's Python codec and in the
product's C++ codec -- which also pins node ids and member order, because the
encoding addresses members by metadata index (src/FastNoise/Metadata.cpp:214-287).
"""
import pytest

from oracle import tree as T
from tests import trees


@pytest.mark.parametrize("encoded", [trees.DEMO_MOUNTAIN, trees.DEMO_CAVES])
def test_oracle_codec_roundtrips_demo_trees(encoded):
    root = T.decode(encoded)
    assert root is not None
    assert T.encode(root) == encoded


@pytest.mark.parametrize("encoded", [trees.DEMO_MOUNTAIN, trees.DEMO_CAVES])
def test_product_codec_roundtrips_demo_trees(native, encoded):
    node = native.Node.from_encoded(encoded)
    assert node is not None
    assert node.encode() == encoded


@pytest.mark.parametrize("make", trees.MIX_TREES, ids=lambda f: f.__name__)
def test_encode_matches_between_oracle_and_product(native, make):
    root = make()
    enc = T.encode(root)
    prod = trees.to_product(root)
    assert prod.encode() == enc
    again = native.Node.from_encoded(enc)
    assert again is not None and again.encode() == enc


@pytest.mark.parametrize("bad", ["", "@", "A", "AAAA", "!!!!", "/w==", "E@BBZEG", "@!AA", "BAAAAAAA", "/wAA"])
def test_malformed_trees_return_null(native, bad):
    assert T.decode(bad) is None
    assert native.Node.from_encoded(bad) is None


def test_base64_run_length_roundtrip():
    for n in (0, 1, 2, 3, 4, 5, 40, 49, 50, 51, 100):
        data = bytes([7]) + bytes(n) + bytes([9, 1, 2])
        enc = T.b64_encode(data)
        assert T.b64_decode(enc) == data, n


def test_metadata_tables_match(native):
    L = native.lib()
    assert L.fnGetMetadataCount() == len(T.META) == 47
    for m in T.META:
        i = m.id
        assert L.fnGetMetadataName(i).decode() == m.name
        assert L.fnGetMetadataVariableCount(i) == len(m.variables)
        for k, v in enumerate(m.variables):
            assert L.fnGetMetadataVariableName(i, k).decode() == v.name
            assert L.fnGetMetadataVariableType(i, k) == v.type
            assert L.fnGetMetadataVariableDimensionIdx(i, k) == v.dim
            assert L.fnGetMetadataVariableDefaultIntEnum(i, k) == v.default
            assert L.fnGetMetadataEnumCount(i, k) == len(v.enums)
            for e, name in enumerate(v.enums):
                assert L.fnGetMetadataEnumName(i, k, e).decode() == name
        assert L.fnGetMetadataNodeLookupCount(i) == len(m.lookups)
        for k, l in enumerate(m.lookups):
            assert L.fnGetMetadataNodeLookupName(i, k).decode() == l.name
            assert L.fnGetMetadataNodeLookupDimensionIdx(i, k) == l.dim
        assert L.fnGetMetadataHybridCount(i) == len(m.hybrids)
        for k, h in enumerate(m.hybrids):
            assert L.fnGetMetadataHybridName(i, k).decode() == h.name
            assert L.fnGetMetadataHybridDimensionIdx(i, k) == h.dim
            assert L.fnGetMetadataHybridDefault(i, k) == pytest.approx(h.default)
        assert [L.fnGetMetadataGroupName(i, g).decode() for g in range(L.fnGetMetadataGroupCount(i))] == list(m.groups)


def test_metadata_sentinels(native):
    L = native.lib()
    assert L.fnGetMetadataName(47).decode() == "INVALID NODE ID"
    assert L.fnGetMetadataName(-1).decode() == "INVALID NODE ID"
    assert L.fnGetMetadataVariableCount(99) == -1
    assert L.fnGetMetadataVariableName(6, 99).decode() == "INVALID VARIABLE INDEX"
    assert L.fnGetMetadataEnumName(11, 4, 99).decode() == "INVALID ENUM INDEX"
    assert L.fnNewFromMetadata(200, 0) is None
    L.fnDeleteNodeRef(None)   # no-op per the reference header


def test_setters_reject_wrong_types(native):
    warp_fractal = native.Node.new("DomainWarpFractalProgressive")
    simplex = native.Node.new("Simplex")
    L = native.lib()
    assert not L.fnSetNodeLookup(warp_fractal.handle, 0, simplex.handle)      # needs a DomainWarp node
    assert L.fnSetNodeLookup(warp_fractal.handle, 0, native.Node.new("DomainWarpGradient").handle)
    assert not L.fnSetVariableFloat(simplex.handle, 99, 1.0)
    assert not L.fnSetHybridFloat(simplex.handle, 0, 1.0)                     # Simplex has no hybrids


def test_reference_counting_keeps_children_alive(native):
    fbm = native.Node.new("FractalFBm")
    child = native.Node.new("Perlin")
    fbm.set("Source", child)
    del child                                  # parent still holds the Perlin node
    assert fbm.encode() == T.encode(T.N("FractalFBm", Source=T.N("Perlin")))
