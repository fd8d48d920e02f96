"""Node-tree model for the CPU oracle (TEST INFRASTRUCTURE, never shipped).

This module is part of the parity oracle.  Only tests, ``__graft_entry__.smoke()``
and ``bench.py``'s CPU-baseline leg may import it.  It restates, in plain Python,
the parts of FastNoise2 that describe *which* tree is evaluated:

* the node registry (ids are registration order, ``src/FastNoise/FastSIMD_Build.inl:86-143``)
  and each node's member lists in metadata order (base class first, because the
  ``MetadataT<>`` constructors chain; ``include/FastNoise/Generators/*.h``);
* the encoded node-tree format: ``Metadata::SerialiseNodeData`` /
  ``DeserialiseSmartNodeInternal`` (``src/FastNoise/Metadata.cpp:88-308, 355-506``)
  and the ``@``-run-length Base64 (``src/FastNoise/Base64.h:12-192``).

A tree is held as a list of *set operations* in the order the reference would call
the member setters (variables carry raw 32-bit ``ValueUnion`` bits), so that
stateful setters (``VariableRange::SetOutputMin``/``SetOutputMax``,
``Terrace::SetSmoothness``...) replay exactly on both the oracle and the product.

Parity of the value oracle is UNPINNED: the reference ships no golden values and
its arithmetic layer (FastSIMD @ 16450dae9528727e500e7254f635a671f9c7ee2d) is not
vendored.  The only reference fixtures for this path are the two demo trees
(``tools/NodeEditor/util/DemoNodeTrees.inl:5-6``), which must decode.
"""
from __future__ import annotations

import struct
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence, Tuple, Union

# ---------------------------------------------------------------------------
# Metadata table
# ---------------------------------------------------------------------------

F, I, E = 0, 1, 2          # MemberVariable::eType (include/FastNoise/Metadata.h:68-73)

DIST_FUNC = ("Euclidean", "Euclidean Squared", "Manhattan", "Hybrid", "Max Axis", "Minkowski")
BOOLEAN = ("False", "True")
DIMS = ("X", "Y", "Z", "W")
RETURN_TYPE = ("Index0", "Index0Add1", "Index0Sub1", "Index0Mul1", "Index0Div1")
INTERP = ("Linear", "Hermite", "Quintic")
VEC_SCHEME = ("Orthogonal Gradient Matrix", "Gradient Outer Product")
PLANE_ROT = ("Improve XY Planes", "Improve XZ Planes")


def f2i(v: float) -> int:
    """float -> raw int32 bits (ValueUnion)."""
    return struct.unpack("<i", struct.pack("<f", float(v)))[0]


def i2f(v: int) -> float:
    return struct.unpack("<f", struct.pack("<i", int(v)))[0]


@dataclass(frozen=True)
class Var:
    name: str
    type: int
    default: int            # raw ValueUnion bits
    vmin: int = 0
    vmax: int = 0
    enums: Tuple[str, ...] = ()
    dim: int = -1


@dataclass(frozen=True)
class Hyb:
    name: str
    default: float
    dim: int = -1


@dataclass(frozen=True)
class Look:
    name: str
    dim: int = -1
    warp_only: bool = False     # GeneratorSourceT<DomainWarp> (Fractal<DomainWarp>, DomainWarpFractal.h:67-93)


@dataclass(frozen=True)
class Meta:
    id: int
    name: str
    groups: Tuple[str, ...]
    variables: Tuple[Var, ...]
    lookups: Tuple[Look, ...]
    hybrids: Tuple[Hyb, ...]
    # class-initialised member values that differ from the metadata default
    # (DistanceToPoint::mDistanceFunction, BasicGenerators.h:289 vs :305)
    initial: Tuple[Tuple[int, int], ...] = ()


def vf(name, d, lo=0.0, hi=0.0, dim=-1):
    return Var(name, F, f2i(d), f2i(lo), f2i(hi), (), dim)


def vi(name, d, lo=0, hi=0):
    return Var(name, I, int(d), int(lo), int(hi))


def ve(name, d, names):
    return Var(name, E, int(d), 0, 0, tuple(names))


def per_dim_f(name, d):
    return tuple(vf(name, d, dim=k) for k in range(4))


def per_dim_h(name, d):
    return tuple(Hyb(name, d, k) for k in range(4))


# Member chains (BasicGenerators.h:37, 73, 121-122)
_SCALE = (vf("Feature Scale", 100.0),)
_SEED = (vi("Seed Offset", 0),)
_RANGE = (vf("Output Min", -1.0), vf("Output Max", 1.0))
_NOISE = _SCALE + _SEED + _RANGE
_CELL_H = (Hyb("Minkowski P", 1.5), Hyb("Grid Jitter", 1.0), Hyb("Size Jitter", 0.0))  # Cellular.h:40-53
_DF_CELL = ve("Distance Function", 1, DIST_FUNC)                                        # Cellular.h:36-38
_FRACT_H = (Hyb("Gain", 0.5), Hyb("Weighted Strength", 0.0))                             # Fractal.h:38-48
_FRACT_V = (vi("Octaves", 3, 2, 16), vf("Lacunarity", 2.0))                              # Fractal.h:50-60
_WARP_V = _SCALE + _SEED + per_dim_f("Amplitude Scaling", 1.0)                           # DomainWarp.h:28-35
_WARP_H = (Hyb("Warp Amplitude", 50.0),)

_L = Look
_TABLE = [
    ("Constant", ("Basic Generators",), (vf("Value", 1.0),), (), ()),
    ("White", ("Basic Generators",), _SEED + _RANGE, (), ()),
    ("Checkerboard", ("Basic Generators",), _SCALE + _RANGE, (), ()),
    ("SineWave", ("Basic Generators",), _SCALE + _RANGE, (), ()),
    ("Gradient", ("Basic Generators",), per_dim_f("Multiplier", 0.0), (), per_dim_h("Offset", 0.0)),
    ("DistanceToPoint", ("Basic Generators",), (ve("Distance Function", 0, DIST_FUNC),), (),
     per_dim_h("Point", 0.0) + (Hyb("Minkowski P", 1.5),)),
    ("Simplex", ("Coherent Noise",), _NOISE, (), ()),
    ("SuperSimplex", ("Coherent Noise",), _NOISE, (), ()),
    ("Perlin", ("Coherent Noise",), _NOISE, (), ()),
    ("Value", ("Coherent Noise",), _NOISE, (), ()),
    ("CellularValue", ("Coherent Noise",), _NOISE + (_DF_CELL, vi("Value Index", 0, 0, 3)), (), _CELL_H),
    ("CellularDistance", ("Coherent Noise",),
     _NOISE + (_DF_CELL, vi("Distance Index 0", 0, 0, 3), vi("Distance Index 1", 1, 0, 3),
               ve("Return Type", 0, RETURN_TYPE)), (), _CELL_H),
    ("CellularLookup", ("Coherent Noise",), _SCALE + _SEED + (_DF_CELL,), (_L("Lookup"),), _CELL_H),
    ("FractalFBm", ("Fractal",), _FRACT_V, (_L("Source"),), _FRACT_H),
    ("PingPong", ("Modifiers",), (), (_L("Source"),), (Hyb("Ping Pong Strength", 2.0),)),
    ("FractalRidged", ("Fractal",), _FRACT_V, (_L("Source"),), _FRACT_H),
    ("DomainWarpSimplex", ("Domain Warp",), _WARP_V + (ve("Vectorization Scheme", 0, VEC_SCHEME),),
     (_L("Source"),), _WARP_H),
    ("DomainWarpSuperSimplex", ("Domain Warp",), _WARP_V + (ve("Vectorization Scheme", 0, VEC_SCHEME),),
     (_L("Source"),), _WARP_H),
    ("DomainWarpGradient", ("Domain Warp",), _WARP_V, (_L("Source"),), _WARP_H),
    ("DomainWarpFractalProgressive", ("Domain Warp", "Fractal"), _FRACT_V, (_L("Domain Warp Source", -1, True),), _FRACT_H),
    ("DomainWarpFractalIndependent", ("Domain Warp", "Fractal"), _FRACT_V, (_L("Domain Warp Source", -1, True),), _FRACT_H),
    ("Add", ("Operators",), (), (_L("LHS"),), (Hyb("RHS", 0.0),)),
    ("Subtract", ("Operators",), (), (), (Hyb("LHS", 0.0), Hyb("RHS", 0.0))),
    ("Multiply", ("Operators",), (), (_L("LHS"),), (Hyb("RHS", 0.0),)),
    ("Divide", ("Operators",), (), (), (Hyb("LHS", 0.0), Hyb("RHS", 0.0))),
    ("Abs", ("Modifiers",), (), (_L("Source"),), ()),
    ("Min", ("Blends",), (), (_L("LHS"),), (Hyb("RHS", 0.0),)),
    ("Max", ("Blends",), (), (_L("LHS"),), (Hyb("RHS", 0.0),)),
    ("MinSmooth", ("Blends",), (), (_L("LHS"),), (Hyb("RHS", 0.0), Hyb("Smoothness", 0.1))),
    ("MaxSmooth", ("Blends",), (), (_L("LHS"),), (Hyb("RHS", 0.0), Hyb("Smoothness", 0.1))),
    ("SignedSquareRoot", ("Modifiers",), (), (_L("Source"),), ()),
    ("PowFloat", ("Blends",), (), (), (Hyb("Value", 2.0), Hyb("Pow", 2.0))),
    ("PowInt", ("Blends",), (vi("Pow", 2, 2, 0),), (_L("Value"),), ()),
    ("DomainScale", ("Domain Modifiers",), (vf("Scaling", 1.0),), (_L("Source"),), ()),
    ("DomainOffset", ("Domain Modifiers",), (), (_L("Source"),), per_dim_h("Offset", 0.0)),
    ("DomainRotate", ("Domain Modifiers",), (vf("Yaw", 0.0), vf("Pitch", 0.0), vf("Roll", 0.0)), (_L("Source"),), ()),
    ("DomainAxisScale", ("Domain Modifiers",), per_dim_f("Scaling", 1.0), (_L("Source"),), ()),
    ("SeedOffset", ("Modifiers",), (vi("Seed Offset", 1),), (_L("Source"),), ()),
    ("ConvertRGBA8", ("Modifiers",), (vf("Min", -1.0), vf("Max", 1.0)), (_L("Source"),), ()),
    ("GeneratorCache", ("Modifiers",), (), (_L("Source"),), ()),
    ("Fade", ("Blends",), (ve("Interpolation", 0, INTERP),), (_L("A"), _L("B")),
     (Hyb("Fade", 0.0), Hyb("Fade Min", -1.0), Hyb("Fade Max", 1.0))),
    ("Remap", ("Modifiers",), (ve("Clamp Output", 0, BOOLEAN),), (_L("Source"),),
     (Hyb("From Min", -1.0), Hyb("From Max", 1.0), Hyb("To Min", 0.0), Hyb("To Max", 1.0))),
    ("Terrace", ("Modifiers",), (vf("Step Count", 1.0),), (_L("Source"),), (Hyb("Smoothness", 0.0),)),
    ("AddDimension", ("Domain Modifiers",), (), (_L("Source"),), (Hyb("New Dimension Position", 0.0),)),
    ("RemoveDimension", ("Domain Modifiers",), (ve("Remove Dimension", 1, DIMS),), (_L("Source"),), ()),
    ("Modulus", ("Operators",), (), (), (Hyb("LHS", 0.0), Hyb("RHS", 0.0))),
    ("DomainRotatePlane", ("Domain Modifiers",), (ve("Rotation Type", 0, PLANE_ROT),), (_L("Source"),), ()),
]

META: List[Meta] = []
for _i, (_n, _g, _v, _l, _h) in enumerate(_TABLE):
    _init = ((0, 1),) if _n == "DistanceToPoint" else ()
    META.append(Meta(_i, _n, _g, tuple(_v), tuple(_l), tuple(_h), _init))
META_BY_NAME: Dict[str, Meta] = {m.name: m for m in META}
WARP_NODES = ("DomainWarpSimplex", "DomainWarpSuperSimplex", "DomainWarpGradient")
assert len(META) == 47

# ---------------------------------------------------------------------------
# Tree model
# ---------------------------------------------------------------------------

SetOp = Tuple[str, int, object]   # ("var", idx, bits) | ("lookup", idx, Node) | ("hnode", idx, Node) | ("hfloat", idx, float)


class Node:
    """One generator node: metadata + ordered setter calls (+ NodeData-style state)."""

    def __init__(self, name: str):
        self.meta = META_BY_NAME[name]
        self.ops: List[SetOp] = []
        m = self.meta
        # NodeData view (Metadata.h:201-233): starts from metadata defaults
        self.variables = [v.default for v in m.variables]
        self.lookups: List[Optional[Node]] = [None] * len(m.lookups)
        self.hybrids: List[Tuple[Optional[Node], float]] = [(None, h.default) for h in m.hybrids]

    # -- member resolution -------------------------------------------------
    def _index(self, seq, name: str, dim: Optional[int]) -> int:
        for k, mem in enumerate(seq):
            if mem.name == name and (dim is None or mem.dim == dim or mem.dim == -1):
                if dim is not None and mem.dim == -1 and dim != -1:
                    continue
                return k
        raise KeyError(f"{self.meta.name} has no member {name!r} dim={dim}")

    def set_var(self, name: str, value, dim: Optional[int] = None) -> "Node":
        k = self._index(self.meta.variables, name, dim)
        var = self.meta.variables[k]
        if isinstance(value, str):
            value = var.enums.index(value)
        bits = f2i(value) if var.type == F else int(value)
        return self.set_var_bits(k, bits)

    def set_var_bits(self, k: int, bits: int) -> "Node":
        bits = ((int(bits) + 2**31) % 2**32) - 2**31
        self.ops.append(("var", k, bits))
        self.variables[k] = bits
        return self

    def accepts_lookup(self, k: int, node: "Node") -> bool:
        return not self.meta.lookups[k].warp_only or node.meta.name in WARP_NODES

    def set_lookup(self, name: str, node: "Node", dim: Optional[int] = None) -> "Node":
        k = self._index(self.meta.lookups, name, dim)
        if not self.accepts_lookup(k, node):
            raise TypeError(f"{self.meta.name}.{name} needs a domain-warp node, got {node.meta.name}")
        self.ops.append(("lookup", k, node))
        self.lookups[k] = node
        return self

    def set_hybrid(self, name: str, value: Union[float, "Node"], dim: Optional[int] = None) -> "Node":
        k = self._index(self.meta.hybrids, name, dim)
        if isinstance(value, Node):
            self.ops.append(("hnode", k, value))
            self.hybrids[k] = (value, self.hybrids[k][1])
        else:
            self.ops.append(("hfloat", k, float(value)))
            self.hybrids[k] = (None, float(value))
        return self

    def set(self, name: str, value, dim: Optional[int] = None) -> "Node":
        """Set any member by name: variable, node lookup or hybrid."""
        m = self.meta
        if any(v.name == name for v in m.variables):
            return self.set_var(name, value, dim)
        if any(l.name == name for l in m.lookups):
            return self.set_lookup(name, value, dim)
        return self.set_hybrid(name, value, dim)

    # -- traversal ---------------------------------------------------------
    def children(self) -> List["Node"]:
        out = [n for n in self.lookups if n is not None]
        out += [h[0] for h in self.hybrids if h[0] is not None]
        return out

    def __repr__(self):
        return f"Node({self.meta.name})"


def N(name: str, **members) -> Node:
    """Convenience constructor: ``N("Simplex", **{"Feature Scale": 50})`` style is
    awkward, so member names use underscores: ``N("FractalFBm", Source=..., Octaves=5)``."""
    node = Node(name)
    for key, val in members.items():
        node.set(key.replace("_", " "), val)
    return node


# ---------------------------------------------------------------------------
# Base64 with '@' run-length compression of 'A'  (src/FastNoise/Base64.h)
# ---------------------------------------------------------------------------

_ENC = "ABCDEFGHIJKLMNOPQRSTUVWXYZabcdefghijklmnopqrstuvwxyz0123456789+/"
_DEC = {c: i for i, c in enumerate(_ENC)}
_DEC["="] = 0


def b64_encode(data: bytes) -> str:
    """Standard Base64, then every run of >=3 'A' becomes '@' + table[run-3]
    (runs longer than 66 are split); Base64.h:12-92."""
    plain = []
    n = len(data)
    i = 0
    while i + 2 < n:
        b0, b1, b2 = data[i], data[i + 1], data[i + 2]
        plain += [_ENC[b0 >> 2], _ENC[((b0 & 3) << 4) | (b1 >> 4)], _ENC[((b1 & 15) << 2) | (b2 >> 6)], _ENC[b2 & 63]]
        i += 3
    if i < n:
        b0 = data[i]
        plain.append(_ENC[b0 >> 2])
        if i == n - 1:
            plain += [_ENC[(b0 & 3) << 4], "="]
        else:
            b1 = data[i + 1]
            plain += [_ENC[((b0 & 3) << 4) | (b1 >> 4)], _ENC[(b1 & 15) << 2]]
        plain.append("=")
    out: List[str] = []
    run = 0

    def flush():
        nonlocal run
        if run >= 3:
            out.append("@" + _ENC[run - 3])
        else:
            out.extend("A" * run)
        run = 0

    for c in plain:
        if c == "A":
            run += 1
            if run == len(_ENC) + 2:        # 66 'A's fill one '@' + table[63] token
                out.append("@" + _ENC[run - 3])
                run = 0
        else:
            flush()
            out.append(c)
    flush()
    return "".join(out)


def b64_decode(text: str) -> bytes:
    """Inverse of :func:`b64_encode`; returns b"" on malformed input (Base64.h:94-192)."""
    expanded = []
    i = 0
    while i < len(text):
        c = text[i]
        if c == "@":
            if i + 1 >= len(text) or text[i + 1] not in _DEC:
                return b""
            expanded.append("A" * (_DEC[text[i + 1]] + 3))
            i += 2
        else:
            expanded.append(c)
            i += 1
    s = "".join(expanded)
    if len(s) == 0 or len(s) % 4 != 0:
        return b""
    out_len = len(s) // 4 * 3
    if text.endswith("="):
        out_len -= 1
        if text.endswith("=="):
            out_len -= 1
    out = bytearray()
    for k in range(0, len(s), 4):
        vals = [_DEC.get(ch, 64) & 0xFF for ch in s[k:k + 4]]
        triple = ((vals[0] << 18) + (vals[1] << 12) + (vals[2] << 6) + vals[3]) & 0xFFFFFFFF
        out += bytes([(triple >> 16) & 0xFF, (triple >> 8) & 0xFF, triple & 0xFF])
    return bytes(out[:out_len])


# ---------------------------------------------------------------------------
# Encoded node tree  (src/FastNoise/Metadata.cpp:88-308 and 355-506)
# ---------------------------------------------------------------------------

T_VAR, T_LOOKUP, T_HLOOKUP, T_HVAR, T_END = 0, 1, 2, 3, 4


def _member_byte(t: int, index: int) -> int:
    return (t & 7) | ((index & 31) << 3)


def encode(root: Node) -> str:
    """Serialise a tree the way ``Metadata::SerialiseNodeData`` does: only
    non-default variables are written, shared nodes become 0xFF back-references,
    consecutive node ends are run-length coded."""
    stream = bytearray()
    ref_ids: Dict[int, int] = {}
    end_stack = [0]

    def check_end():
        if end_stack[0] > 0:
            stream.append(_member_byte(T_END, end_stack[0] - 1))
            end_stack[0] = 0

    def put(data: bytes):
        check_end()
        stream.extend(data)

    def node_end():
        end_stack[0] += 1
        if end_stack[0] >= 32:
            check_end()

    def ser(node: Node):
        if id(node) in ref_ids:
            put(bytes([0xFF]))
            put(struct.pack("<H", ref_ids[id(node)]))
            return
        m = node.meta
        put(bytes([m.id]))
        for k, var in enumerate(m.variables):
            if node.variables[k] != var.default:
                put(bytes([_member_byte(T_VAR, k)]))
                put(struct.pack("<i", node.variables[k]))
        if m.lookups:
            put(bytes([_member_byte(T_LOOKUP, len(m.lookups))]))
        for k in range(len(m.lookups)):
            child = node.lookups[k]
            if child is None:
                raise ValueError(f"{m.name}: lookup {m.lookups[k].name} not set")
            ser(child)
        for k, hyb in enumerate(m.hybrids):
            hn, hv = node.hybrids[k]
            if hn is None:
                if f2i(hv) != f2i(hyb.default):
                    put(bytes([_member_byte(T_HVAR, k)]))
                    put(struct.pack("<f", hv))
            else:
                put(bytes([_member_byte(T_HLOOKUP, k)]))
                ser(hn)
        node_end()
        ref_ids[id(node)] = len(ref_ids)

    ser(root)
    check_end()
    return b64_encode(bytes(stream))


class _Stream:
    def __init__(self, data: bytes):
        self.data = data
        self.pos = 0
        self.end_stack = 0

    def read(self, fmt: str):
        if self.end_stack > 0:
            return None
        size = struct.calcsize(fmt)
        if self.pos + size > len(self.data):
            return None
        val = struct.unpack_from(fmt, self.data, self.pos)[0]
        self.pos += size
        return val

    def read_member(self):
        if self.end_stack > 0:
            self.end_stack -= 1
            return (T_END, 0)
        if self.pos + 1 > len(self.data):
            return None
        b = self.data[self.pos]
        self.pos += 1
        t, idx = b & 7, b >> 3
        if t == T_END:
            self.end_stack = idx
        return (t, idx)


def decode(text: str) -> Optional[Node]:
    """Rebuild the tree with setter calls in stream order, following
    ``DeserialiseSmartNodeInternal``.  Returns None where the reference returns nullptr."""
    st = _Stream(b64_decode(text))
    refs: List[Node] = []

    def des() -> Optional[Node]:
        nid = st.read("<B")
        if nid is None:
            return None
        if nid == 0xFF:
            rid = st.read("<H")
            if rid is None or rid >= len(refs):
                return None
            return refs[rid]
        if nid >= len(META):
            return None
        m = META[nid]
        node = Node(m.name)
        mem = st.read_member()
        if mem is None:
            return None
        while mem[0] == T_VAR:
            v = st.read("<i")
            if v is None:
                return None
            if mem[1] < len(m.variables):
                node.set_var_bits(mem[1], v)
            mem = st.read_member()
            if mem is None:
                return None
        if mem[0] == T_LOOKUP:
            count = mem[1]
            k = 0
            while k < min(count, len(m.lookups)):
                child = des()
                if child is None or not node.accepts_lookup(k, child):
                    return None
                node.set_lookup(m.lookups[k].name, child, m.lookups[k].dim)
                k += 1
            while k < count:
                if des() is None:
                    return None
                k += 1
            while k < len(m.lookups):
                filler = Node("Constant")
                if not node.accepts_lookup(k, filler):
                    return None
                node.set_lookup(m.lookups[k].name, filler, m.lookups[k].dim)
                k += 1
            mem = st.read_member()
            if mem is None:
                return None
        while mem[0] != T_END:
            if mem[0] == T_HLOOKUP:
                child = des()
                if mem[1] < len(m.hybrids):
                    if child is None:
                        return None
                    node.ops.append(("hnode", mem[1], child))
                    node.hybrids[mem[1]] = (child, node.hybrids[mem[1]][1])
            elif mem[0] == T_HVAR:
                v = st.read("<f")
                if v is None:
                    return None
                if mem[1] < len(m.hybrids):
                    node.ops.append(("hfloat", mem[1], v))
                    node.hybrids[mem[1]] = (None, v)
            mem = st.read_member()
            if mem is None:
                return None
        refs.append(node)
        return node

    return des()


def walk(root: Node) -> List[Node]:
    """Unique nodes in post-order (children before parents)."""
    seen: Dict[int, Node] = {}
    order: List[Node] = []

    def rec(n: Node):
        if id(n) in seen:
            return
        seen[id(n)] = n
        for _, _, arg in n.ops:
            if isinstance(arg, Node):
                rec(arg)
        order.append(n)

    rec(root)
    return order
