"""ctypes front-end to the C oracle (TEST INFRASTRUCTURE, never shipped).

Builds ``oracle/fn_oracle.c`` into ``oracle/_build/libfn_oracle.so`` with the
recipe in :func:`build` (gcc ``-O3`` tuned for the host CPU, ``-ffp-contract=off``
so that only the explicit ``fmaf`` calls fuse), instantiates a :class:`oracle.tree.Node` tree by
replaying its setter calls in order, and exposes the reference's batch drivers
(``Generator.inl`` GenUniformGrid2D/3D/4D, GenPositionArray2D/3D/4D,
GenTileable2D, GenSingle*), each returning ``(values, (min, max))``.

Parity is unpinned: see the header of ``fn_oracle.c``.
"""
from __future__ import annotations

import ctypes
import os
import platform
import subprocess
from typing import Dict, Optional, Sequence, Tuple

import numpy as np

from .tree import Node, walk

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libfn_oracle.so")
SRC = os.path.join(HERE, "fn_oracle.c")

LIB_COUNT = os.path.join(BUILD, "libfn_oracle_count.so")
OPCOUNT_H = os.path.join(HERE, "opcount.h")

_lib = None
_lib_count = None


def build(force: bool = False) -> str:
    """Compile the oracle shared library (a few seconds)."""
    os.makedirs(BUILD, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    flags = ["-O3", "-std=c11", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-fvisibility=hidden"]
    flags += native_cpu_flags()          # hardware fmaf and the host's vector units; IEEE results unchanged
    tmp = LIB + f".tmp{os.getpid()}"
    subprocess.run(["gcc", *flags, "-o", tmp, SRC, "-lm", "-lpthread"], check=True)
    os.replace(tmp, LIB)
    return LIB


def native_cpu_flags():
    """Code generation for the CPU this runs on: ``-march=native`` on x86-64,
    ``-mcpu=native`` on AArch64 (GCC's spelling for each)."""
    m = platform.machine()
    if m in ("x86_64", "AMD64"):
        return ["-march=native"]
    if m in ("aarch64", "arm64"):
        return ["-mcpu=native"]
    return []


def cpu_description() -> dict:
    """Host CPU facts recorded beside every CPU timing: architecture, model name, threads."""
    model = ""
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                key = line.split(":", 1)[0].strip().lower()
                if key in ("model name", "cpu model", "hardware") and ":" in line:
                    model = line.split(":", 1)[1].strip()
                    break
    except OSError:
        pass
    if not model:
        try:                             # util-linux names Arm cores from their part numbers
            out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
            for line in out.splitlines():
                if line.lower().startswith("model name:"):
                    model = line.split(":", 1)[1].strip()
                    break
        except (OSError, subprocess.SubprocessError):
            pass
    if not model and platform.machine() in ("aarch64", "arm64"):
        # Arm kernels list implementer / part numbers instead of a name
        try:
            parts = {}
            with open("/proc/cpuinfo") as f:
                for line in f:
                    if ":" in line:
                        k, v = line.split(":", 1)
                        parts.setdefault(k.strip(), v.strip())
            model = f"implementer {parts.get('CPU implementer', '?')} part {parts.get('CPU part', '?')}"
        except OSError:
            pass
    return {"uname_m": platform.machine(), "cpu_model": model, "nproc": os.cpu_count(),
            "compiler_flags": " ".join(["-O3", "-ffp-contract=off", *native_cpu_flags()])}


def build_count(force: bool = False) -> str:
    """Compile the oracle as C++ with the counting scalar type (opcount.h)."""
    os.makedirs(BUILD, exist_ok=True)
    newest = max(os.path.getmtime(SRC), os.path.getmtime(OPCOUNT_H))
    if not force and os.path.exists(LIB_COUNT) and os.path.getmtime(LIB_COUNT) >= newest:
        return LIB_COUNT
    tmp = LIB_COUNT + f".tmp{os.getpid()}"
    subprocess.run(["g++", "-x", "c++", "-std=c++17", "-O2", "-DOC_COUNT", f"-I{HERE}", "-ffp-contract=off",
                    "-fPIC", "-shared", "-fvisibility=hidden", "-o", tmp, SRC, "-lm", "-lpthread"], check=True)
    os.replace(tmp, LIB_COUNT)
    return LIB_COUNT


def count_ops(root: Node, points: np.ndarray, seed: int) -> float:
    """Mean FS-level operations per point of `root` over the rows of `points` (n x dim)."""
    global _lib_count
    if _lib_count is None:
        build_count()
        L = ctypes.CDLL(LIB_COUNT)
        L.on_new.restype = ctypes.c_void_p
        L.on_new.argtypes = [ctypes.c_int]
        L.on_set_var.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int32]
        L.on_set_lookup.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        L.on_set_hybrid_node.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        L.on_set_hybrid_float.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_float]
        L.on_free.argtypes = [ctypes.c_void_p]
        L.on_count_ops.restype = ctypes.c_double
        L.on_count_ops.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_float), ctypes.c_int]
        _lib_count = L
    L = _lib_count
    handles = {}
    for node in walk(root):
        h = L.on_new(node.meta.id)
        handles[id(node)] = h
        for kind, idx, arg in node.ops:
            if kind == "var":
                L.on_set_var(h, idx, int(arg))
            elif kind == "lookup":
                L.on_set_lookup(h, idx, handles[id(arg)])
            elif kind == "hnode":
                L.on_set_hybrid_node(h, idx, handles[id(arg)])
            else:
                L.on_set_hybrid_float(h, idx, float(arg))
    pts = np.ascontiguousarray(points, np.float32)
    total = 0.0
    for row in pts:
        p = np.zeros(4, np.float32)
        p[:len(row)] = row
        total += L.on_count_ops(handles[id(root)], len(row), _fptr(p), int(np.int32(seed)))
    for h in handles.values():
        L.on_free(h)
    return total / max(len(pts), 1)


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        vp, fp, ip, c_int, c_float = ctypes.c_void_p, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_int), ctypes.c_int, ctypes.c_float
        L.on_new.restype = vp
        L.on_new.argtypes = [c_int]
        L.on_free.argtypes = [vp]
        L.on_set_var.argtypes = [vp, c_int, ctypes.c_int32]
        L.on_set_lookup.argtypes = [vp, c_int, vp]
        L.on_set_hybrid_node.argtypes = [vp, c_int, vp]
        L.on_set_hybrid_float.argtypes = [vp, c_int, c_float]
        L.on_set_unfused.argtypes = [c_int]
        L.on_gen_grid.argtypes = [vp, c_int, fp, fp, ip, fp, c_int, c_int, fp]
        L.on_gen_positions.argtypes = [vp, c_int, fp, ctypes.c_int64, ctypes.POINTER(fp), fp, c_int, c_int, fp]
        L.on_gen_tileable.argtypes = [vp, fp, c_int, c_int, c_float, c_float, c_int, c_int, fp]
        L.on_gen_single.restype = c_float
        L.on_gen_single.argtypes = [vp, c_int, fp, c_int]
        L.on_gen_requests.restype = c_int
        L.on_gen_requests.argtypes = [ctypes.c_void_p, c_int, c_int, ctypes.c_int64]
        L.on_serve_paced.restype = c_int
        L.on_serve_paced.argtypes = [ctypes.c_void_p, c_int, ctypes.c_void_p, c_int, ctypes.c_void_p]
        L.fn_sinf.restype = c_float
        L.fn_sinf.argtypes = [c_float]
        L.fn_cosf.restype = c_float
        L.fn_cosf.argtypes = [c_float]
        L.fn_powf.restype = c_float
        L.fn_powf.argtypes = [c_float, c_float]
        _lib = L
    return _lib


def _fptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


class OracleTree:
    """A tree instantiated inside the C oracle."""

    def __init__(self, root: Node, unfused: bool = False):
        L = lib()
        self.unfused = unfused
        self._handles: Dict[int, int] = {}
        for node in walk(root):
            h = L.on_new(node.meta.id)
            self._handles[id(node)] = h
            for kind, idx, arg in node.ops:
                if kind == "var":
                    L.on_set_var(h, idx, int(arg))
                elif kind == "lookup":
                    L.on_set_lookup(h, idx, self._handles[id(arg)])
                elif kind == "hnode":
                    L.on_set_hybrid_node(h, idx, self._handles[id(arg)])
                elif kind == "hfloat":
                    L.on_set_hybrid_float(h, idx, float(arg))
        self.root = self._handles[id(root)]

    def __del__(self):
        if _lib is not None:
            for h in self._handles.values():
                _lib.on_free(h)

    def _mode(self):
        lib().on_set_unfused(1 if self.unfused else 0)

    def grid(self, offset: Sequence[float], count: Sequence[int], step: Sequence[float], seed: int,
             threads: int = 0) -> Tuple[np.ndarray, Tuple[float, float]]:
        """GenUniformGrid{2,3,4}D: out[(..*Y + y)*X + x], x fastest."""
        dim = len(count)
        total = int(np.prod([max(c, 0) for c in count]))
        out = np.empty(max(total, 1), np.float32)
        off = np.asarray(offset, np.float32)
        cnt = np.asarray(count, np.int32)
        st = np.asarray(step, np.float32)
        mm = np.zeros(2, np.float32)
        self._mode()
        lib().on_gen_grid(self.root, dim, _fptr(out), _fptr(off), cnt.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                          _fptr(st), int(np.int32(seed)), threads or os.cpu_count(), _fptr(mm))
        return out[:total], (float(mm[0]), float(mm[1]))

    def positions(self, pos: Sequence[np.ndarray], offset: Sequence[float], seed: int,
                  threads: int = 0) -> Tuple[np.ndarray, Tuple[float, float]]:
        """GenPositionArray{2,3,4}D."""
        dim = len(pos)
        arrs = [np.ascontiguousarray(p, np.float32) for p in pos]
        count = len(arrs[0])
        out = np.empty(max(count, 1), np.float32)
        ptrs = (ctypes.POINTER(ctypes.c_float) * 4)(*[_fptr(a) for a in arrs], *([None] * (4 - dim)))
        off = np.asarray(offset, np.float32)
        mm = np.zeros(2, np.float32)
        self._mode()
        lib().on_gen_positions(self.root, dim, _fptr(out), count, ptrs, _fptr(off), int(np.int32(seed)),
                               threads or os.cpu_count(), _fptr(mm))
        return out[:count], (float(mm[0]), float(mm[1]))

    def tileable(self, x_size: int, y_size: int, x_step: float, y_step: float, seed: int,
                 threads: int = 0) -> Tuple[np.ndarray, Tuple[float, float]]:
        """GenTileable2D."""
        total = max(x_size, 0) * max(y_size, 0)
        out = np.empty(max(total, 1), np.float32)
        mm = np.zeros(2, np.float32)
        self._mode()
        lib().on_gen_tileable(self.root, _fptr(out), x_size, y_size, x_step, y_step, int(np.int32(seed)),
                              threads or os.cpu_count(), _fptr(mm))
        return out[:total], (float(mm[0]), float(mm[1]))

    def single(self, pos: Sequence[float], seed: int) -> float:
        """GenSingle{2,3,4}D."""
        p = np.zeros(4, np.float32)
        p[:len(pos)] = pos
        self._mode()
        return float(lib().on_gen_single(self.root, len(pos), _fptr(p), int(np.int32(seed))))


class OracleRequest(ctypes.Structure):
    """One request of :func:`gen_requests` (the fields of the product's fnGenRequest)."""
    _fields_ = [("root", ctypes.c_void_p), ("kind", ctypes.c_int), ("seed", ctypes.c_int),
                ("count", ctypes.c_int * 4), ("offset", ctypes.c_float * 4), ("step", ctypes.c_float * 4),
                ("positions", ctypes.POINTER(ctypes.c_float) * 4), ("out", ctypes.POINTER(ctypes.c_float)),
                ("minmax", ctypes.POINTER(ctypes.c_float))]


KIND_GRID2D, KIND_GRID3D, KIND_GRID4D, KIND_TILEABLE2D, KIND_POSITIONS2D, KIND_POSITIONS3D, KIND_POSITIONS4D = range(7)


def request(tree: "OracleTree", kind: int, out: np.ndarray, minmax: np.ndarray, seed: int, count=(0, 0, 0, 0),
            offset=(0, 0, 0, 0), step=(1, 1, 1, 1), positions=()) -> OracleRequest:
    """Fill one OracleRequest; `out` (float32) and `minmax` (float32[2]) must stay alive until the call."""
    r = OracleRequest()
    r.root = tree.root
    r.kind = kind
    r.seed = int(np.int32(seed))
    for k in range(4):
        r.count[k] = int(count[k]) if k < len(count) else 0
        r.offset[k] = float(offset[k]) if k < len(offset) else 0.0
        r.step[k] = float(step[k]) if k < len(step) else 1.0
        r.positions[k] = _fptr(positions[k]) if k < len(positions) else None
    r.out = _fptr(out)
    r.minmax = _fptr(minmax)
    return r


def gen_requests(reqs: Sequence[OracleRequest], threads: int = 0, split: int = 0, unfused: bool = False) -> None:
    """Evaluate a batch of requests on the oracle's persistent worker pool: whole requests go
    to threads, largest first (requests above `split` points, when split > 0, are cut into
    ranges of that size).  Fills every request's out and minmax."""
    arr = (OracleRequest * len(reqs))(*reqs)
    lib().on_set_unfused(1 if unfused else 0)
    if lib().on_gen_requests(ctypes.cast(arr, ctypes.c_void_p), len(reqs), threads or os.cpu_count(), int(split)) != 0:
        raise MemoryError("oracle batch: allocation failed")


def serve_paced(reqs: Sequence[OracleRequest], arrivals_us, threads: int = 0) -> np.ndarray:
    """Open-loop serving on the host cores: request k arrives arrivals_us[k] microseconds after
    the start; `threads` workers serve the requests in arrival order.  Returns each request's
    latency (completion minus arrival, microseconds)."""
    arr = (OracleRequest * len(reqs))(*reqs)
    times = np.ascontiguousarray(arrivals_us, np.float64)
    lat = np.zeros(len(reqs), np.float64)
    lib().on_set_unfused(0)
    lib().on_serve_paced(ctypes.cast(arr, ctypes.c_void_p), len(reqs), times.ctypes.data, threads or os.cpu_count(),
                         lat.ctypes.data)
    return lat


def sinf(x: float) -> float:
    return float(lib().fn_sinf(x))


def cosf(x: float) -> float:
    return float(lib().fn_cosf(x))


def powf(x: float, y: float) -> float:
    return float(lib().fn_powf(x, y))
