"""fastnoise2_gb300 -- GB300 (sm_103a) backend for FastNoise2 node trees.

Python host mirror of FastNoise2's API for the node-tree generation path,
bound to the C-ABI in ``include/FastNoise/FastNoise_C.h`` (the same entry
points as the reference's ``FastNoise_C.h`` plus device-pointer additions).

    import fastnoise2_gb300 as fn
    node = fn.Node.from_encoded("...")            # FastNoise::NewFromEncodedNodeTree
    simplex = fn.Node.new("Simplex")              # FastNoise::New<Simplex>()
    simplex.set("Feature Scale", 50.0)            # SetScale(50)
    out, (mn, mx) = simplex.gen_uniform_grid_3d((0, 0, 0), (64, 64, 64), (1, 1, 1), 1337)

Generation always runs on the GPU.  If the native library is missing the
import fails; if a call cannot run on the GPU, :class:`FastNoiseError` is raised.
"""
from __future__ import annotations

import ctypes
import math
import os
from typing import Optional, Sequence, Tuple, Union

import numpy as np

__all__ = ["Node", "FastNoiseError", "lib", "library_path", "metadata_count", "metadata_name", "node_id"]

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_lib", "libfastnoise_gb300.so")


class FastNoiseError(RuntimeError):
    """A GPU generation call failed (status code and message from the library)."""

    def __init__(self, code: int, message: str):
        super().__init__(f"fastnoise_gb300 error {code}: {message}")
        self.code = code
        self.message = message


def library_path() -> str:
    return _LIB_PATH


_lib = None
_FP = ctypes.POINTER(ctypes.c_float)


def _declare(L):
    c_int, c_float, vp, cp, c_bool, c_uint = ctypes.c_int, ctypes.c_float, ctypes.c_void_p, ctypes.c_char_p, ctypes.c_bool, ctypes.c_uint
    sig = {
        "fnNewFromEncodedNodeTree": (vp, [cp, c_uint]),
        "fnDeleteNodeRef": (None, [vp]),
        "fnGetActiveFeatureSet": (c_uint, [vp]),
        "fnGetMetadataID": (c_int, [vp]),
        "fnGenUniformGrid2D": (None, [vp, vp, c_float, c_float, c_int, c_int, c_float, c_float, c_int, vp]),
        "fnGenUniformGrid3D": (None, [vp, vp, c_float, c_float, c_float, c_int, c_int, c_int, c_float, c_float, c_float, c_int, vp]),
        "fnGenUniformGrid4D": (None, [vp, vp] + [c_float] * 4 + [c_int] * 4 + [c_float] * 4 + [c_int, vp]),
        "fnGenPositionArray2D": (None, [vp, vp, c_int, vp, vp, c_float, c_float, c_int, vp]),
        "fnGenPositionArray3D": (None, [vp, vp, c_int, vp, vp, vp, c_float, c_float, c_float, c_int, vp]),
        "fnGenPositionArray4D": (None, [vp, vp, c_int, vp, vp, vp, vp, c_float, c_float, c_float, c_float, c_int, vp]),
        "fnGenTileable2D": (None, [vp, vp, c_int, c_int, c_float, c_float, c_int, vp]),
        "fnGenSingle2D": (c_float, [vp, c_float, c_float, c_int]),
        "fnGenSingle3D": (c_float, [vp, c_float, c_float, c_float, c_int]),
        "fnGenSingle4D": (c_float, [vp, c_float, c_float, c_float, c_float, c_int]),
        "fnGetMetadataCount": (c_int, []),
        "fnGetMetadataName": (cp, [c_int]),
        "fnNewFromMetadata": (vp, [c_int, c_uint]),
        "fnGetMetadataVariableCount": (c_int, [c_int]),
        "fnGetMetadataVariableName": (cp, [c_int, c_int]),
        "fnGetMetadataVariableType": (c_int, [c_int, c_int]),
        "fnGetMetadataVariableDimensionIdx": (c_int, [c_int, c_int]),
        "fnGetMetadataEnumCount": (c_int, [c_int, c_int]),
        "fnGetMetadataEnumName": (cp, [c_int, c_int, c_int]),
        "fnSetVariableFloat": (c_bool, [vp, c_int, c_float]),
        "fnSetVariableIntEnum": (c_bool, [vp, c_int, c_int]),
        "fnGetMetadataNodeLookupCount": (c_int, [c_int]),
        "fnGetMetadataNodeLookupName": (cp, [c_int, c_int]),
        "fnGetMetadataNodeLookupDimensionIdx": (c_int, [c_int, c_int]),
        "fnSetNodeLookup": (c_bool, [vp, c_int, vp]),
        "fnGetMetadataHybridCount": (c_int, [c_int]),
        "fnGetMetadataHybridName": (cp, [c_int, c_int]),
        "fnGetMetadataHybridDimensionIdx": (c_int, [c_int, c_int]),
        "fnSetHybridNodeLookup": (c_bool, [vp, c_int, vp]),
        "fnSetHybridFloat": (c_bool, [vp, c_int, c_float]),
        "fnGetMetadataDescription": (cp, [c_int]),
        "fnGetMetadataGroupCount": (c_int, [c_int]),
        "fnGetMetadataGroupName": (cp, [c_int, c_int]),
        "fnGetMetadataVariableDescription": (cp, [c_int, c_int]),
        "fnGetMetadataVariableDefaultFloat": (c_float, [c_int, c_int]),
        "fnGetMetadataVariableDefaultIntEnum": (c_int, [c_int, c_int]),
        "fnGetMetadataVariableMinFloat": (c_float, [c_int, c_int]),
        "fnGetMetadataVariableMaxFloat": (c_float, [c_int, c_int]),
        "fnGetMetadataNodeLookupDescription": (cp, [c_int, c_int]),
        "fnGetMetadataHybridDescription": (cp, [c_int, c_int]),
        "fnGetMetadataHybridDefault": (c_float, [c_int, c_int]),
        "fnGetLastError": (c_int, []),
        "fnGetLastErrorString": (cp, []),
        "fnSerialiseNodeTree": (c_int, [vp, ctypes.c_char_p, c_int]),
        "fnPrepare": (c_int, [vp, c_int]),
        "fnCompileInfo": (c_int, [vp, c_int, ctypes.POINTER(c_int), ctypes.POINTER(c_int)]),
        "fnGenUniformGrid2DDevice": (c_int, [vp, vp, c_float, c_float, c_int, c_int, c_float, c_float, c_int, vp, vp]),
        "fnGenUniformGrid3DDevice": (c_int, [vp, vp, c_float, c_float, c_float, c_int, c_int, c_int, c_float, c_float, c_float, c_int, vp, vp]),
        "fnJitCompile": (c_int, [vp, vp, c_int]),
        "fnBuildChunkMeshBloxel": (c_int, [vp, c_int, c_int, c_int, c_int, c_int, c_float, c_int, vp, vp]),
        "fnBuildChunkMeshDmc": (c_int, [vp, c_int, c_int, c_int, c_int, c_int, c_float, c_int, vp, vp]),
        "fnBuildChunkMeshesDmc": (c_int, [vp, c_int, c_int, vp, c_int, c_float, c_int, vp, vp]),
        "fnBuildChunkMeshesBloxel": (c_int, [vp, c_int, c_int, vp, c_int, c_float, c_int, vp, vp]),
        "fnBuildChunkMeshHeightmap": (c_int, [vp, c_int, c_int, c_int, c_int, c_float, vp, vp]),
        "fnGetBatchInfo": (c_int, [vp]),
        "fnJitCheck": (c_int, [vp, vp, c_int, ctypes.POINTER(c_int)]),
        "fnJitSetCacheDir": (c_int, [ctypes.c_char_p]),
        "fnJitGetCacheInfo": (c_int, [ctypes.c_char_p, c_int, ctypes.POINTER(ctypes.c_ulonglong), ctypes.POINTER(ctypes.c_ulonglong)]),
        "fnSetJitEnabled": (c_int, [c_int]),
        "fnSetAutoSpecialise": (c_int, [c_int]),
        "fnAutoSpecialiseWait": (c_int, [c_int]),
        "fnJitIsSpecialised": (c_int, [vp, c_int]),
        "fnGenUniformGrid3DDeviceNoAlloc": (c_int, [vp, vp, c_float, c_float, c_float, c_int, c_int, c_int, c_float, c_float, c_float, c_int, vp, vp]),
        "fnGenUniformGrid4DDevice": (c_int, [vp, vp] + [c_float] * 4 + [c_int] * 4 + [c_float] * 4 + [c_int, vp, vp]),
        "fnGenPositionArray2DDevice": (c_int, [vp, vp, c_int, vp, vp, c_float, c_float, c_int, vp, vp]),
        "fnGenPositionArray3DDevice": (c_int, [vp, vp, c_int, vp, vp, vp, c_float, c_float, c_float, c_int, vp, vp]),
        "fnGenPositionArray4DDevice": (c_int, [vp, vp, c_int, vp, vp, vp, vp, c_float, c_float, c_float, c_float, c_int, vp, vp]),
        "fnGenTileable2DDevice": (c_int, [vp, vp, c_int, c_int, c_float, c_float, c_int, vp, vp]),
        "fnGenBatchDevice": (c_int, [vp, c_int, vp, c_int]),
        "fnAutotuneBatch": (c_int, [vp, c_int, vp]),
        "fnGenEachDevice": (c_int, [vp, c_int, vp, c_int]),
        "fnGenBatchHost": (c_int, [vp, c_int, c_int]),
        "fnServerCreate": (vp, [vp]),
        "fnServerDestroy": (None, [vp]),
        "fnServerSubmit": (c_int, [vp, vp, vp]),
        "fnServerPoll": (c_int, [vp, ctypes.c_ulonglong]),
        "fnServerSubmitMany": (c_int, [vp, vp, c_int, vp]),
        "fnServerWaitMany": (c_int, [vp, vp, c_int, c_int]),
        "fnServerWait": (c_int, [vp, ctypes.c_ulonglong, c_int, _FP, vp]),
        "fnServerCancel": (c_int, [vp, ctypes.c_ulonglong]),
        "fnServerRelease": (c_int, [vp, ctypes.c_ulonglong]),
        "fnServerGetStats": (c_int, [vp, vp]),
        "fnServerResetStats": (c_int, [vp]),
        "fnGenPreviewTextureDevice": (c_int, [vp, c_int, c_int, c_int, vp, c_float, c_int, vp, vp, vp]),
        "fnEditorIpcSetup": (vp, [ctypes.c_bool]),
        "fnEditorIpcRelease": (None, [vp]),
        "fnEditorIpcSendSelectedNode": (ctypes.c_bool, [vp, cp]),
        "fnEditorIpcSendImportRequest": (ctypes.c_bool, [vp, cp]),
        "fnEditorIpcPollMessage": (c_int, [vp, vp, c_int]),
        "fnEditorIpcSetNodeEditorPath": (None, [cp]),
        "fnEditorIpcStartNodeEditor": (ctypes.c_bool, [cp, ctypes.c_bool, ctypes.c_bool]),
        "fnLiveTreeCreate": (vp, [vp, cp, vp, c_int, c_int]),
        "fnLiveTreeUpdate": (c_int, [vp]),
        "fnLiveTreeAcquire": (vp, [vp, vp]),
        "fnLiveTreeGetInfo": (c_int, [vp, vp]),
        "fnLiveTreeDelete": (None, [vp]),
        "fnAutotuneLoad": (c_int, [cp]),
        "fnAutotuneSave": (c_int, [cp]),
        "fnServerSubmitPaced": (c_int, [vp, vp, c_int, vp, vp]),
        "fnSetMeshDensityForm": (c_int, [c_int]),
        "fnJitCheckBatchVariants": (c_int, [vp, vp, c_int, ctypes.POINTER(c_int)]),
        "fnGenEachPaced": (c_int, [vp, c_int, vp, vp, vp]),
        "fnGetVariableBits": (c_int, [vp, c_int, ctypes.POINTER(c_int)]),
        "fnGetNodeLookupRef": (vp, [vp, c_int]),
        "fnGetHybridNodeLookupRef": (vp, [vp, c_int]),
        "fnGetHybridFloat": (c_int, [vp, c_int, ctypes.POINTER(c_float)]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    return L


def lib():
    """The loaded native library (raises ImportError if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            raise ImportError(f"{_LIB_PATH} is missing: build it with `python -m fastnoise2_gb300.build` "
                              "(this package has no CPU fallback)")
        _lib = _declare(ctypes.CDLL(_LIB_PATH))
    return _lib


def _check():
    L = lib()
    code = L.fnGetLastError()
    if code:
        raise FastNoiseError(code, L.fnGetLastErrorString().decode())


def _fp(a: np.ndarray):
    return a.ctypes.data_as(_FP)


def _i32(v) -> int:
    """An integer wrapped to int32 (seeds are int32 in the C interface)."""
    return ((int(v) + 0x80000000) & 0xFFFFFFFF) - 0x80000000


KIND_GRID2D, KIND_GRID3D, KIND_GRID4D, KIND_TILEABLE2D, KIND_POSITIONS2D, KIND_POSITIONS3D, KIND_POSITIONS4D = range(7)
BATCH_SYNC, BATCH_NO_GRAPH = 1, 2


class GenRequest(ctypes.Structure):
    """fnGenRequest: one request of a batched launch (include/FastNoise/FastNoise_C.h)."""
    _fields_ = [("node", ctypes.c_void_p), ("kind", ctypes.c_int), ("seed", ctypes.c_int),
                ("count", ctypes.c_int * 4), ("offset", ctypes.c_float * 4), ("step", ctypes.c_float * 4),
                ("positions", ctypes.c_void_p * 4), ("out", ctypes.c_void_p), ("minMax", ctypes.POINTER(ctypes.c_float))]


def make_request(node: "Node", kind: int, out_ptr: int, seed: int, count=(0, 0, 0, 0), offset=(0, 0, 0, 0),
                 step=(1, 1, 1, 1), positions=(0, 0, 0, 0), minmax: Optional[np.ndarray] = None) -> GenRequest:
    r = GenRequest()
    r.node = node.handle
    r._keep = node          # the request holds the Python node, so its native tree outlives the request
    r.kind = kind
    r.seed = int(np.int32(seed))
    for k in range(4):
        r.count[k] = int(count[k]) if k < len(count) else 0
        r.offset[k] = float(offset[k]) if k < len(offset) else 0.0
        r.step[k] = float(step[k]) if k < len(step) else 0.0
        r.positions[k] = int(positions[k]) if k < len(positions) and positions[k] else None
    r.out = out_ptr
    if minmax is not None:
        r.minMax = minmax.ctypes.data_as(_FP)
    return r


def gen_batch(requests, stream: int = 0, sync: bool = True, graph: bool = True) -> None:
    """fnGenBatchDevice over a sequence of GenRequest (or a prebuilt request_array())."""
    arr = request_array(requests)
    flags = (BATCH_SYNC if sync else 0) | (0 if graph else BATCH_NO_GRAPH)
    if lib().fnGenBatchDevice(arr, len(requests), stream or None, flags) != 0:
        _check()


def request_array(requests):
    """A ctypes array of GenRequest (build it once for request lists that are launched repeatedly)."""
    return requests if isinstance(requests, ctypes.Array) else (GenRequest * len(requests))(*requests)


def gen_batch_host(requests, graph: bool = True) -> None:
    """fnGenBatchHost: requests whose `out` is host memory; returns when every output is on the host."""
    arr = request_array(requests)
    if lib().fnGenBatchHost(arr, len(arr), 0 if graph else BATCH_NO_GRAPH) != 0:
        _check()


def gen_each(requests, stream: int = 0, sync: bool = True) -> None:
    """fnGenEachDevice: one plain launch per request (the per-call path)."""
    arr = request_array(requests)
    if lib().fnGenEachDevice(arr, len(requests), stream or None, BATCH_SYNC if sync else 0) != 0:
        _check()


def gen_each_paced(requests, arrivals_us, stream: int = 0) -> np.ndarray:
    """fnGenEachPaced: the per-call path driven by arrival times; returns each request's latency
    (microseconds from its arrival to its min/max on the host)."""
    arr = request_array(requests)
    times = np.ascontiguousarray(arrivals_us, np.float64)
    assert len(times) == len(arr)
    lat = np.zeros(len(arr), np.float64)
    if lib().fnGenEachPaced(arr, len(arr), times.ctypes.data, stream or None, lat.ctypes.data) != 0:
        _check()
    return lat


def autotune_batch(requests, stream: int = 0) -> None:
    arr = (GenRequest * len(requests))(*requests)
    if lib().fnAutotuneBatch(arr, len(requests), stream or None) != 0:
        _check()


def _jit_arrays(pairs):
    nodes = (ctypes.c_void_p * len(pairs))(*[n._h for n, _ in pairs])
    dims = (ctypes.c_int * len(pairs))(*[int(d) for _, d in pairs])
    return nodes, dims


def jit_compile(pairs) -> None:
    """Build specialised kernels for [(node, dimension), ...] (fnJitCompile)."""
    nodes, dims = _jit_arrays(pairs)
    if lib().fnJitCompile(nodes, dims, len(pairs)) != 0:
        _check()


MESH_DENSITY_ARRAY, MESH_DENSITY_SPARSE = 0, 1


def set_mesh_density_form(form: int) -> int:
    """fnSetMeshDensityForm: MESH_DENSITY_ARRAY (default) or MESH_DENSITY_SPARSE; returns the previous."""
    rc = lib().fnSetMeshDensityForm(int(form))
    if rc < 0:
        raise FastNoiseError(rc, "invalid mesh density form")
    return rc


def jit_check_batch_variants(pairs) -> int:
    """NVRTC-compile the other batch-kernel variants for [(node, dimension), ...] without loading them."""
    nodes, dims = _jit_arrays(pairs)
    n = ctypes.c_int(0)
    if lib().fnJitCheckBatchVariants(nodes, dims, len(pairs), ctypes.byref(n)) != 0:
        _check()
    return n.value


def autotune_save(path: str) -> None:
    if lib().fnAutotuneSave(str(path).encode()) != 0:
        raise FastNoiseError(-1, f"could not write {path}")


def autotune_load(path: str) -> None:
    if lib().fnAutotuneLoad(str(path).encode()) != 0:
        raise FastNoiseError(-1, f"could not read {path}")


def jit_set_cache_dir(path) -> None:
    """fnJitSetCacheDir: the on-disk cache of specialised modules for this process (None = off)."""
    lib().fnJitSetCacheDir(None if path is None else str(path).encode())


def jit_cache_info() -> dict:
    """fnJitGetCacheInfo: the cache directory in use ("" = off) and this process's hits and misses."""
    buf = ctypes.create_string_buffer(4096)
    hits, misses = ctypes.c_ulonglong(0), ctypes.c_ulonglong(0)
    lib().fnJitGetCacheInfo(buf, len(buf), ctypes.byref(hits), ctypes.byref(misses))
    return {"dir": buf.value.decode(), "hits": hits.value, "misses": misses.value}


def jit_check(pairs) -> int:
    """NVRTC-compile the module for [(node, dimension), ...] without loading it; returns cubin bytes."""
    nodes, dims = _jit_arrays(pairs)
    n = ctypes.c_int(0)
    if lib().fnJitCheck(nodes, dims, len(pairs), ctypes.byref(n)) != 0:
        _check()
    return n.value


class ChunkMesh(ctypes.Structure):
    """fnChunkMesh: device vertex (x, y, z, light) and index buffers plus the results."""
    _fields_ = [("vertices", ctypes.c_void_p), ("indices", ctypes.c_void_p), ("vertexCapacity", ctypes.c_int),
                ("indexCapacity", ctypes.c_int), ("vertexCount", ctypes.c_int), ("indexCount", ctypes.c_int),
                ("minAirY", ctypes.c_float), ("maxSolidY", ctypes.c_float), ("minMax", ctypes.c_float * 2)]

    def result(self) -> dict:
        return {"vertexCount": self.vertexCount, "indexCount": self.indexCount, "minAirY": self.minAirY,
                "maxSolidY": self.maxSolidY, "minMax": (self.minMax[0], self.minMax[1])}


def _mesh(rc: int, mesh: ChunkMesh) -> dict:
    if rc != 0 and rc != -4:
        _check()
    out = mesh.result()
    out["fits"] = rc == 0
    return out


def build_chunk_mesh_bloxel(node: "Node", size: int, pos, seed: int, iso: float, up_axis_z: bool, vertices_ptr: int,
                            vertex_capacity: int, indices_ptr: int, index_capacity: int, stream: int = 0) -> dict:
    """fnBuildChunkMeshBloxel into device buffers; returns counts, heights, min/max and whether it fit."""
    m = ChunkMesh(vertices_ptr or None, indices_ptr or None, vertex_capacity, index_capacity, 0, 0, 0.0, 0.0)
    rc = lib().fnBuildChunkMeshBloxel(node.handle, int(size), int(pos[0]), int(pos[1]), int(pos[2]), int(np.int32(seed)),
                                      float(iso), 1 if up_axis_z else 0, ctypes.byref(m), stream or None)
    return _mesh(rc, m)


def build_chunk_mesh_dmc(node: "Node", size: int, pos, seed: int, iso: float, up_axis_z: bool, vertices_ptr: int,
                         vertex_capacity: int, indices_ptr: int, index_capacity: int, stream: int = 0) -> dict:
    """fnBuildChunkMeshDmc (dual marching cubes) into device buffers; same result fields as the bloxel mesher."""
    m = ChunkMesh(vertices_ptr or None, indices_ptr or None, vertex_capacity, index_capacity, 0, 0, 0.0, 0.0)
    rc = lib().fnBuildChunkMeshDmc(node.handle, int(size), int(pos[0]), int(pos[1]), int(pos[2]), int(np.int32(seed)),
                                   float(iso), 1 if up_axis_z else 0, ctypes.byref(m), stream or None)
    return _mesh(rc, m)


def build_chunk_meshes(kind: str, node: "Node", size: int, positions, seed: int, iso: float, up_axis_z: bool, buffers,
                       stream: int = 0) -> list:
    """fnBuildChunkMeshesDmc / fnBuildChunkMeshesBloxel (kind "dmc" / "bloxel"): many chunks in one call.
    buffers: one (vertices_ptr, vertex_capacity, indices_ptr, index_capacity) per chunk."""
    n = len(positions)
    pos = (ctypes.c_int * (3 * n))(*[int(v) for p in positions for v in p])
    meshes = (ChunkMesh * n)(*[ChunkMesh(b[0] or None, b[2] or None, b[1], b[3], 0, 0, 0.0, 0.0) for b in buffers])
    fnc = lib().fnBuildChunkMeshesDmc if kind == "dmc" else lib().fnBuildChunkMeshesBloxel
    rc = fnc(node.handle, int(size), n, pos, int(np.int32(seed)), float(iso), 1 if up_axis_z else 0, meshes, stream or None)
    if rc != 0 and rc != -4:
        _check()
    out = []
    for m in meshes:
        r = m.result()
        r["fits"] = m.vertexCount <= m.vertexCapacity and m.indexCount <= m.indexCapacity
        out.append(r)
    return out


def build_chunk_mesh_heightmap(node: "Node", size: int, pos, seed: int, multiplier: float, vertices_ptr: int,
                               vertex_capacity: int, indices_ptr: int, index_capacity: int, stream: int = 0) -> dict:
    """fnBuildChunkMeshHeightmap into device buffers (pos = (x, z))."""
    m = ChunkMesh(vertices_ptr or None, indices_ptr or None, vertex_capacity, index_capacity, 0, 0, 0.0, 0.0)
    rc = lib().fnBuildChunkMeshHeightmap(node.handle, int(size), int(pos[0]), int(pos[1]), int(np.int32(seed)),
                                         float(multiplier), ctypes.byref(m), stream or None)
    return _mesh(rc, m)


def gen_preview_texture(node: "Node", gen_type: int, size, offset, scale: float, seed: int, pixels_ptr: int,
                        minmax_ptr: int = 0, stream: int = 0) -> None:
    """fnGenPreviewTextureDevice: the Node Editor's RGBA8 preview image into device uint32 pixels."""
    off = (ctypes.c_float * 4)(*[float(v) for v in (list(offset) + [0.0] * 4)[:4]])
    rc = lib().fnGenPreviewTextureDevice(node.handle, int(gen_type), int(size[0]), int(size[1]), off, float(scale),
                                         int(np.int32(seed)), pixels_ptr or None, minmax_ptr or None, stream or None)
    if rc != 0:
        _check()
        raise FastNoiseError(rc, "fnGenPreviewTextureDevice failed")


class EditorChannel:
    """The Node Editor's shared-memory channel (NodeEditorIpc_C.h): send and poll encoded trees."""

    SELECTED_NODE, IMPORT_REQUEST = 1, 2

    def __init__(self, read_previous: bool = False):
        self._h = lib().fnEditorIpcSetup(bool(read_previous))
        if not self._h:
            raise OSError("fnEditorIpcSetup failed (no POSIX shared memory?)")

    @property
    def handle(self) -> int:
        return self._h

    def send_selected(self, encoded: str) -> bool:
        return bool(lib().fnEditorIpcSendSelectedNode(self._h, encoded.encode()))

    def send_import(self, encoded: str) -> bool:
        return bool(lib().fnEditorIpcSendImportRequest(self._h, encoded.encode()))

    def poll(self, size: int = 65536):
        """(message type, tree) of the newest unseen message; type 0 = none, negative = error."""
        buf = ctypes.create_string_buffer(max(size, 1))
        t = lib().fnEditorIpcPollMessage(self._h, buf if size > 0 else None, size)
        return t, (buf.value.decode() if t > 0 else None)

    def close(self):
        if self._h:
            lib().fnEditorIpcRelease(self._h)
            self._h = None

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.fnEditorIpcRelease(self._h)
            self._h = None


def set_node_editor_path(path: Optional[str]) -> None:
    lib().fnEditorIpcSetNodeEditorPath(path.encode() if path else None)


def start_node_editor(encoded: Optional[str] = None, detached: bool = False, child: bool = True) -> bool:
    return bool(lib().fnEditorIpcStartNodeEditor(encoded.encode() if encoded else None, detached, child))


class LiveTreeInfo(ctypes.Structure):
    _fields_ = [("version", ctypes.c_ulonglong), ("rejected", ctypes.c_ulonglong), ("lastStatus", ctypes.c_int),
                ("lastError", ctypes.c_char * 256)]


class LiveTree:
    """fnLiveTree*: a tree that follows a Node Editor channel (hot swap of the selected tree)."""

    def __init__(self, channel: Optional[EditorChannel], initial: Optional[str], dims=(3,), poll_ms: int = 0):
        self._channel = channel                       # keeps the channel open while the tree lives
        arr = (ctypes.c_int * len(dims))(*dims)
        self._h = lib().fnLiveTreeCreate(channel.handle if channel else None, initial.encode() if initial else None,
                                          arr, len(dims), int(poll_ms))
        if not self._h:
            _check()
            raise FastNoiseError(-1, "fnLiveTreeCreate failed")

    def update(self) -> int:
        return lib().fnLiveTreeUpdate(self._h)

    def acquire(self):
        """(Node or None, version) of the current tree."""
        v = ctypes.c_ulonglong(0)
        h = lib().fnLiveTreeAcquire(self._h, ctypes.byref(v))
        return (Node(h) if h else None), v.value

    def info(self) -> dict:
        i = LiveTreeInfo()
        lib().fnLiveTreeGetInfo(self._h, ctypes.byref(i))
        return {"version": i.version, "rejected": i.rejected, "lastStatus": i.lastStatus, "lastError": i.lastError.decode()}

    def close(self):
        if self._h:
            lib().fnLiveTreeDelete(self._h)
            self._h = None

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.fnLiveTreeDelete(self._h)
            self._h = None


class BatchInfo(ctypes.Structure):
    _fields_ = [("requests", ctypes.c_int), ("specialised", ctypes.c_int), ("tilePoints", ctypes.c_int),
                ("ctas", ctypes.c_int), ("workItems", ctypes.c_ulonglong), ("points", ctypes.c_ulonglong),
                ("uploadBytes", ctypes.c_ulonglong), ("kernels", ctypes.c_int)]


def batch_info() -> dict:
    """Shape of this thread's last gen_batch launch (fnGetBatchInfo)."""
    info = BatchInfo()
    if lib().fnGetBatchInfo(ctypes.byref(info)) != 0:
        _check()
    return {k: getattr(info, k) for k, _ in info._fields_}


def set_auto_specialise(uses: int) -> int:
    """Interpreter runs after which a tree is specialised in the background (0 = off); returns the old value."""
    return lib().fnSetAutoSpecialise(int(uses))


def auto_specialise_wait(timeout_ms: int = -1) -> bool:
    """True once no background specialisation is queued or running."""
    return lib().fnAutoSpecialiseWait(int(timeout_ms)) == 0


def is_specialised(node: "Node", dim: int) -> bool:
    rc = lib().fnJitIsSpecialised(node.handle, int(dim))
    if rc < 0:
        _check()
    return rc == 1


def set_jit_enabled(on: bool) -> bool:
    """Use specialised kernels where built (True, default) or the interpreter only; returns the old setting."""
    return bool(lib().fnSetJitEnabled(1 if on else 0))


class ServerConfig(ctypes.Structure):
    _fields_ = [("poolBytes", ctypes.c_ulonglong), ("streams", ctypes.c_int), ("maxBatchRequests", ctypes.c_int),
                ("maxBatchPoints", ctypes.c_longlong), ("idleWaitMicros", ctypes.c_int)]


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_ulonglong), ("completed", ctypes.c_ulonglong), ("failed", ctypes.c_ulonglong),
                ("batches", ctypes.c_ulonglong), ("points", ctypes.c_ulonglong), ("p50Micros", ctypes.c_double),
                ("p99Micros", ctypes.c_double), ("maxMicros", ctypes.c_double), ("meanMicros", ctypes.c_double),
                ("poolUsed", ctypes.c_ulonglong), ("poolCapacity", ctypes.c_ulonglong), ("queueDepth", ctypes.c_int),
                ("inflight", ctypes.c_int), ("overlappedBatches", ctypes.c_ulonglong), ("maxInflightBatches", ctypes.c_int),
                ("maxConcurrentBatches", ctypes.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Server:
    """Continuous-batching request server (fnServerCreate ... fnServerDestroy)."""

    def __init__(self, pool_bytes: int = 1 << 30, streams: int = 3, max_batch_requests: int = 1024,
                 max_batch_points: int = 64 << 20, idle_wait_us: int = 50):
        cfg = ServerConfig(pool_bytes, streams, max_batch_requests, max_batch_points, idle_wait_us)
        self._h = lib().fnServerCreate(ctypes.byref(cfg))
        if not self._h:
            _check()
            raise FastNoiseError(-3, "server could not start")

    def close(self):
        if self._h:
            lib().fnServerDestroy(self._h)
            self._h = None

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            self.close()

    def submit(self, request: GenRequest) -> int:
        t = ctypes.c_ulonglong(0)
        if lib().fnServerSubmit(self._h, ctypes.byref(request), ctypes.byref(t)) != 0:
            _check()
        return t.value

    def submit_many(self, requests, as_array: bool = False):
        """Queue many requests at once (all or nothing); returns their tickets (a list, or the
        ctypes array itself with `as_array`).  `requests` may be a prebuilt request_array()."""
        n = len(requests)
        arr = requests if isinstance(requests, ctypes.Array) else (GenRequest * n)(*requests)
        t = (ctypes.c_ulonglong * n)()
        if lib().fnServerSubmitMany(self._h, arr, n, t) != 0:
            _check()
        return t if as_array else list(t)

    def submit_paced(self, requests, arrivals_us):
        """Open-loop submission (fnServerSubmitPaced): requests[k] is queued arrivals_us[k]
        microseconds after the call starts; returns the tickets (a ctypes array)."""
        n = len(requests)
        arr = request_array(requests)
        times = np.ascontiguousarray(arrivals_us, np.float64)
        assert len(times) == n
        t = (ctypes.c_ulonglong * n)()
        if lib().fnServerSubmitPaced(self._h, arr, n, times.ctypes.data, t) != 0:
            _check()
        return t

    def wait_many(self, tickets, timeout_ms: int = -1) -> None:
        """Wait until every ticket has finished; raises FastNoiseError on failure or timeout."""
        n = len(tickets)
        t = tickets if isinstance(tickets, ctypes.Array) else (ctypes.c_ulonglong * n)(*tickets)
        rc = lib().fnServerWaitMany(self._h, t, n, timeout_ms)
        if rc != 0:
            raise FastNoiseError(rc, lib().fnGetLastErrorString().decode())

    def poll(self, ticket: int) -> int:
        return lib().fnServerPoll(self._h, ticket)

    def wait(self, ticket: int, timeout_ms: int = -1):
        """Returns (min, max, device output pointer); raises FastNoiseError on failure or timeout."""
        mm = np.zeros(2, np.float32)
        ptr = ctypes.c_void_p(0)
        rc = lib().fnServerWait(self._h, ticket, timeout_ms, _fp(mm), ctypes.byref(ptr))
        if rc != 0:
            raise FastNoiseError(rc, lib().fnGetLastErrorString().decode())
        return float(mm[0]), float(mm[1]), ptr.value

    def cancel(self, ticket: int) -> int:
        return lib().fnServerCancel(self._h, ticket)

    def release(self, ticket: int) -> int:
        return lib().fnServerRelease(self._h, ticket)

    def stats(self) -> dict:
        s = ServerStats()
        lib().fnServerGetStats(self._h, ctypes.byref(s))
        return s.as_dict()

    def reset_stats(self) -> None:
        lib().fnServerResetStats(self._h)


def metadata_count() -> int:
    return lib().fnGetMetadataCount()


def metadata_name(node_id: int) -> str:
    return lib().fnGetMetadataName(node_id).decode()


def node_id(name: str) -> int:
    for i in range(metadata_count()):
        if metadata_name(i) == name:
            return i
    raise KeyError(name)


class Node:
    """Reference-counted handle to a node (FastNoise::SmartNode<>)."""

    def __init__(self, handle: int):
        if not handle:
            raise ValueError("null node handle")
        self._h = handle

    # -- construction -------------------------------------------------------
    @classmethod
    def new(cls, name_or_id: Union[str, int]) -> "Node":
        nid = node_id(name_or_id) if isinstance(name_or_id, str) else int(name_or_id)
        h = lib().fnNewFromMetadata(nid, 0)
        if not h:
            raise KeyError(name_or_id)
        return cls(h)

    @classmethod
    def from_encoded(cls, encoded: str) -> Optional["Node"]:
        h = lib().fnNewFromEncodedNodeTree(encoded.encode(), 0)
        return cls(h) if h else None

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.fnDeleteNodeRef(self._h)
            self._h = None

    @property
    def handle(self) -> int:
        return self._h

    @property
    def id(self) -> int:
        return lib().fnGetMetadataID(self._h)

    @property
    def name(self) -> str:
        return metadata_name(self.id)

    # -- members -----------------------------------------------------------
    def _find(self, kind: str, name: str, dim: Optional[int]) -> int:
        L, nid = lib(), self.id
        count = {"var": L.fnGetMetadataVariableCount, "lookup": L.fnGetMetadataNodeLookupCount,
                 "hybrid": L.fnGetMetadataHybridCount}[kind](nid)
        getn = {"var": L.fnGetMetadataVariableName, "lookup": L.fnGetMetadataNodeLookupName,
                "hybrid": L.fnGetMetadataHybridName}[kind]
        getd = {"var": L.fnGetMetadataVariableDimensionIdx, "lookup": L.fnGetMetadataNodeLookupDimensionIdx,
                "hybrid": L.fnGetMetadataHybridDimensionIdx}[kind]
        for i in range(count):
            if getn(nid, i).decode() == name and (dim is None or getd(nid, i) == dim):
                return i
        return -1

    def set(self, name: str, value, dim: Optional[int] = None) -> "Node":
        """Set a member variable, node lookup or hybrid by its metadata name."""
        L = lib()
        i = self._find("var", name, dim)
        if i >= 0:
            vtype = L.fnGetMetadataVariableType(self.id, i)
            if isinstance(value, str):
                names = [L.fnGetMetadataEnumName(self.id, i, e).decode() for e in range(L.fnGetMetadataEnumCount(self.id, i))]
                value = names.index(value)
            ok = L.fnSetVariableFloat(self._h, i, float(value)) if vtype == 0 else L.fnSetVariableIntEnum(self._h, i, int(value))
        elif (i := self._find("lookup", name, dim)) >= 0:
            ok = L.fnSetNodeLookup(self._h, i, value.handle)
        elif (i := self._find("hybrid", name, dim)) >= 0:
            ok = L.fnSetHybridNodeLookup(self._h, i, value.handle) if isinstance(value, Node) else L.fnSetHybridFloat(self._h, i, float(value))
        else:
            raise KeyError(f"{self.name} has no member {name!r}")
        if not ok:
            raise ValueError(f"{self.name}.{name} rejected {value!r}")
        return self

    def set_var_bits(self, index: int, bits: int) -> "Node":
        """fnSetVariableIntEnum with raw ValueUnion bits (how encoded trees set variables)."""
        lib().fnSetVariableIntEnum(self._h, index, int(np.int32(np.uint32(bits & 0xFFFFFFFF))))
        return self

    def encode(self) -> str:
        L = lib()
        n = L.fnSerialiseNodeTree(self._h, None, 0)
        if n < 0:
            _check()
        buf = ctypes.create_string_buffer(n + 1)
        L.fnSerialiseNodeTree(self._h, buf, n + 1)
        return buf.value.decode()

    def compile_info(self, dim: int) -> Tuple[int, int]:
        """(instructions, registers) of the device program for `dim` (host-only compile)."""
        ni, nr = ctypes.c_int(0), ctypes.c_int(0)
        if lib().fnCompileInfo(self._h, dim, ctypes.byref(ni), ctypes.byref(nr)) != 0:
            _check()
        return ni.value, nr.value

    def prepare(self, dim: int) -> None:
        if lib().fnPrepare(self._h, dim) != 0:
            _check()

    # -- generation (host memory, reference-compatible) ----------------------
    def gen_uniform_grid(self, offset: Sequence[float], count: Sequence[int], step: Sequence[float], seed: int,
                         out: Optional[np.ndarray] = None) -> Tuple[np.ndarray, Tuple[float, float]]:
        dim = len(count)
        total = math.prod(max(int(c), 0) for c in count)
        if out is None:
            out = np.empty(max(total, 1), np.float32)
        mm = np.zeros(2, np.float32)
        L = lib()
        f = {2: L.fnGenUniformGrid2D, 3: L.fnGenUniformGrid3D, 4: L.fnGenUniformGrid4D}.get(dim)
        if f is None:
            raise ValueError("dimension must be 2, 3 or 4")
        f(self._h, out.ctypes.data, *offset, *count, *step, _i32(seed), mm.ctypes.data)
        _check()
        return out[:total], (float(mm[0]), float(mm[1]))

    def gen_uniform_grid_2d(self, offset, count, step, seed, out=None):
        return self.gen_uniform_grid(offset, count, step, seed, out)

    def gen_uniform_grid_3d(self, offset, count, step, seed, out=None):
        return self.gen_uniform_grid(offset, count, step, seed, out)

    def gen_uniform_grid_4d(self, offset, count, step, seed, out=None):
        return self.gen_uniform_grid(offset, count, step, seed, out)

    def gen_position_array(self, positions: Sequence[np.ndarray], offset: Sequence[float], seed: int,
                           out: Optional[np.ndarray] = None) -> Tuple[np.ndarray, Tuple[float, float]]:
        dim = len(positions)
        arrs = [np.ascontiguousarray(p, np.float32) for p in positions]
        count = len(arrs[0])
        if out is None:
            out = np.empty(max(count, 1), np.float32)
        mm = np.zeros(2, np.float32)
        L = lib()
        f = {2: L.fnGenPositionArray2D, 3: L.fnGenPositionArray3D, 4: L.fnGenPositionArray4D}.get(dim)
        if f is None:
            raise ValueError("dimension must be 2, 3 or 4")
        f(self._h, out.ctypes.data, count, *(a.ctypes.data for a in arrs), *offset, _i32(seed), mm.ctypes.data)
        _check()
        return out[:count], (float(mm[0]), float(mm[1]))

    def gen_tileable_2d(self, size: Sequence[int], step: Sequence[float], seed: int,
                        out: Optional[np.ndarray] = None) -> Tuple[np.ndarray, Tuple[float, float]]:
        total = max(int(size[0]), 0) * max(int(size[1]), 0)
        if out is None:
            out = np.empty(max(total, 1), np.float32)
        mm = np.zeros(2, np.float32)
        lib().fnGenTileable2D(self._h, out.ctypes.data, int(size[0]), int(size[1]), float(step[0]), float(step[1]), _i32(seed),
                              mm.ctypes.data)
        _check()
        return out[:total], (float(mm[0]), float(mm[1]))

    def gen_single(self, pos: Sequence[float], seed: int) -> float:
        L = lib()
        s = int(np.int32(seed))
        p = list(map(float, pos))
        v = {2: L.fnGenSingle2D, 3: L.fnGenSingle3D, 4: L.fnGenSingle4D}[len(p)](self._h, *p, s)
        _check()
        return float(v)

    # -- generation into device memory (additions) ---------------------------
    def gen_uniform_grid_device(self, out_ptr: int, offset, count, step, seed: int, minmax_ptr: int = 0,
                                stream: int = 0) -> None:
        """Queue a grid into device memory `out_ptr` on `stream` (a cudaStream_t value)."""
        L = lib()
        dim = len(count)
        f = {2: L.fnGenUniformGrid2DDevice, 3: L.fnGenUniformGrid3DDevice, 4: L.fnGenUniformGrid4DDevice}[dim]
        rc = f(self._h, out_ptr, *map(float, offset), *map(int, count), *map(float, step), int(np.int32(seed)),
               minmax_ptr or None, stream or None)
        if rc != 0:
            _check()

    def gen_position_array_device(self, out_ptr: int, count: int, pos_ptrs: Sequence[int], offset, seed: int,
                                  minmax_ptr: int = 0, stream: int = 0) -> None:
        L = lib()
        dim = len(pos_ptrs)
        f = {2: L.fnGenPositionArray2DDevice, 3: L.fnGenPositionArray3DDevice, 4: L.fnGenPositionArray4DDevice}[dim]
        rc = f(self._h, out_ptr, int(count), *pos_ptrs, *map(float, offset), int(np.int32(seed)), minmax_ptr or None, stream or None)
        if rc != 0:
            _check()

    def gen_tileable_2d_device(self, out_ptr: int, size, step, seed: int, minmax_ptr: int = 0, stream: int = 0) -> None:
        rc = lib().fnGenTileable2DDevice(self._h, out_ptr, int(size[0]), int(size[1]), float(step[0]), float(step[1]),
                                         int(np.int32(seed)), minmax_ptr or None, stream or None)
        if rc != 0:
            _check()
