"""Build libfastnoise_gb300.so in-tree (fastnoise2_gb300/_lib/).

CUDA sources are compiled for sm_103a only, with ``-fmad=false`` so that the
kernels fuse multiply-adds exactly where the reference's FS::FMulAdd does and
nowhere else; host sources use ``-ffp-contract=off`` for the same reason
(parameters such as 1/scale are computed on the host).  Translation units are
compiled in parallel; unchanged objects are reused.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT, "libfastnoise_gb300.so")
ROOT = os.path.dirname(HERE)

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SOURCES = ["fn_kernels.cu", "fn_static_scratch.cu"]
CPP_SOURCES = ["fn_node.cpp", "fn_compile.cpp", "fn_runtime.cpp", "fn_batch.cpp", "fn_server.cpp", "fn_capi.cpp"]

CXXFLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fvisibility=hidden", "-Wall",
            f"-I{CUDA_HOME}/include", f"-I{ROOT}/include"]
NVCCFLAGS = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "--expt-relaxed-constexpr",
                    "-Xcompiler", "-fPIC,-ffp-contract=off,-fvisibility=hidden", f"-I{ROOT}/include"]


def _deps_newer(obj: str, src: str) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "FastNoise", "FastNoise_C.h"))
    return any(os.path.getmtime(p) > t for p in [src, *headers, __file__])


def _compile(src: str) -> str:
    path = os.path.join(CSRC, src)
    obj = os.path.join(OUT, src + ".o")
    if not _deps_newer(obj, path):
        return obj
    if src.endswith(".cu"):
        cmd = [NVCC, *NVCCFLAGS, "-c", path, "-o", obj + ".tmp"]
    else:
        cmd = ["g++", *CXXFLAGS, "-c", path, "-o", obj + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(obj + ".tmp", obj)
    return obj


def build(verbose: bool = False) -> str:
    """Compile every translation unit and link the shared library; returns its path."""
    os.makedirs(OUT, exist_ok=True)
    if not os.path.exists(NVCC):
        raise RuntimeError(f"nvcc not found at {NVCC}")
    sources = CU_SOURCES + CPP_SOURCES
    with ThreadPoolExecutor(max_workers=min(8, len(sources))) as ex:
        objs = list(ex.map(_compile, sources))
    if os.path.exists(LIB) and all(os.path.getmtime(o) <= os.path.getmtime(LIB) for o in objs):
        return LIB
    cmd = ["g++", "-shared", "-o", LIB + ".tmp", *objs, f"-L{CUDA_HOME}/lib64", "-lcudart", "-lpthread",
           f"-Wl,-rpath,{CUDA_HOME}/lib64"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(LIB + ".tmp", LIB)
    if verbose:
        print("built", LIB)
    return LIB


def clean() -> None:
    if os.path.isdir(OUT):
        shutil.rmtree(OUT)


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
