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

CU_SOURCES = ["fn_kernels.cu", "fn_static_scratch.cu", "fn_mesh.cu"]
CPP_SOURCES = ["fn_node.cpp", "fn_compile.cpp", "fn_runtime.cpp", "fn_batch.cpp", "fn_server.cpp", "fn_capi.cpp",
               "fn_jit.cpp", "fn_ipc.cpp", "fn_live.cpp", "fn_capi_mesh.cpp"]

# Headers handed to NVRTC at run time (in this order), embedded into the library.
JIT_HEADERS = ["fn_types.h", "fn_device.cuh", "fn_eval.cuh"]
JIT_SRC = os.path.join(OUT, "fn_embedded_src.gen.cpp")

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


def _write_embedded_source() -> None:
    """Generate the C++ file holding the device headers as one string for NVRTC.

    Include lines and include guards are dropped (the headers are concatenated in
    dependency order) and the fixed-width integer types come from a prelude, since
    NVRTC has no standard headers."""
    parts = ["#define FN_DEVICE_NO_STDINT\n",
             "typedef unsigned char uint8_t; typedef unsigned short uint16_t; typedef unsigned int uint32_t;\n",
             "typedef int int32_t; typedef long long int64_t; typedef unsigned long long uint64_t;\n"]
    for h in JIT_HEADERS:
        for line in open(os.path.join(CSRC, h)):
            if line.lstrip().startswith(("#include", "#pragma once")):
                continue
            parts.append(line)
    text = "".join(parts)
    body = ("// generated by fastnoise2_gb300/build.py -- do not edit\n"
            "namespace fn {\nconst char* embedded_device_source()\n{\n    static const char* s =\n")
    # split into chunks below the compilers' single-literal limits
    chunk = 8000
    for i in range(0, len(text), chunk):
        body += '        R"FNSRC(' + text[i:i + chunk] + ')FNSRC"\n'
    body += "        ;\n    return s;\n}\n}  // namespace fn\n"
    if os.path.exists(JIT_SRC) and open(JIT_SRC).read() == body:
        return
    with open(JIT_SRC + ".tmp", "w") as f:
        f.write(body)
    os.replace(JIT_SRC + ".tmp", JIT_SRC)


def _compile(src: str) -> str:
    if os.path.isabs(src):
        path, obj = src, os.path.join(OUT, os.path.basename(src) + ".o")
        if os.path.exists(obj) and os.path.getmtime(obj) >= os.path.getmtime(path):
            return obj
        cmd = ["g++", *CXXFLAGS, "-c", path, "-o", obj + ".tmp"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        os.replace(obj + ".tmp", obj)
        return obj
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
    _write_embedded_source()
    sources = CU_SOURCES + CPP_SOURCES + [JIT_SRC]
    with ThreadPoolExecutor(max_workers=min(8, len(sources))) as ex:
        objs = list(ex.map(_compile, sources))
    if os.path.exists(LIB) and all(os.path.getmtime(o) <= os.path.getmtime(LIB) for o in objs):
        return LIB
    cmd = ["g++", "-shared", "-o", LIB + ".tmp", *objs, f"-L{CUDA_HOME}/lib64", "-lcudart", "-lnvrtc", "-lpthread", "-lrt", "-ldl",
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
