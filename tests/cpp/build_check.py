"""Build the C++ checks in tests/cpp/ (cpp_api_check.cpp, latency_check.cpp) against the
headers in include/ and the in-tree library (g++, a few seconds); binaries go to tests/_build/."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
OUT_DIR = os.path.join(ROOT, "tests", "_build")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def build(name: str = "cpp_api_check") -> str:
    from fastnoise2_gb300 import build as product
    lib = product.build()
    lib_dir = os.path.dirname(lib)
    src = os.path.join(ROOT, "tests", "cpp", name + ".cpp")
    out = os.path.join(OUT_DIR, name)
    os.makedirs(OUT_DIR, exist_ok=True)
    headers = [os.path.join(dp, f) for dp, _, fs in os.walk(os.path.join(ROOT, "include")) for f in fs]
    newest = max(os.path.getmtime(p) for p in [src, lib, *headers])
    if os.path.exists(out) and os.path.getmtime(out) >= newest:
        return out
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror", f"-I{ROOT}/include", f"-I{CUDA_HOME}/include", src,
           "-o", out + ".tmp", f"-L{lib_dir}", "-lfastnoise_gb300", f"-L{CUDA_HOME}/lib64", "-lcudart", "-lpthread",
           f"-Wl,-rpath,{lib_dir}", f"-Wl,-rpath,{CUDA_HOME}/lib64"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(out + ".tmp", out)
    return out
