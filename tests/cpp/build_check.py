"""Build tests/cpp/cpp_api_check.cpp against the C++ headers in include/ and the in-tree
library (g++, a few seconds); the binary goes to tests/_build/."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
SRC = os.path.join(ROOT, "tests", "cpp", "cpp_api_check.cpp")
OUT_DIR = os.path.join(ROOT, "tests", "_build")
BIN = os.path.join(OUT_DIR, "cpp_api_check")


def build() -> str:
    from fastnoise2_gb300 import build as product
    lib = product.build()
    lib_dir = os.path.dirname(lib)
    os.makedirs(OUT_DIR, exist_ok=True)
    headers = [os.path.join(dp, f) for dp, _, fs in os.walk(os.path.join(ROOT, "include")) for f in fs]
    newest = max(os.path.getmtime(p) for p in [SRC, lib, *headers])
    if os.path.exists(BIN) and os.path.getmtime(BIN) >= newest:
        return BIN
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror", f"-I{ROOT}/include", SRC, "-o", BIN + ".tmp",
           f"-L{lib_dir}", "-lfastnoise_gb300", "-lpthread", f"-Wl,-rpath,{lib_dir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(BIN + ".tmp", BIN)
    return BIN
