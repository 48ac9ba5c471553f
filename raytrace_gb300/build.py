"""Build recipe for the GB300 renderer library and the CPU oracle.

Compiles every CUDA translation unit for sm_103a with nvcc and the host C++ layer with g++,
in parallel, into raytrace_gb300/_build/librt_gb300.so. Object files are rebuilt when their
source or any header of the package is newer. No cmake, no torch extension machinery: the
library is a plain C-ABI shared object loaded with ctypes.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(BUILD, "librt_gb300.so")

NVCC = os.environ.get("NVCC", "nvcc")
CXX = os.environ.get("CXX", "g++")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                     "-Xptxas", "-O3", "--expt-relaxed-constexpr"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function"]


def _headers() -> list[str]:
    pats = ["csrc/*.cuh", "csrc/*.h", "cpp/*.h"]
    out = [os.path.join(ROOT, "include", "rt_gb300.h")]
    for p in pats:
        out += glob.glob(os.path.join(PKG, p))
    return out


def _stale(obj: str, src: str, deps: list[str]) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in [src] + deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def build(verbose: bool = False, jobs: int | None = None) -> str:
    """Compile (incrementally) and link librt_gb300.so; returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    deps = _headers()
    units = []
    for src in sorted(glob.glob(os.path.join(PKG, "csrc", "*.cu"))):
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        units.append((src, obj, [NVCC] + NVCC_FLAGS + ["-c", src, "-o", obj]))
    for src in sorted(glob.glob(os.path.join(PKG, "cpp", "*.cpp")) + glob.glob(os.path.join(PKG, "csrc", "*.cpp"))):
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        inc = ["-I", "/usr/local/cuda/include"]
        units.append((src, obj, [CXX] + CXX_FLAGS + inc + ["-c", src, "-o", obj]))
    todo = [u for u in units if _stale(u[1], u[0], deps)]
    with cf.ThreadPoolExecutor(max_workers=jobs or min(16, os.cpu_count() or 4)) as ex:
        futs = {ex.submit(_run, u[2]): u for u in todo}
        for f in cf.as_completed(futs):
            f.result()
            if verbose:
                print("compiled", os.path.basename(futs[f][0]), flush=True)
    objs = [u[1] for u in units]
    if todo or not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        _run([NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart", "-lpthread"])
        if verbose:
            print("linked", LIB, flush=True)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
    sys.exit(0)
