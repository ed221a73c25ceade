"""Builds libmole_gpu.so (sm_103a) in-tree under mole_gb300/_build/.

Each translation unit compiles in its own nvcc process, in parallel, and is
skipped when its object is newer than every source and header; the objects
are linked into one shared library that exports the C ABI of
include/mole_gpu.h.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libmole_gpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build mole_gb300")
    return p


def sources() -> list[str]:
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def headers() -> list[str]:
    return sorted(glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(ROOT, "include", "*.h")))


def _stale(obj: str, deps: list[str]) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src: str, verbose: bool) -> str:
    obj = os.path.join(OUT, os.path.basename(src) + ".o")
    if not _stale(obj, [src] + headers()):
        return obj
    cmd = [nvcc(), *ARCH, *FLAGS, "-c", src, "-o", obj + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {os.path.basename(src)}:\n{r.stderr[-4000:]}")
    os.replace(obj + ".tmp", obj)
    if verbose:
        print(f"  compiled {os.path.basename(src)}", flush=True)
    return obj


def build(jobs: int | None = None, verbose: bool = False) -> str:
    """Compile every CUDA translation unit and link libmole_gpu.so; returns its path."""
    os.makedirs(OUT, exist_ok=True)
    srcs = sources()
    jobs = jobs or max(1, os.cpu_count() or 1)
    # the slowest translation units (largest spin families, double-float) first
    # so the parallel build finishes sooner
    def weight(s: str) -> int:
        b = os.path.basename(s)
        return (os.path.getsize(s) + 100000 * ("_2_2" in b) + 60000 * ("inst_df" in b or "inst_nn" in b)
                + 40000 * ("_2_1" in b) + 200000 * (b == "capi.cu"))

    srcs.sort(key=lambda s: -weight(s))
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    if _stale(LIB, objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", LIB + ".tmp", *sorted(objs), "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr[-4000:]}")
        os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
    sys.exit(0)
