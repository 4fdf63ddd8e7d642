"""Build ``libpjg.so`` from ``csrc/`` with nvcc for sm_103a (in-tree).

The library lands in ``pyjess_gb300/_lib/``.  Each translation unit is
compiled in its own nvcc process (in parallel), then linked; host code is
built with ``-ffp-contract=off`` so its FP64 arithmetic (template distance
matrices) is identical on x86-64 and aarch64.
"""

from __future__ import annotations

import concurrent.futures
import os
import pathlib
import shutil
import subprocess
import sys

HERE = pathlib.Path(__file__).resolve().parent
CSRC = HERE / "csrc"
LIBDIR = HERE / "_lib"
LIB = LIBDIR / "libpjg.so"
INCLUDE = HERE.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3", "-std=c++17", "-lineinfo", "--expt-relaxed-constexpr",
    "-Xcompiler", "-fPIC,-ffp-contract=off,-O2",
    "-I", str(INCLUDE),
]
SOURCES = ["pjg_kernels.cu", "pjg_api.cu", "pjg_io.cpp"]
# library variants: "" the product library; "prof" adds the search profile
# (event counts and section cycles of k_search, written per query to the
# file named by PJG_PROF_OUT) and is never the timed build; "blk8"/"blk16"
# cull by blocks of 8/16 leaves instead of 32, "w10" runs the search with
# 10 warps a block, "rank" orders tie-free lists by the rank method instead
# of axis partitions, "part256"/"part512" order tie-free lists longer than
# 256/512 entries by sorted axes instead of axis partitions (measured against
# each other)
VARIANTS = {"": [], "prof": ["-DPJG_SEARCH_PROF=1"], "blk8": ["-DPJG_CULL_BLK=8"], "blk16": ["-DPJG_CULL_BLK=16"],
            "blk8prof": ["-DPJG_CULL_BLK=8", "-DPJG_SEARCH_PROF=1"], "w10": ["-DPJG_SEARCH_WARPS=10"],
            "rank": ["-DPJG_LEAF_RANK=1"], "rankprof": ["-DPJG_LEAF_RANK=1", "-DPJG_SEARCH_PROF=1"],
            "part256": ["-DPJG_PART_MAX=256"], "part512": ["-DPJG_PART_MAX=512"]}


def lib_path(variant: str = "") -> pathlib.Path:
    return LIB if not variant else LIBDIR / f"libpjg_{variant}.so"


def nvcc() -> str:
    path = shutil.which("nvcc")
    if path:
        return path
    cand = pathlib.Path("/usr/local/cuda/bin/nvcc")
    if cand.exists():
        return str(cand)
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libpjg")


def _stale(lib: pathlib.Path = LIB) -> bool:
    if not lib.exists():
        return True
    t = lib.stat().st_mtime
    deps = (list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.cpp")) +
            [INCLUDE / "pjg.h", pathlib.Path(__file__)])
    return any(p.stat().st_mtime > t for p in deps)


def build(force: bool = False, verbose: bool = False, extra=(), variant: str = "") -> pathlib.Path:
    lib = lib_path(variant)
    if not force and not _stale(lib):
        return lib
    extra = [*VARIANTS[variant], *extra]
    LIBDIR.mkdir(exist_ok=True)
    objdir = LIBDIR / ("obj" if not variant else f"obj_{variant}")
    objdir.mkdir(exist_ok=True)
    cc = nvcc()

    def compile_one(src):
        obj = objdir / (src + ".o")
        cmd = [cc, *ARCH, *NVCC_FLAGS, *extra, "-c", str(CSRC / src), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr, file=sys.stderr)
        return obj

    with concurrent.futures.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = lib.with_suffix(".so.tmp")
    cmd = [cc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
