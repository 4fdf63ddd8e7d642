"""ctypes wrapper of the CPU oracle (``oracle/jess_oracle.cpp``).

TEST INFRASTRUCTURE ONLY: imported by the tests, ``__graft_entry__.smoke()``
and the CPU-baseline leg of ``bench.py``; never by the product package.
"""

from __future__ import annotations

import ctypes as C
import os
import pathlib
import subprocess

import numpy as np

from pyjess_gb300._abi import QueryParams, Stats, ptr

HERE = pathlib.Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "libjess_oracle.so"

# Child push order of the kd-tree query, selected by the golden fixture
# (tests/test_oracle_golden.py): 1 = right subtree visited first.
KD_RIGHT_FIRST = 1

_lib = None


def build() -> pathlib.Path:
    """Compile the oracle with the committed Makefile (idempotent)."""
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB_PATH


# cell sizes (A) of the uniform grids the culling counts model
CULL_GRID = (2.0, 3.0, 4.0, 6.0)


def lib():
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            build()
        L = C.CDLL(str(LIB_PATH))
        L.oracle_query.restype = C.c_void_p
        L.oracle_query.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int]
        for name in ("oracle_hit_count", "oracle_hit_atom_count", "oracle_stream_count",
                     "oracle_stream_atom_count", "oracle_warning_count"):
            getattr(L, name).restype = C.c_int64
            getattr(L, name).argtypes = [C.c_void_p]
        L.oracle_hits.argtypes = [C.c_void_p] + [C.c_void_p] * 8
        L.oracle_stream.argtypes = [C.c_void_p] + [C.c_void_p] * 7
        L.oracle_warnings.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.oracle_stats.argtypes = [C.c_void_p, C.c_void_p]
        L.oracle_free.argtypes = [C.c_void_p]
        L.oracle_boundary_stats.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.oracle_set_kd_right_first.argtypes = [C.c_int]
        L.oracle_set_kd_right_first(KD_RIGHT_FIRST)
        L.oracle_set_cull_stats.argtypes = [C.c_int]
        L.oracle_cull_stats.argtypes = [C.c_void_p, C.c_void_p]
        _lib = L
    return _lib


def query(ptemplates, pstructures, *, rmsd_threshold, distance_cutoff, max_dynamic_distance,
          max_candidates=-1, ignore_chain=0, best_match=False, reorder=True, threads=1,
          stream=False, kd_right_first=None, cull_stats=False):
    """Run the oracle; returns a dict of NumPy arrays (hits, stream, warnings, stats).
    cull_stats: also count, for every kd range query on a list of 64 or more
    points, the points each culling scheme would load (``out["cull"]``)."""
    L = lib()
    if kd_right_first is not None:
        L.oracle_set_kd_right_first(int(kd_right_first))
    L.oracle_set_cull_stats(1 if cull_stats else 0)
    P = QueryParams(rmsd_threshold=rmsd_threshold, distance_cutoff=distance_cutoff,
                    max_dynamic_distance=max_dynamic_distance,
                    max_candidates=-1 if max_candidates is None else int(max_candidates),
                    ignore_chain=int(ignore_chain), best_match=int(best_match),
                    reorder=int(reorder), mode=0, guard_band=0.0)
    tset = ptemplates.abi()
    sset = pstructures.abi()
    h = L.oracle_query(C.byref(tset), C.byref(sset), C.byref(P), int(threads), int(stream))
    try:
        out = {}
        n = L.oracle_hit_count(h)
        na = L.oracle_hit_atom_count(h)
        hits = {
            "count": n,
            "structure": np.zeros(n, np.int32),
            "template": np.zeros(n, np.int32),
            "ordinal": np.zeros(n, np.int64),
            "rmsd": np.zeros(n, np.float64),
            "rotation": np.zeros((n, 9), np.float64),
            "centres": np.zeros((n, 6), np.float64),
            "atom_offset": np.zeros(n + 1, np.int64),
            "atoms": np.zeros(na, np.int32),
        }
        L.oracle_hits(h, *(hits[k].ctypes.data for k in
                           ("structure", "template", "ordinal", "rmsd", "rotation", "centres",
                            "atom_offset", "atoms")))
        out["hits"] = hits
        if stream:
            m = L.oracle_stream_count(h)
            ma = L.oracle_stream_atom_count(h)
            st = {
                "count": m,
                "structure": np.zeros(m, np.int32),
                "template": np.zeros(m, np.int32),
                "ordinal": np.zeros(m, np.int64),
                "rmsd": np.zeros(m, np.float64),
                "nan_rot": np.zeros(m, np.int32),
                "atom_offset": np.zeros(m + 1, np.int64),
                "atoms": np.zeros(ma, np.int32),
            }
            L.oracle_stream(h, *(st[k].ctypes.data for k in
                                 ("structure", "template", "ordinal", "rmsd", "nan_rot",
                                  "atom_offset", "atoms")))
            out["stream"] = st
        w = L.oracle_warning_count(h)
        ws = np.zeros(w, np.int32)
        wb = np.zeros(w, np.int64)
        L.oracle_warnings(h, ws.ctypes.data, wb.ctypes.data)
        out["warnings"] = (ws, wb)
        stats = Stats()
        L.oracle_stats(h, C.byref(stats))
        out["stats"] = stats.as_dict()
        tests, near = C.c_int64(), C.c_int64()
        L.oracle_boundary_stats(h, C.byref(tests), C.byref(near))
        out["boundary"] = {"tests": tests.value, "near": near.value}
        if cull_stats:
            v = np.zeros(13 + 2 * len(CULL_GRID), np.int64)
            L.oracle_cull_stats(h, v.ctypes.data)
            out["cull"] = {
                **dict(zip(("queries", "points", "in_box", "children", "kd_nodes", "blocks_hit", "block_loaded",
                            "sub_hit", "sub_loaded", "groups", "group_members", "group_blocks_hit",
                            "group_loaded"), (int(x) for x in v[:13]))),
                "grid": {g: {"cells": int(v[13 + 2 * i]), "loaded": int(v[14 + 2 * i])}
                         for i, g in enumerate(CULL_GRID)}}
        return out
    finally:
        L.oracle_free(h)
