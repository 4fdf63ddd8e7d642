"""ctypes mirrors of the structs declared in ``include/pjg.h``."""

from __future__ import annotations

import ctypes as C

import numpy as np


class TemplateSet(C.Structure):
    _fields_ = [
        ("n_templates", C.c_int32),
        ("atom_offset", C.POINTER(C.c_int32)),
        ("code", C.POINTER(C.c_int32)),
        ("res_seq", C.POINTER(C.c_int32)),
        ("chain", C.POINTER(C.c_uint8)),
        ("xyz", C.POINTER(C.c_double)),
        ("dist_weight", C.POINTER(C.c_double)),
        ("name_offset", C.POINTER(C.c_int32)),
        ("names", C.POINTER(C.c_uint8)),
        ("resname_offset", C.POINTER(C.c_int32)),
        ("resnames", C.POINTER(C.c_uint8)),
        ("dim", C.POINTER(C.c_int32)),
    ]


class StructureSet(C.Structure):
    _fields_ = [
        ("n_structures", C.c_int32),
        ("atom_offset", C.POINTER(C.c_int64)),
        ("xyz", C.POINTER(C.c_double)),
        ("name", C.POINTER(C.c_uint8)),
        ("resname", C.POINTER(C.c_uint8)),
        ("chain", C.POINTER(C.c_uint8)),
        ("res_seq", C.POINTER(C.c_int32)),
        ("serial", C.POINTER(C.c_int32)),
    ]


class QueryParams(C.Structure):
    _fields_ = [
        ("rmsd_threshold", C.c_double),
        ("distance_cutoff", C.c_double),
        ("max_dynamic_distance", C.c_double),
        ("max_candidates", C.c_int32),
        ("ignore_chain", C.c_int32),
        ("best_match", C.c_int32),
        ("reorder", C.c_int32),
        ("mode", C.c_int32),
        ("guard_band", C.c_double),
        ("count_only", C.c_int32),
    ]


class Tuning(C.Structure):
    """pjg_tuning: execution knobs of pjg_query (0 keeps a default)."""

    _fields_ = [
        ("leaf_levels", C.c_int32),
        ("block_min", C.c_int32),
        ("tile_cap", C.c_int32),
        ("pair_grain", C.c_int32),
        ("leaf_rank_max", C.c_int32),
        ("leaf_reach", C.c_int32),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class Stats(C.Structure):
    _fields_ = [
        ("pairs", C.c_int64),
        ("candidate_entries", C.c_int64),
        ("partials", C.c_int64),
        ("complete", C.c_int64),
        ("passing", C.c_int64),
        ("hits", C.c_int64),
        ("fp64_rechecks", C.c_int64),
        ("leaf_exact", C.c_int64),
        ("leaf_sorted", C.c_int64),
        ("leaf_replays", C.c_int64),
        ("bytes_candidates", C.c_int64),
        ("bytes_expansion", C.c_int64),
        ("bytes_superposition", C.c_int64),
        ("ms_candidates", C.c_double),
        ("ms_expansion", C.c_double),
        ("ms_superposition", C.c_double),
        ("ms_total", C.c_double),
        ("launches", C.c_int32),
        ("chunks", C.c_int32),
        ("leaf_lists", C.c_int64),
        ("leaf_entries", C.c_int64),
        ("suspensions", C.c_int64),
        ("search_rounds", C.c_int32),
        ("row_splits", C.c_int32),
        ("leaf_shared", C.c_int64),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


def ptr(array: np.ndarray, ctype):
    """Pointer to the data of a C-contiguous array (kept alive by the caller)."""
    assert array.flags["C_CONTIGUOUS"]
    return array.ctypes.data_as(C.POINTER(ctype))
