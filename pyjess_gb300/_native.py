"""ctypes binding of ``libpjg.so`` (the C ABI declared in ``include/pjg.h``).

There is no CPU fallback: if the library is missing or no CUDA device is
visible, every entry point here raises `RuntimeError`.
"""

from __future__ import annotations

import ctypes as C
import os
import threading

import numpy as np

from ._abi import QueryParams, Stats, StructureSet, TemplateSet, Tuning
from ._build import build, lib_path

MODE_PLAIN_FP64 = 0
MODE_BATCHED_FP32 = 1
MODE_BATCHED_FP64 = 2

PJG_OK = 0
_STATUS = {1: "invalid argument", 2: "out of memory", 3: "CUDA error", 4: "no CUDA device",
           5: "timeout", 6: "capacity exceeded"}

# every symbol of include/pjg.h
EXPORTED = (
    "pjg_init", "pjg_last_error", "pjg_templates_create", "pjg_templates_destroy",
    "pjg_structures_create", "pjg_structures_destroy", "pjg_query", "pjg_results_count",
    "pjg_results_atom_count", "pjg_results_copy", "pjg_results_warning_count",
    "pjg_results_warnings", "pjg_results_superposed", "pjg_results_stats", "pjg_results_destroy",
    "pjg_set_tuning", "pjg_get_tuning",
    "pjg_device_name", "pjg_parse_pdb", "pjg_superpose_noalloc", "pjg_noalloc_last_error",
)

_lib = None
_lock = threading.Lock()
_initialized = False


def load(build_if_missing: bool = True):
    """Load the library (building it in-tree first if it is absent).
    ``PJG_LIB_VARIANT=prof`` loads the search-profile build instead."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        variant = os.environ.get("PJG_LIB_VARIANT", "")
        lib = lib_path(variant)
        if not lib.exists():
            if not build_if_missing:
                raise RuntimeError(f"{lib.name} not built ({lib}); run pyjess_gb300._build.build()")
            build(variant=variant)
        L = C.CDLL(str(lib))
        L.pjg_init.argtypes = [C.c_int32]
        L.pjg_init.restype = C.c_int
        L.pjg_last_error.restype = C.c_char_p
        L.pjg_templates_create.argtypes = [C.POINTER(TemplateSet), C.POINTER(C.c_void_p)]
        L.pjg_templates_create.restype = C.c_int
        L.pjg_templates_destroy.argtypes = [C.c_void_p]
        L.pjg_structures_create.argtypes = [C.POINTER(StructureSet), C.POINTER(C.c_void_p)]
        L.pjg_structures_create.restype = C.c_int
        L.pjg_structures_destroy.argtypes = [C.c_void_p]
        L.pjg_query.argtypes = [C.c_void_p, C.c_void_p, C.POINTER(QueryParams), C.POINTER(C.c_void_p)]
        L.pjg_query.restype = C.c_int
        L.pjg_results_count.argtypes = [C.c_void_p]
        L.pjg_results_count.restype = C.c_int64
        L.pjg_results_atom_count.argtypes = [C.c_void_p]
        L.pjg_results_atom_count.restype = C.c_int64
        L.pjg_results_copy.argtypes = [C.c_void_p] + [C.c_void_p] * 8
        L.pjg_results_copy.restype = C.c_int
        L.pjg_results_warning_count.argtypes = [C.c_void_p]
        L.pjg_results_warning_count.restype = C.c_int64
        L.pjg_results_warnings.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.pjg_results_warnings.restype = C.c_int
        L.pjg_results_stats.argtypes = [C.c_void_p, C.POINTER(Stats)]
        L.pjg_results_stats.restype = C.c_int
        L.pjg_results_destroy.argtypes = [C.c_void_p]
        L.pjg_results_superposed.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.pjg_results_superposed.restype = C.c_int
        L.pjg_set_tuning.argtypes = [C.POINTER(Tuning)]
        L.pjg_set_tuning.restype = C.c_int
        L.pjg_get_tuning.argtypes = [C.POINTER(Tuning)]
        L.pjg_get_tuning.restype = C.c_int
        L.pjg_device_name.argtypes = [C.c_char_p, C.c_int32]
        L.pjg_device_name.restype = C.c_int
        L.pjg_parse_pdb.argtypes = [C.c_char_p, C.c_int64, C.c_int32, C.c_void_p, C.c_int64,
                                    C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
        L.pjg_parse_pdb.restype = C.c_int
        _lib = L
        return L


def _check(status: int, what: str):
    if status != PJG_OK:
        msg = _lib.pjg_last_error().decode(errors="replace")
        raise RuntimeError(f"{what}: {_STATUS.get(status, status)}: {msg}")


def init(device: int | None = None):
    """Select the CUDA device (``PJG_DEVICE`` env var, default 0)."""
    global _initialized
    L = load()
    if device is None:
        device = int(os.environ.get("PJG_DEVICE", os.environ.get("LOCAL_RANK", "0")))
    _check(L.pjg_init(device), "pjg_init")
    _initialized = True
    return L


def _ready():
    if not _initialized:
        init()
    return _lib


class Templates:
    """Device-resident templates (``pjg_templates``)."""

    def __init__(self, packed):
        L = _ready()
        self._packed = packed
        self._abi = packed.abi()
        h = C.c_void_p()
        _check(L.pjg_templates_create(C.byref(self._abi), C.byref(h)), "pjg_templates_create")
        self.handle = h

    def __del__(self):
        if getattr(self, "handle", None) and _lib is not None:
            _lib.pjg_templates_destroy(self.handle)
            self.handle = None


class Structures:
    """Device-resident structures (``pjg_structures``)."""

    def __init__(self, packed):
        L = _ready()
        self._packed = packed
        self._abi = packed.abi()
        h = C.c_void_p()
        _check(L.pjg_structures_create(C.byref(self._abi), C.byref(h)), "pjg_structures_create")
        self.handle = h

    def __del__(self):
        if getattr(self, "handle", None) and _lib is not None:
            _lib.pjg_structures_destroy(self.handle)
            self.handle = None


def structures_for(molecules) -> Structures:
    from ._pack import pack_molecules

    return Structures(pack_molecules(molecules))


class Result:
    """Hits of one `pjg_query` call, copied out as NumPy arrays."""

    def __init__(self, handle):
        self.handle = handle
        self._arrays = None

    def __del__(self):
        if getattr(self, "handle", None) and _lib is not None:
            _lib.pjg_results_destroy(self.handle)
            self.handle = None

    def arrays(self) -> dict:
        if self._arrays is None:
            L = _lib
            n = L.pjg_results_count(self.handle)
            na = L.pjg_results_atom_count(self.handle)
            a = {
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
            _check(L.pjg_results_copy(self.handle, *(a[k].ctypes.data for k in (
                "structure", "template", "ordinal", "rmsd", "rotation", "centres", "atom_offset", "atoms"))),
                "pjg_results_copy")
            self._arrays = a
        return self._arrays

    def superposed(self, structures: "Structures") -> np.ndarray:
        """Every hit's matched atoms in its template's frame, (atoms, 3),
        computed on the device (pjg_results_superposed)."""
        L = _lib
        na = L.pjg_results_atom_count(self.handle)
        out = np.zeros((na, 3), np.float64)
        _check(L.pjg_results_superposed(self.handle, structures.handle, out.ctypes.data), "pjg_results_superposed")
        return out

    def warnings(self):
        L = _lib
        n = L.pjg_results_warning_count(self.handle)
        s = np.zeros(n, np.int32)
        b = np.zeros(n, np.int64)
        _check(L.pjg_results_warnings(self.handle, s.ctypes.data, b.ctypes.data), "pjg_results_warnings")
        return s, b

    def warnings_by_structure(self, n_structures: int):
        s, b = self.warnings()
        out = [[] for _ in range(n_structures)]
        for si, bi in zip(s, b):
            out[int(si)].append(int(bi))
        return out

    def stats(self) -> dict:
        st = Stats()
        _check(_lib.pjg_results_stats(self.handle, C.byref(st)), "pjg_results_stats")
        return st.as_dict()


def query(templates: Templates, structures: Structures, params: QueryParams) -> Result:
    L = _ready()
    h = C.c_void_p()
    _check(L.pjg_query(templates.handle, structures.handle, C.byref(params), C.byref(h)), "pjg_query")
    return Result(h)


def set_tuning(tuning: dict | None):
    """Set the process-wide execution tuning (``None``: the defaults)."""
    L = _ready()
    if tuning is None:
        _check(L.pjg_set_tuning(None), "pjg_set_tuning")
        return
    t = Tuning(**{k: int(v) for k, v in tuning.items() if k in dict(Tuning._fields_)})
    _check(L.pjg_set_tuning(C.byref(t)), "pjg_set_tuning")


def get_tuning() -> dict:
    L = _ready()
    t = Tuning()
    _check(L.pjg_get_tuning(C.byref(t)), "pjg_get_tuning")
    return t.as_dict()


def device_name() -> str:
    L = _ready()
    buf = C.create_string_buffer(256)
    _check(L.pjg_device_name(buf, 256), "pjg_device_name")
    return buf.value.decode(errors="replace")


PDB_IGNORE_ENDMDL = 1
PDB_SKIP_HETATM = 2


def parse_pdb_records(data: bytes, flags: int, dtype):
    """Atom records of a PDB text by the library's native reader: (records,
    end offset), or None when the text needs the general reader (a record in
    a form the native reader does not take).  Host code: no device needed."""
    L = load()
    cap = data.count(b"\n") + 1
    records = np.empty(cap, dtype=dtype)
    n, end, stop = C.c_int64(), C.c_int64(), C.c_int64()
    st = L.pjg_parse_pdb(data, len(data), int(flags), records.ctypes.data, cap, C.byref(n), C.byref(end),
                         C.byref(stop))
    if st != PJG_OK:
        return None
    return records[: n.value], end.value
