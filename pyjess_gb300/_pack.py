"""Packing of templates and molecules into the flat arrays of the C ABI.

`PackedTemplates` and `PackedStructures` hold NumPy arrays laid out as
``pjg_template_set`` / ``pjg_structure_set`` in ``include/pjg.h`` expect them;
``.abi()`` returns the ctypes struct pointing into those arrays (the packed
object must stay alive while the struct is used).
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from ._abi import StructureSet, TemplateSet, ptr
import ctypes as C


@dataclass
class PackedTemplates:
    atom_offset: np.ndarray      # int32 [T+1]
    code: np.ndarray             # int32 [A]
    res_seq: np.ndarray          # int32 [A]
    chain: np.ndarray            # uint8 [A, 2]
    xyz: np.ndarray              # float64 [A, 3]
    dist_weight: np.ndarray      # float64 [A]
    name_offset: np.ndarray      # int32 [A+1]
    names: np.ndarray            # uint8 [*, 4]
    resname_offset: np.ndarray   # int32 [A+1]
    resnames: np.ndarray         # uint8 [*, 4]
    dim: np.ndarray              # int32 [T]

    @property
    def n_templates(self) -> int:
        return len(self.atom_offset) - 1

    def subset(self, indices) -> "PackedTemplates":
        """The templates at `indices`, repacked contiguously (in that order)."""
        indices = np.asarray(indices, dtype=np.int64)
        a_lo, a_hi = self.atom_offset[indices], self.atom_offset[indices + 1]
        atoms = (np.concatenate([np.arange(a, b) for a, b in zip(a_lo, a_hi)]).astype(np.int64)
                 if len(indices) else np.zeros(0, np.int64))

        def ragged(offsets, values):
            lo, hi = offsets[atoms], offsets[atoms + 1]
            off = np.zeros(len(atoms) + 1, np.int32)
            np.cumsum(hi - lo, out=off[1:])
            rows = (np.concatenate([np.arange(a, b) for a, b in zip(lo, hi)]).astype(np.int64)
                    if len(atoms) else np.zeros(0, np.int64))
            return off, np.ascontiguousarray(values[rows])

        name_off, names = ragged(self.name_offset, self.names)
        res_off, resnames = ragged(self.resname_offset, self.resnames)
        aoff = np.zeros(len(indices) + 1, np.int32)
        np.cumsum(a_hi - a_lo, out=aoff[1:])
        return PackedTemplates(
            atom_offset=aoff, code=np.ascontiguousarray(self.code[atoms]),
            res_seq=np.ascontiguousarray(self.res_seq[atoms]), chain=np.ascontiguousarray(self.chain[atoms]),
            xyz=np.ascontiguousarray(self.xyz[atoms]), dist_weight=np.ascontiguousarray(self.dist_weight[atoms]),
            name_offset=name_off, names=names, resname_offset=res_off, resnames=resnames,
            dim=np.ascontiguousarray(self.dim[indices]))

    def abi(self) -> TemplateSet:
        s = TemplateSet()
        s.n_templates = self.n_templates
        s.atom_offset = ptr(self.atom_offset, C.c_int32)
        s.code = ptr(self.code, C.c_int32)
        s.res_seq = ptr(self.res_seq, C.c_int32)
        s.chain = ptr(self.chain, C.c_uint8)
        s.xyz = ptr(self.xyz, C.c_double)
        s.dist_weight = ptr(self.dist_weight, C.c_double)
        s.name_offset = ptr(self.name_offset, C.c_int32)
        s.names = ptr(self.names, C.c_uint8)
        s.resname_offset = ptr(self.resname_offset, C.c_int32)
        s.resnames = ptr(self.resnames, C.c_uint8)
        s.dim = ptr(self.dim, C.c_int32)
        return s


@dataclass
class PackedStructures:
    atom_offset: np.ndarray      # int64 [S+1]
    xyz: np.ndarray              # float64 [N, 3]
    name: np.ndarray             # uint8 [N, 4]
    resname: np.ndarray          # uint8 [N, 4]
    chain: np.ndarray            # uint8 [N, 2]
    res_seq: np.ndarray          # int32 [N]
    serial: np.ndarray           # int32 [N]

    @property
    def n_structures(self) -> int:
        return len(self.atom_offset) - 1

    @property
    def n_atoms(self) -> int:
        return int(self.atom_offset[-1])

    def abi(self) -> StructureSet:
        s = StructureSet()
        s.n_structures = self.n_structures
        s.atom_offset = ptr(self.atom_offset, C.c_int64)
        s.xyz = ptr(self.xyz, C.c_double)
        s.name = ptr(self.name, C.c_uint8)
        s.resname = ptr(self.resname, C.c_uint8)
        s.chain = ptr(self.chain, C.c_uint8)
        s.res_seq = ptr(self.res_seq, C.c_int32)
        s.serial = ptr(self.serial, C.c_int32)
        return s

    def nbytes(self) -> int:
        return sum(getattr(self, f).nbytes for f in
                   ("atom_offset", "xyz", "name", "resname", "chain", "res_seq", "serial"))

    def subset(self, indices) -> "PackedStructures":
        """The structures at `indices`, repacked contiguously."""
        indices = np.asarray(indices, dtype=np.int64)
        lo = self.atom_offset[indices]
        hi = self.atom_offset[indices + 1]
        counts = hi - lo
        sel = np.concatenate([np.arange(a, b) for a, b in zip(lo, hi)]) if len(indices) else np.zeros(0, np.int64)
        off = np.zeros(len(indices) + 1, dtype=np.int64)
        np.cumsum(counts, out=off[1:])
        return PackedStructures(
            atom_offset=off,
            xyz=np.ascontiguousarray(self.xyz[sel]),
            name=np.ascontiguousarray(self.name[sel]),
            resname=np.ascontiguousarray(self.resname[sel]),
            chain=np.ascontiguousarray(self.chain[sel]),
            res_seq=np.ascontiguousarray(self.res_seq[sel]),
            serial=np.ascontiguousarray(self.serial[sel]),
        )


def _bytes_rows(values, width):
    if not values:
        return np.zeros((0, width), dtype=np.uint8)
    return np.frombuffer(b"".join(values), dtype=np.uint8).reshape(-1, width).copy()


def pack_templates(templates) -> PackedTemplates:
    """Pack `Template` objects (index order kept)."""
    atom_offset = [0]
    code, res_seq, chain, xyz, weight = [], [], [], [], []
    name_offset, names, resname_offset, resnames = [0], [], [0], []
    dim = []
    for tpl in templates:
        for a in tpl._atoms:
            code.append(a._code)
            res_seq.append(a._resseq)
            chain.append(a._chain)
            xyz.append(a._pos)
            weight.append(a._weight)
            names.extend(a._names)
            name_offset.append(len(names))
            resnames.extend(a._resnames)
            resname_offset.append(len(resnames))
        atom_offset.append(len(code))
        dim.append(tpl.dimension)
    return PackedTemplates(
        atom_offset=np.asarray(atom_offset, dtype=np.int32),
        code=np.asarray(code, dtype=np.int32),
        res_seq=np.asarray(res_seq, dtype=np.int32),
        chain=_bytes_rows(chain, 2),
        xyz=np.asarray(xyz, dtype=np.float64).reshape(-1, 3),
        dist_weight=np.asarray(weight, dtype=np.float64),
        name_offset=np.asarray(name_offset, dtype=np.int32),
        names=_bytes_rows(names, 4),
        resname_offset=np.asarray(resname_offset, dtype=np.int32),
        resnames=_bytes_rows(resnames, 4),
        dim=np.asarray(dim, dtype=np.int32),
    )


def pack_molecules(molecules) -> PackedStructures:
    """Pack `Molecule` objects (their record arrays) into one structure set."""
    molecules = list(molecules)
    counts = [len(m._atoms) for m in molecules]
    off = np.zeros(len(molecules) + 1, dtype=np.int64)
    np.cumsum(counts, out=off[1:])
    if molecules:
        recs = np.concatenate([m._atoms for m in molecules])
    else:
        from ._records import ATOM_DTYPE

        recs = np.zeros(0, dtype=ATOM_DTYPE)
    n = len(recs)
    return PackedStructures(
        atom_offset=off,
        xyz=np.ascontiguousarray(recs["x"], dtype=np.float64).reshape(n, 3),
        name=np.ascontiguousarray(recs["name"]).view(np.uint8).reshape(n, 4),
        resname=np.ascontiguousarray(recs["resname"]).view(np.uint8).reshape(n, 4),
        chain=np.ascontiguousarray(recs["chain"]).view(np.uint8).reshape(n, 2),
        res_seq=np.ascontiguousarray(recs["resseq"], dtype=np.int32),
        serial=np.ascontiguousarray(recs["serial"], dtype=np.int32),
    )
