"""PDB input/output for molecules, atoms and templates.

Mirrors ``src/pyjess/_io.py`` of the reference (``PDBMoleculeParser`` and
``PDBMoleculeWriter``, lines 52-103 and 257-321) and the fixed-column atom
record the reference parses in C (``Atom_parse``).  The column layout is the
PDB ATOM/HETATM record: serial 7-11, name 13-16, altLoc 17, resName 18-20,
chain 21-22 (two characters, as the reference stores ``chainID1`` and
``chainID2``), resSeq 23-26, iCode 27, x/y/z 31-54, occupancy 55-60,
tempFactor 61-66, segID 73-76, element 77-78, charge 79-80.
"""

from __future__ import annotations

import datetime
import io
import os
import typing
import warnings

import numpy as np

from ._records import ATOM_DTYPE, encode_token


class nullcontext:
    """A context manager returning its argument (for already-open files)."""

    def __init__(self, value):
        self.value = value

    def __enter__(self):
        return self.value

    def __exit__(self, *exc):
        return False


def _int_field(text: str, default: int = 0) -> int:
    text = text.strip()
    if not text:
        return default
    return int(text)


def _float_field(text: str, default: float = 0.0) -> float:
    text = text.strip()
    if not text:
        return default
    return float(text)


def parse_atom_line(line: str, row) -> None:
    """Fill a structured ``ATOM_DTYPE`` row from one ATOM/HETATM line."""
    if len(line) < 54:
        raise ValueError(f"Failed to parse atom: {line!r}")
    line = line.rstrip("\r\n").ljust(80)
    raw = line.encode("ascii")
    row["serial"] = _int_field(line[6:11])
    row["name"] = np.void(encode_token(raw[12:16], 4))
    row["altloc"] = raw[16]
    row["resname"] = np.void(encode_token(raw[17:20], 3) + b"\0")
    row["chain"] = np.void(raw[20:22])
    row["resseq"] = _int_field(line[22:26])
    row["icode"] = raw[26]
    row["x"] = (float(line[30:38]), float(line[38:46]), float(line[46:54]))
    row["occupancy"] = _float_field(line[54:60])
    row["temp_factor"] = _float_field(line[60:66])
    row["segid"] = np.void(encode_token(raw[72:76], 4))
    row["element"] = np.void(encode_token(raw[76:78], 2))
    charge = line[78:80].strip()
    value = 0
    if charge:
        try:
            if charge[-1] in "+-" and charge[:-1].isdigit():
                value = int(charge[:-1]) * (1 if charge[-1] == "+" else -1)
            else:
                value = int(charge)
        except ValueError:
            value = 0
    row["charge"] = value


def parse_pdb(file, *, ignore_endmdl=False, skip_hetatm=False):
    """Return (records, id, date, name) for a PDB text stream."""
    id_ = date = name = None
    lines = []
    for line in file:
        if line.startswith("HEADER"):
            if id_ is None:
                id_ = line[62:66].strip() or None
            if date is None:
                text = line[50:59].strip()
                if text:
                    date = datetime.datetime.strptime(text, "%d-%b-%y").date()
            if name is None:
                name = line[10:50].strip() or None
        elif line.startswith("ATOM"):
            lines.append(line)
        elif line.startswith("HETATM") and not skip_hetatm:
            lines.append(line)
        elif line.startswith("ENDMDL"):
            if not ignore_endmdl:
                break
        elif line.lower().startswith(("data_", "loop_")):
            raise ValueError("mmCIF data tags found, file is not in PDB format")
    records = np.zeros(len(lines), dtype=ATOM_DTYPE)
    for i, line in enumerate(lines):
        parse_atom_line(line, records[i])
    return records, id_, date, name


class PDBMoleculeParser:
    """Parse a molecule from PDB text (``_io.py:52-103`` of the reference)."""

    def __init__(self, id=None, date=None, name=None, ignore_endmdl=False, skip_hetatm=False):
        self.id = id
        self.date = date
        self.name = name
        self.ignore_endmdl = ignore_endmdl
        self.skip_hetatm = skip_hetatm

    def loads(self, text, molecule_type):
        return self.load(io.StringIO(text), molecule_type)

    def load(self, file, molecule_type):
        try:
            handle = open(file)
        except TypeError:
            handle = nullcontext(file)
        with handle as f:
            records, id_, date, name = parse_pdb(
                f, ignore_endmdl=self.ignore_endmdl, skip_hetatm=self.skip_hetatm
            )
        return molecule_type._from_records(
            records,
            id=self.id if self.id is not None else id_,
            date=self.date if self.date is not None else date,
            name=self.name if self.name is not None else name,
        )


class PDBMoleculeWriter:
    """Write a molecule as PDB text (``_io.py:257-321`` of the reference)."""

    def __init__(self, write_header: bool = True):
        self.write_header = write_header

    def dumps(self, molecule) -> str:
        f = io.StringIO()
        self.dump(f, molecule)
        return f.getvalue()

    def dump(self, file, molecule) -> None:
        try:
            handle = open(file, "w")
        except TypeError:
            handle = nullcontext(file)
        with handle as f:
            if self.write_header:
                name = molecule.name or ""
                if len(name) > 40:
                    warnings.warn(f"Truncating name too long for PDB: {name!r}", UserWarning, stacklevel=3)
                    name = name[:40]
                id_ = molecule.id or ""
                if len(id_) > 4:
                    warnings.warn(f"Truncating ID too long for PDB: {id_!r}", UserWarning, stacklevel=3)
                    id_ = id_[:4]
                date = "" if molecule.date is None else molecule.date.strftime("%d-%b-%y").upper()
                f.write(f"{'HEADER':<6}{'':4}{name:40}{date:9}{'':3}{id_:4}\n")
            for atom in molecule:
                atom.dump(f, format="pdb")
