"""Byte-level record layouts shared by the Python API, the C ABI and the oracle.

The reference stores an atom as a C struct (``Atom.h``: coordinates, occupancy,
serial, a 4-byte name, a 3-byte residue name, two chain characters, residue
number, ...).  Here a molecule is a NumPy structured array with one row per
atom; the columns that the matching path reads are exported as flat arrays
(`pack_structures`) and handed to the C ABI without per-atom Python objects.

Token encoding follows the reference's Cython layer
(``src/pyjess/_jess.pyx:128-135`` ``encode_token``): spaces and NUL bytes are
stored as ``'_'``; atom names shorter than 4 characters get a leading ``'_'``
(``_jess.pyx:1053-1056`` for atoms, ``:1484-1488`` for template atoms);
residue names are 3 characters followed by a NUL byte.
"""

from __future__ import annotations

import numpy as np

ATOM_DTYPE = np.dtype(
    [
        ("x", "<f8", (3,)),
        ("occupancy", "<f4"),
        ("temp_factor", "<f4"),
        ("serial", "<i4"),
        ("name", "V4"),
        ("altloc", "u1"),
        ("resname", "V4"),
        ("chain", "V2"),
        ("resseq", "<i4"),
        ("icode", "u1"),
        ("segid", "V4"),
        ("element", "V2"),
        ("charge", "i1"),
    ]
)


def encode_token(raw: bytes, n: int) -> bytes:
    """Pad/crop ``raw`` to ``n`` bytes, spaces and NULs become ``'_'``."""
    raw = raw[:n].ljust(n, b"\0")
    return bytes(0x5F if c in (0x20, 0) else c for c in raw)


def decode_token(raw: bytes) -> str:
    """Inverse of `encode_token` for display: ``'_'`` and NUL become spaces."""
    return bytes(0x20 if c in (0x5F, 0) else c for c in raw).decode("ascii")


def encode_atom_name(name) -> bytes:
    """Atom names: at most 4 characters, a leading ``'_'`` when shorter."""
    b = bytearray(name, "ascii") if isinstance(name, str) else bytearray(name)
    if len(b) > 4:
        raise ValueError(f"Invalid atom name: {name!r}")
    if len(b) < 4:
        b.insert(0, ord("_"))
    return encode_token(bytes(b), 4)


def encode_residue_name(name) -> bytes:
    """Residue names: 3 encoded characters and a NUL byte (4 bytes)."""
    b = name.encode("ascii") if isinstance(name, str) else bytes(name)
    if len(b) > 3:
        raise ValueError(f"Invalid residue name: {name!r}")
    return encode_token(b, 3) + b"\0"


def encode_chain(chain_id: str) -> bytes:
    """Two chain characters (``chainID1``, ``chainID2``) as in ``Atom.h``."""
    if len(chain_id) > 2:
        raise ValueError(f"Invalid chain ID: {chain_id!r}")
    if len(chain_id) == 2:
        return chain_id.encode("ascii")
    if len(chain_id) == 1:
        return b" " + chain_id.encode("ascii")
    return b" 0"


def void_bytes(v) -> bytes:
    return bytes(v.tobytes())


# one-letter residue codes accepted in the alternate-residue columns of
# template lines, with their three-letter names
RESIDUE_CODES = {
    "A": "ALA", "C": "CYS", "D": "ASP", "E": "GLU", "F": "PHE", "G": "GLY",
    "H": "HIS", "I": "ILE", "K": "LYS", "L": "LEU", "M": "MET", "N": "ASN",
    "P": "PRO", "O": "PYL", "Q": "GLN", "R": "ARG", "S": "SER", "T": "THR",
    "U": "SEC", "V": "VAL", "W": "TRP", "Y": "TYR", "X": "XXX",
}
# inverse table used when writing template lines (21 standard codes)
RESIDUE_LETTERS = {
    "ALA": "A", "CYS": "C", "ASP": "D", "GLU": "E", "PHE": "F", "GLY": "G",
    "HIS": "H", "ILE": "I", "LYS": "K", "LEU": "L", "MET": "M", "ASN": "N",
    "PRO": "P", "GLN": "Q", "ARG": "R", "SER": "S", "THR": "T", "VAL": "V",
    "TRP": "W", "TYR": "Y", "XXX": "X",
}
