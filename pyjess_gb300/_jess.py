"""Python API of the GB300 template matcher.

Mirrors the public classes of PyJess 0.10.1 (``src/pyjess/_jess.pyx``,
``src/pyjess/_jess.pyi``): `Mat4`, `Molecule`, `Atom`, `TemplateAtom`,
`Template`, `Query`, `Hit` and `Jess`, with the same constructor arguments,
properties, error behaviour and text formats.  The difference is underneath:
molecules and templates are stored as NumPy record arrays, and
`Jess.query` runs the whole search for a molecule on the GPU through the
C ABI of ``libpjg.so`` (``include/pjg.h``), then hands out the hits one by
one as the reference's iterator does.  `Jess.query_many` is an addition that
batches many molecules into one device query.
"""

from __future__ import annotations

import functools
import io
import math
import typing
import warnings
from datetime import date as _date

import numpy as np

from . import _records as R
from ._io import CIFMoleculeParser, PDBMoleculeParser, PDBMoleculeWriter, nullcontext

__all__ = ["Mat4", "Molecule", "Atom", "TemplateAtom", "Template", "Query", "Hit", "Jess"]

MATCH_MODES = frozenset(list(range(-1, 9)) + list(range(100, 108)))

# logE = logA + alpha * rmsd + beta * dim + ln(n) (TessTemplate_logE,
# patches/TessTemplate.c.patch:164-170).  logA = -8.5 is visible there; the
# values of alpha and beta are not, and were fitted to the log(E) column of
# the reference's golden output (all 156 hits of 1AMY+1.3.3.txt and the
# doctest hit of _jess.pyx:2651, every value reproduced to two decimals).
_LOGE_A = -8.5
_LOGE_ALPHA = 2.5
_LOGE_BETA = -0.7


# --- Mat4 -------------------------------------------------------------------


class Mat4:
    """A 4x4 matrix of double precision (``_jess.pyx:177-240``)."""

    __slots__ = ("_data",)

    def __init__(self, data):
        if len(data) != 4:
            raise ValueError("invalid dimensions")
        m = np.zeros((4, 4), dtype=np.float64)
        for i, row in enumerate(data):
            if len(row) != 4:
                raise ValueError("invalid dimensions")
            for j, x in enumerate(row):
                m[i, j] = x
        self._data = m

    @classmethod
    def _wrap(cls, array) -> "Mat4":
        m = cls.__new__(cls)
        m._data = np.ascontiguousarray(array, dtype=np.float64).reshape(4, 4)
        return m

    @property
    def shape(self):
        return (4, 4)

    def __array__(self, dtype=None, copy=None):
        return self._data if dtype is None else self._data.astype(dtype)

    def __getitem__(self, index):
        return self._data[index]

    def __matmul__(self, other):
        other = np.asarray(other, dtype=np.float64)
        if other.shape != (4, 4):
            raise ValueError(f"dimension error: expected shape (4, 4), got {tuple(other.shape)!r}")
        res = np.zeros((4, 4))
        for i in range(4):
            for j in range(4):
                acc = 0.0
                for k in range(4):
                    acc += self._data[i, k] * other[k, j]
                res[i, j] = acc
        return Mat4._wrap(res)

    def __reduce__(self):
        return type(self), (self._data.tolist(),)

    def __eq__(self, other):
        if not isinstance(other, Mat4):
            return NotImplemented
        return bool(np.array_equal(self._data, other._data))

    def __repr__(self):
        return f"Mat4({self._data.tolist()!r})"


def _matrix16(matrix) -> np.ndarray:
    m = np.asarray(matrix, dtype=np.float64)
    if m.shape != (4, 4):
        raise ValueError(f"dimension error: expected shape (4, 4), got {tuple(m.shape)!r}")
    return m


def _apply(mat: np.ndarray, xyz) -> tuple:
    # Atom._transform (_jess.pyx:1259-1273): x_i = sum_j M[i][j] * (x, 1)_j
    tmp = (float(xyz[0]), float(xyz[1]), float(xyz[2]), 1.0)
    out = []
    for i in range(3):
        acc = 0.0
        for j in range(4):
            acc += mat[i, j] * tmp[j]
        out.append(acc)
    return tuple(out)


# --- Atom -------------------------------------------------------------------


class Atom:
    """A single atom in a molecule (``_jess.pyx:909-1330``)."""

    __slots__ = ("_arr", "_i")

    @classmethod
    def load(cls, file):
        return cls.loads(file.read())

    @classmethod
    def loads(cls, text):
        if isinstance(text, (bytes, bytearray)):
            text = bytes(text).decode("ascii")
        arr = np.zeros(1, dtype=R.ATOM_DTYPE)
        try:
            from ._io import parse_atom_line

            parse_atom_line(text.splitlines()[0] if text else text, arr[0])
        except (ValueError, IndexError, UnicodeError) as err:
            raise ValueError(f"Failed to parse atom: {text!r}") from err
        atom = cls.__new__(cls)
        atom._arr = arr
        atom._i = 0
        return atom

    def __init__(
        self,
        *,
        serial: int,
        name: str,
        residue_name: str,
        chain_id: str,
        residue_number: int,
        x: float,
        y: float,
        z: float,
        occupancy: float = 0.0,
        temperature_factor: float = 0.0,
        altloc: str = " ",
        insertion_code: str = " ",
        segment: str = "",
        element: str = "",
        charge: int = 0,
    ):
        if len(name) > 4:
            raise ValueError(f"Invalid atom name: {name!r}")
        if len(residue_name) > 3:
            raise ValueError(f"Invalid residue name: {residue_name!r}")
        if len(segment) > 4:
            raise ValueError(f"Invalid segment: {segment!r}")
        if len(element) > 2:
            raise ValueError(f"Invalid element: {element!r}")
        if len(chain_id) > 2:
            raise ValueError(f"Invalid chain ID: {chain_id!r}")
        arr = np.zeros(1, dtype=R.ATOM_DTYPE)
        row = arr[0]
        row["serial"] = serial
        row["altloc"] = ord(altloc)
        row["resseq"] = residue_number
        row["icode"] = ord(insertion_code)
        row["x"] = (x, y, z)
        row["occupancy"] = occupancy
        row["temp_factor"] = temperature_factor
        row["charge"] = charge
        row["resname"] = np.void(R.encode_token(residue_name.encode("ascii"), 3) + b"\0")
        row["segid"] = np.void(R.encode_token(segment.encode("ascii"), 4))
        row["element"] = np.void(R.encode_token(element.encode("ascii").rjust(2, b"\0"), 2))
        row["chain"] = np.void(R.encode_chain(chain_id))
        row["name"] = np.void(R.encode_atom_name(name))
        self._arr = arr
        self._i = 0

    @classmethod
    def _view(cls, arr, i):
        atom = cls.__new__(cls)
        atom._arr = arr
        atom._i = i
        return atom

    @property
    def _row(self):
        return self._arr[self._i]

    def _raw(self, field) -> bytes:
        return R.void_bytes(self._arr[field][self._i])

    def _state(self) -> dict:
        return {
            "serial": self.serial,
            "name": self.name,
            "altloc": self.altloc,
            "residue_name": self.residue_name,
            "chain_id": self.chain_id,
            "residue_number": self.residue_number,
            "insertion_code": self.insertion_code,
            "x": self.x,
            "y": self.y,
            "z": self.z,
            "temperature_factor": self.temperature_factor,
            "occupancy": self.occupancy,
            "segment": self.segment,
            "element": self.element,
            "charge": self.charge,
        }

    def __reduce__(self):
        return functools.partial(type(self), **self._state()), ()

    def __repr__(self):
        args = ", ".join(f"{k}={v!r}" for k, v in self._state().items() if v is not None)
        return f"{type(self).__name__}({args})"

    def __eq__(self, other):
        if not isinstance(other, Atom):
            return NotImplemented
        return self._state() == other._state()

    def __hash__(self):
        return hash(tuple(self._state().values()))

    def __copy__(self):
        return self.copy()

    def __sizeof__(self):
        return object.__sizeof__(self) + R.ATOM_DTYPE.itemsize

    @property
    def serial(self) -> int:
        return int(self._arr["serial"][self._i])

    @property
    def altloc(self) -> str:
        return chr(self._arr["altloc"][self._i])

    @property
    def name(self) -> str:
        return self._raw("name")[:4].decode("ascii").strip("_")

    @property
    def residue_name(self) -> str:
        return self._raw("resname")[:3].decode("ascii").strip("_")

    @property
    def residue_number(self) -> int:
        return int(self._arr["resseq"][self._i])

    @property
    def segment(self) -> str:
        return self._raw("segid")[:4].decode("ascii").strip("_")

    @property
    def element(self) -> str:
        return self._raw("element")[:2].decode("ascii").strip("_").strip("\0")

    @property
    def insertion_code(self) -> str:
        return chr(self._arr["icode"][self._i])

    @property
    def chain_id(self) -> str:
        return self._raw("chain").decode("ascii").strip()

    @property
    def occupancy(self) -> float:
        return float(self._arr["occupancy"][self._i])

    @property
    def temperature_factor(self) -> float:
        return float(self._arr["temp_factor"][self._i])

    @property
    def charge(self) -> int:
        return int(self._arr["charge"][self._i])

    @property
    def x(self) -> float:
        return float(self._arr["x"][self._i, 0])

    @property
    def y(self) -> float:
        return float(self._arr["x"][self._i, 1])

    @property
    def z(self) -> float:
        return float(self._arr["x"][self._i, 2])

    def copy(self) -> "Atom":
        return Atom._view(self._arr[self._i : self._i + 1].copy(), 0)

    def dumps(self, format: str = "pdb") -> str:
        f = io.StringIO()
        self.dump(f, format=format)
        return f.getvalue()

    def dump(self, file, format: str = "pdb") -> None:
        file.write(_format_atom(self._arr, self._i, None))

    def transform(self, matrix) -> "Atom":
        mat = _matrix16(matrix)
        copy = self.copy()
        copy._arr["x"][0] = _apply(mat, copy._arr["x"][0])
        return copy


def _format_atom(arr, i, xyz) -> str:
    row = arr[i]
    name = R.decode_token(R.void_bytes(row["name"])[:4])
    resname = R.decode_token(R.void_bytes(row["resname"])[:3])
    elem = R.decode_token(R.void_bytes(row["element"])[:2])
    chain = R.void_bytes(row["chain"]).decode("ascii")
    x = row["x"] if xyz is None else xyz
    return (
        f"ATOM  {int(row['serial']):5d}{name:>5s}{chr(row['altloc'])}{resname:<3s}"
        f"{chain[0]}{chain[1]}{int(row['resseq']):4d}{chr(row['icode']):<4s}"
        f"{x[0]:8.3f}{x[1]:8.3f}{x[2]:8.3f}{float(row['occupancy']):6.2f}"
        f"{float(row['temp_factor']):6.2f}          {elem:>2s}\n"
    )


# --- Molecule -----------------------------------------------------------------


class Molecule:
    """A molecule structure, as a sequence of `Atom` objects (``_jess.pyx:243-907``)."""

    __slots__ = ("_atoms", "_id", "_date", "_name", "_packed", "__weakref__")

    @classmethod
    def loads(cls, text, format="pdb", *, id=None, date=None, name=None,
              ignore_endmdl=False, use_author=False, skip_hetatm=False):
        return cls.load(io.StringIO(text), format=format, id=id, date=date, name=name,
                        ignore_endmdl=ignore_endmdl, use_author=use_author, skip_hetatm=skip_hetatm)

    @classmethod
    def load(cls, file, format="detect", *, id=None, date=None, name=None,
             ignore_endmdl=False, use_author=False, skip_hetatm=False):
        if format not in ("detect", "pdb", "cif"):
            raise ValueError(f"invalid value for `format` argument: {format!r}")
        if format == "detect":
            # mmCIF when the first line after leading '#' comment lines
            # starts a data block or a loop (``_jess.pyx:407-434``)
            if hasattr(file, "read"):
                text = file.read()
            else:
                with open(file) as f:
                    text = f.read()
            first = next((line for line in text.splitlines() if not line.startswith("#")), "")
            format = "cif" if first.startswith(("data_", "loop_")) else "pdb"
            file = io.StringIO(text)
        if format == "cif":
            parser = CIFMoleculeParser(id=id, date=date, name=name, use_author=use_author,
                                       skip_hetatm=skip_hetatm, ignore_endmdl=ignore_endmdl)
        else:
            parser = PDBMoleculeParser(id=id, date=date, name=name, ignore_endmdl=ignore_endmdl,
                                       skip_hetatm=skip_hetatm)
        return parser.load(file, molecule_type=cls)

    @classmethod
    def from_biopython(cls, structure, id=None, date=None, name=None):
        atoms = []
        for c in structure.get_chains():
            for r in c.get_residues():
                _, residue_number, insertion_code = r.id
                for a in r.get_atoms():
                    coord = a.get_coord()
                    atoms.append(Atom(
                        name=a.fullname, x=coord[0], y=coord[1], z=coord[2], altloc=a.altloc,
                        charge=a.pqr_charge or 0, occupancy=a.occupancy, serial=a.serial_number,
                        residue_name=r.resname, residue_number=residue_number, segment=r.segid,
                        insertion_code=insertion_code, chain_id=c.id, temperature_factor=a.bfactor,
                        element=a.element,
                    ))
        return cls(atoms, id=structure.id if id is None else id, date=date, name=name)

    @classmethod
    def from_gemmi(cls, model, id=None, date=None, name=None):
        atoms = []
        for cra in model.all():
            a, r, c = cra.atom, cra.residue, cra.chain
            atoms.append(Atom(
                name=a.padded_name(), x=a.pos[0], y=a.pos[1], z=a.pos[2],
                altloc=" " if a.altloc == "\0" else a.altloc, charge=a.charge,
                element=a.element.name.upper(), occupancy=a.occ, temperature_factor=a.b_iso,
                serial=a.serial, segment=r.segment, residue_name=r.name,
                residue_number=r.seqid.num, chain_id=c.name, insertion_code=r.seqid.icode,
            ))
        return cls(atoms, id=id, date=date, name=name)

    @classmethod
    def from_biotite(cls, atom_array, id=None, date=None, name=None):
        atoms = []
        for a in atom_array:
            atoms.append(Atom(
                name=str(a.atom_name), x=a.coord[0], y=a.coord[1], z=a.coord[2],
                altloc=str(getattr(a, "altloc", " ")), charge=getattr(a, "charge", 0),
                element=str(a.element), occupancy=getattr(a, "occupancy", 1.0),
                temperature_factor=a.b_factor, serial=a.atom_id,
                segment=str(getattr(a, "segment", "")), residue_name=str(a.res_name),
                residue_number=a.res_id, chain_id=str(a.chain_id),
                insertion_code=str(a.ins_code).ljust(1),
            ))
        return cls(atoms=atoms, id=id, date=date, name=name)

    def __init__(self, atoms=(), id=None, date=None, name=None):
        if date is not None and not isinstance(date, _date):
            raise TypeError(f"expected datetime.date or None, found {type(date).__name__} ")
        atoms = list(atoms)
        arr = np.zeros(len(atoms), dtype=R.ATOM_DTYPE)
        for i, atom in enumerate(atoms):
            arr[i] = atom._arr[atom._i]
        self._atoms = arr
        self._id = id
        self._date = date
        self._name = name
        self._packed = None

    @classmethod
    def _from_records(cls, records, id=None, date=None, name=None):
        mol = cls.__new__(cls)
        mol._atoms = np.ascontiguousarray(records, dtype=R.ATOM_DTYPE)
        mol._id = id
        mol._date = date
        mol._name = name
        mol._packed = None
        return mol

    def __len__(self):
        return len(self._atoms)

    def __getitem__(self, index):
        if isinstance(index, slice):
            return type(self)._from_records(self._atoms[index].copy(), id=self.id, date=self.date,
                                            name=self.name)
        index = int(index)
        n = len(self._atoms)
        if index < 0:
            index += n
        if index < 0 or index >= n:
            raise IndexError(index)
        return Atom._view(self._atoms, index)

    def __iter__(self):
        for i in range(len(self._atoms)):
            yield Atom._view(self._atoms, i)

    def __copy__(self):
        return self.copy()

    def __eq__(self, other):
        if not isinstance(other, Molecule):
            return NotImplemented
        if self._id != other._id or len(self) != len(other):
            return False
        return all(x == y for x, y in zip(self, other))

    def __hash__(self):
        return hash((self._id, *(hash(x) for x in self)))

    def __reduce__(self):
        return functools.partial(type(self), list(self), id=self.id, name=self.name, date=self.date), ()

    def __sizeof__(self):
        return object.__sizeof__(self) + self._atoms.nbytes

    @property
    def id(self):
        return self._id

    @property
    def date(self):
        return self._date

    @property
    def name(self):
        return self._name

    def conserved(self, cutoff: float = 0.0) -> "Molecule":
        if cutoff <= 0.0:
            return self.copy()
        keep = self._atoms["temp_factor"] >= cutoff
        return type(self)._from_records(self._atoms[keep].copy(), id=self.id, date=self.date,
                                        name=self.name)

    def copy(self) -> "Molecule":
        return type(self)._from_records(self._atoms.copy(), id=self._id, date=self._date,
                                        name=self._name)

    def dumps(self, format="pdb", write_header=True) -> str:
        if format != "pdb":
            raise ValueError(f"invalid value for `format` argument: {format!r}")
        return PDBMoleculeWriter(write_header=write_header).dumps(self)

    def dump(self, file, format="pdb", write_header=True) -> None:
        if format != "pdb":
            raise ValueError(f"invalid value for `format` argument: {format!r}")
        PDBMoleculeWriter(write_header=write_header).dump(file, self)

    def transform(self, matrix) -> "Molecule":
        mat = _matrix16(matrix)
        copy = self.copy()
        xyz = copy._atoms["x"]
        out = np.empty_like(xyz)
        for i in range(3):
            acc = np.zeros(len(xyz))
            for j in range(3):
                acc = acc + mat[i, j] * xyz[:, j]
            out[:, i] = acc + mat[i, 3]
        copy._atoms["x"] = out
        return copy


# --- TemplateAtom ---------------------------------------------------------------


class TemplateAtom:
    """A single template atom (``_jess.pyx:1332-1748``)."""

    __slots__ = ("_code", "_resseq", "_chain", "_pos", "_weight", "_names", "_resnames")

    @classmethod
    def load(cls, file):
        try:
            handle = open(file)
        except TypeError:
            handle = nullcontext(file)
        with handle as f:
            return cls.loads(f.read())

    @classmethod
    def loads(cls, text):
        """Parse one template line.

        The template line is a PDB ATOM record whose serial field holds the
        match mode; extra residue names are one-letter codes in columns 56-61
        and the distance weight follows from column 62 (the layout
        ``TemplateAtom.dump`` writes, ``_jess.pyx:1652-1689``).
        """
        if isinstance(text, (bytes, bytearray)):
            text = bytes(text).decode("ascii")
        line = text.splitlines()[0] if text else ""
        try:
            if not line.startswith(("ATOM", "HETATM")) or len(line) < 54:
                raise ValueError
            code = int(line[6:11])
            raw = line.encode("ascii")
            name = R.encode_token(raw[12:16], 4)
            resnames = [R.encode_token(raw[17:20], 3) + b"\0"]
            chain = line[20:22].encode("ascii")
            resseq = int(line[22:26])
            pos = (float(line[30:38]), float(line[38:46]), float(line[46:54]))
            for ch in line[55:61]:
                if ch == " ":
                    continue
                three = R.RESIDUE_CODES.get(ch)
                if three is None:
                    raise ValueError
                resnames.append(three.encode("ascii") + b"\0")
            rest = line[61:].strip()
            weight = float(rest.split()[0]) if rest else 0.0
        except (ValueError, IndexError, UnicodeError) as err:
            raise ValueError(f"Failed to parse template atom: {text!r}") from err
        if code not in MATCH_MODES:
            raise ValueError(f"Invalid match mode: {code!r}")
        atom = cls.__new__(cls)
        atom._code = code
        atom._resseq = resseq
        atom._chain = chain
        atom._pos = pos
        atom._weight = weight
        atom._names = (name,)
        atom._resnames = tuple(resnames)
        return atom

    def __init__(self, *, chain_id, residue_number, x, y, z, residue_names, atom_names,
                 distance_weight=0.0, match_mode=0):
        if match_mode not in MATCH_MODES:
            raise ValueError(f"Invalid match mode: {match_mode!r}")
        if len(chain_id) > 2:
            raise ValueError(f"Invalid chain ID: {chain_id!r}")
        self._code = int(match_mode)
        self._resseq = int(residue_number)
        self._chain = R.encode_chain(chain_id)
        self._pos = (float(x), float(y), float(z))
        self._weight = float(distance_weight)
        self._names = tuple(R.encode_atom_name(n) for n in atom_names)
        self._resnames = tuple(R.encode_residue_name(n) for n in residue_names)

    def _state(self) -> dict:
        return {
            "chain_id": self.chain_id,
            "residue_number": self.residue_number,
            "x": self.x,
            "y": self.y,
            "z": self.z,
            "residue_names": self.residue_names,
            "atom_names": self.atom_names,
            "distance_weight": self.distance_weight,
            "match_mode": self.match_mode,
        }

    def __repr__(self):
        return f"{type(self).__name__}({', '.join(f'{k}={v!r}' for k, v in self._state().items())})"

    def __copy__(self):
        return self.copy()

    def __eq__(self, other):
        if not isinstance(other, TemplateAtom):
            return NotImplemented
        return self._state() == other._state()

    def __hash__(self):
        return hash(tuple(self._state().values()))

    def __reduce__(self):
        return functools.partial(type(self), **self._state()), ()

    def __sizeof__(self):
        return object.__sizeof__(self) + 5 * len(self._names) + 4 * len(self._resnames) + 64

    @property
    def match_mode(self) -> int:
        return self._code

    @property
    def residue_number(self) -> int:
        return self._resseq

    @property
    def chain_id(self) -> str:
        c1, c2 = chr(self._chain[0]), chr(self._chain[1])
        if c1 == " ":
            return c2
        return (c1 + c2).strip()

    @property
    def x(self) -> float:
        return self._pos[0]

    @property
    def y(self) -> float:
        return self._pos[1]

    @property
    def z(self) -> float:
        return self._pos[2]

    @property
    def atom_names(self):
        return tuple(n.split(b"\0")[0].replace(b"_", b"").decode() for n in self._names)

    @property
    def residue_names(self):
        return tuple(n.split(b"\0")[0].replace(b"_", b"").decode() for n in self._resnames)

    @property
    def distance_weight(self) -> float:
        return self._weight

    def copy(self) -> "TemplateAtom":
        atom = TemplateAtom.__new__(TemplateAtom)
        for slot in TemplateAtom.__slots__:
            setattr(atom, slot, getattr(self, slot))
        return atom

    def dumps(self) -> str:
        f = io.StringIO()
        self.dump(f)
        return f.getvalue()

    def dump(self, file) -> None:
        name = R.decode_token(self._names[0][:4]) if self._names else "    "
        resname = R.decode_token(self._resnames[0][:3]) if self._resnames else "   "
        text = (
            f"ATOM  {self._code:5d} {name:>4s} {resname:>3s}{chr(self._chain[0])}{chr(self._chain[1])}"
            f"{self._resseq:4d}    {self._pos[0]:8.3f}{self._pos[1]:8.3f}{self._pos[2]:8.3f}"
        )
        extra = [" "] * 7
        for k in range(1, len(self._resnames)):
            if k < 7:
                three = self._resnames[k][:3].decode("ascii")
                extra[k] = R.RESIDUE_LETTERS.get(three, "X")
        text += "".join(extra) + f"{self._weight:4.2f}"
        file.write(text)

    def transform(self, matrix) -> "TemplateAtom":
        mat = _matrix16(matrix)
        copy = self.copy()
        copy._pos = _apply(mat, self._pos)
        return copy


# --- Template -----------------------------------------------------------------


class Template:
    """A template, as a sequence of `TemplateAtom` objects (``_jess.pyx:1751-2088``)."""

    __slots__ = ("_atoms", "_id", "_dim", "__weakref__")

    @classmethod
    def loads(cls, text, id=None):
        return cls.load(io.StringIO(text), id=id)

    @classmethod
    def load(cls, file, id=None):
        atoms = []
        try:
            handle = open(file)
        except TypeError:
            handle = nullcontext(file)
        with handle as f:
            for line in f:
                if line.startswith("ATOM"):
                    atoms.append(TemplateAtom.loads(line))
                elif id is None and line.startswith("REMARK PDB_ID"):
                    id = line.split(" ", maxsplit=2)[2].strip()
        return cls(atoms, id=id)

    def __init__(self, atoms=(), id=None):
        self._atoms = tuple(a.copy() for a in atoms)
        self._id = id
        # dimension: distinct (resSeq, chainID1, chainID2) (_jess.pyx:1903-1912)
        self._dim = len({(a._resseq, a._chain[0], a._chain[1]) for a in self._atoms})

    def __len__(self):
        return len(self._atoms)

    def __getitem__(self, index):
        if isinstance(index, slice):
            return type(self)(self._atoms[index], id=self.id)
        index = int(index)
        n = len(self._atoms)
        if index < 0:
            index += n
        if index < 0 or index >= n:
            raise IndexError(index)
        return self._atoms[index]

    def __iter__(self):
        return iter(self._atoms)

    def __copy__(self):
        return self.copy()

    def __eq__(self, other):
        if not isinstance(other, Template):
            return NotImplemented
        return (self.id == other.id and self.dimension == other.dimension
                and len(self) == len(other) and all(x == y for x, y in zip(self, other)))

    def __hash__(self):
        return hash((self.id, *(hash(x) for x in self)))

    def __reduce__(self):
        return type(self), (list(self), self.id)

    def __sizeof__(self):
        n = len(self._atoms)
        return object.__sizeof__(self) + n * n * 8 + sum(a.__sizeof__() for a in self._atoms)

    @property
    def id(self):
        return self._id

    @property
    def dimension(self) -> int:
        return self._dim

    def copy(self) -> "Template":
        tpl = type(self).__new__(type(self))
        tpl._atoms = tuple(a.copy() for a in self._atoms)
        tpl._id = self._id
        tpl._dim = self._dim
        return tpl

    def dumps(self) -> str:
        f = io.StringIO()
        self.dump(f)
        return f.getvalue()

    def dump(self, file, write_id=True) -> None:
        if write_id and self.id is not None:
            file.write(f"REMARK PDB_ID {self.id}\n")
        for atom in self._atoms:
            atom.dump(file)
            file.write("\n")

    def transform(self, matrix) -> "Template":
        mat = _matrix16(matrix)
        tpl = self.copy()
        tpl._atoms = tuple(a.transform(mat) for a in self._atoms)
        return tpl


# --- Hit ----------------------------------------------------------------------


class Hit:
    """A hit between a query molecule and a template (``_jess.pyx:2286-2621``)."""

    __slots__ = ("rmsd", "_rotation", "_centre", "_atoms", "_template", "_molecule")

    def __getstate__(self):
        return {
            "rotation": list(self._rotation),
            "centre": [list(self._centre[0]), list(self._centre[1])],
            "atoms": self.atoms(transform=False),
            "rmsd": self.rmsd,
            "template": self.template(transform=False),
            "molecule": self.molecule(transform=False),
        }

    def __setstate__(self, state):
        self.rmsd = state["rmsd"]
        self._template = state["template"]
        self._molecule = state["molecule"]
        self._rotation = np.array(state["rotation"], dtype=np.float64)
        self._centre = np.array(state["centre"], dtype=np.float64).reshape(2, 3)
        count = len(self._template)
        if len(state["atoms"]) != count:
            raise ValueError(f"unexpected number of atoms: {len(state['atoms'])!r} (expected {count!r})")
        arr = np.zeros(count, dtype=R.ATOM_DTYPE)
        for i, atom in enumerate(state["atoms"]):
            arr[i] = atom._arr[atom._i]
        self._atoms = arr

    def __reduce__(self):
        return (_new_hit, (), self.__getstate__())

    @property
    def transformation(self) -> Mat4:
        M, c, v = self._rotation, self._centre[0], self._centre[1]
        Mc = np.eye(4)
        Mc[0:3, 3] = -c
        Mr = np.eye(4)
        Mr[0:3, 0:3] = np.asarray(M).reshape(3, 3)
        Mv = np.eye(4)
        Mv[0:3, 3] = v
        return Mat4._wrap(Mv) @ Mr @ Mc

    @property
    def inverse_transformation(self) -> Mat4:
        M, c, v = self._rotation, self._centre[0], self._centre[1]
        Mv = np.eye(4)
        Mv[0:3, 3] = -v
        Mr = np.eye(4)
        Mr[0:3, 0:3] = np.asarray(M).reshape(3, 3).T
        Mc = np.eye(4)
        Mc[0:3, 3] = c
        return Mat4._wrap(Mc) @ Mr @ Mv

    @property
    def determinant(self) -> float:
        p = self._rotation
        det = 0.0
        det += p[0] * (p[4] * p[8] - p[5] * p[7])
        det -= p[1] * (p[3] * p[8] - p[5] * p[6])
        det += p[2] * (p[3] * p[7] - p[4] * p[6])
        return float(det)

    @property
    def log_evalue(self) -> float:
        n = len(self._molecule)
        return _LOGE_A + _LOGE_ALPHA * self.rmsd + _LOGE_BETA * float(self._template.dimension) + math.log(n)

    @property
    def evalue(self) -> float:
        return math.exp(self.log_evalue)

    def atoms(self, transform: bool = True) -> list:
        out = []
        trans = np.asarray(self.transformation) if transform else None
        for k in range(len(self._atoms)):
            atom = Atom._view(self._atoms, k)
            if transform:
                atom = atom.transform(trans)
            out.append(atom)
        return out

    def molecule(self, transform: bool = False) -> Molecule:
        if not transform:
            return self._molecule
        return self._molecule.transform(self.transformation)

    def template(self, transform: bool = False) -> Template:
        if not transform:
            return self._template
        return self._template.transform(self.inverse_transformation)

    def dumps(self, format="pdb", transform=True) -> str:
        f = io.StringIO()
        self.dump(f, format=format, transform=transform)
        return f.getvalue()

    def dump(self, file, format="pdb", transform=True) -> None:
        if self._template.id is None:
            raise RuntimeError("cannot dump `Hit` where `self.template.id` is `None`")
        if self._molecule.id is None:
            raise RuntimeError("cannot dump `Hit` where `self.molecule.id` is `None`")
        file.write("REMARK ")
        file.write(self._molecule.id)
        file.write(f" {self.rmsd:5.3f} ")
        file.write(self._template.id)
        file.write(f" Det={self.determinant:4,.1f} log(E)~ {self.log_evalue:4.2f}\n")
        trans = np.asarray(self.transformation)
        for k in range(len(self._atoms)):
            xyz = _apply(trans, self._atoms["x"][k]) if transform else self._atoms["x"][k]
            file.write(_format_atom(self._atoms, k, xyz))
        file.write("ENDMDL\n")


def _new_hit():
    return Hit.__new__(Hit)


# --- Query --------------------------------------------------------------------


class Query:
    """An iterator over the hits of a molecule (``_jess.pyx:2090-2283``).

    The device search for the molecule runs at the first call to `next`;
    the hits come out in the reference's order, with the ``UserWarning`` of
    NaN rotations emitted at the same points of the iteration.
    """

    def __init__(self, jess, molecule, rmsd_threshold, distance_cutoff, max_dynamic_distance,
                 max_candidates, ignore_chain, best_match, reorder):
        self.jess = jess
        self.molecule = molecule
        self.rmsd_threshold = float(rmsd_threshold)
        self.best_match = bool(best_match)
        self.max_candidates = max_candidates
        self.ignore_chain = ignore_chain
        self._distance_cutoff = float(distance_cutoff)
        self._max_dynamic_distance = float(max_dynamic_distance)
        self._reorder = bool(reorder)
        self._hits = None
        self._warnings = None
        self._pos = 0

    def __iter__(self):
        return self

    @property
    def ignore_chain(self):
        return (None, "residues", "atoms")[self._ignore_chain]

    @ignore_chain.setter
    def ignore_chain(self, value):
        if value is None:
            self._ignore_chain = 0
        elif value == "residues":
            self._ignore_chain = 1
        elif value == "atoms":
            self._ignore_chain = 2
        else:
            raise ValueError(f"invalid value for `ignore_chain`: {value!r}")

    @property
    def max_candidates(self):
        return None if self._max_candidates == -1 else self._max_candidates

    @max_candidates.setter
    def max_candidates(self, value):
        if value is None:
            self._max_candidates = -1
        elif value >= 0:
            self._max_candidates = int(value)
        else:
            raise ValueError(f"invalid value for `max_candidates` argument: {value!r}")

    def _params(self, mode):
        from ._native import QueryParams

        return QueryParams(
            rmsd_threshold=self.rmsd_threshold,
            distance_cutoff=self._distance_cutoff,
            max_dynamic_distance=self._max_dynamic_distance,
            max_candidates=self._max_candidates,
            ignore_chain=self._ignore_chain,
            best_match=int(self.best_match),
            reorder=int(self._reorder),
            mode=mode,
        )

    def _run(self):
        from . import _native

        result = _native.query(self.jess._device_templates(), _native.structures_for([self.molecule]),
                               self._params(_native.MODE_BATCHED_FP32))
        self._hits = _materialize(result, self.jess, [self.molecule])[0]
        self._warnings = result.warnings_by_structure(1)[0]

    def __next__(self):
        if self._hits is None:
            self._run()
        for _ in range(self._warnings.count(self._pos)):
            warnings.warn("Jess returned a superposition matrix with NaN values", UserWarning, 2)
        self._warnings = [w for w in self._warnings if w != self._pos]
        if self._pos >= len(self._hits):
            raise StopIteration
        hit = self._hits[self._pos]
        self._pos += 1
        return hit


def _materialize(result, jess, molecules):
    """Build `Hit` objects per molecule from a device result."""
    per = [[] for _ in molecules]
    data = result.arrays()
    for i in range(data["count"]):
        s = int(data["structure"][i])
        t = int(data["template"][i])
        mol = molecules[s]
        a0, a1 = int(data["atom_offset"][i]), int(data["atom_offset"][i + 1])
        hit = Hit.__new__(Hit)
        hit.rmsd = float(data["rmsd"][i])
        hit._rotation = data["rotation"][i].copy()
        hit._centre = data["centres"][i].reshape(2, 3).copy()
        hit._atoms = mol._atoms[data["atoms"][a0:a1]].copy()
        hit._template = jess._templates[t]
        hit._molecule = mol
        per[s].append(hit)
    return per


class HitArrays:
    """Hits of a batched query as NumPy columns, without `Hit` objects.

    An addition (PyJess materialises every hit as an object): for queries
    with millions of hits, building Python objects costs more than the
    search.  Row ``i`` is the hit `Jess.query_many` would return at the same
    position; rows are grouped by molecule (``molecule``, ascending) and, per
    molecule, in ``query()`` order.

    Attributes:
        molecule (`numpy.ndarray` of int32): index of the hit's molecule.
        template (`numpy.ndarray` of int32): index of the template in `Jess`.
        ordinal (`numpy.ndarray` of int64): position of the hit in its
            (molecule, template) candidate stream.
        rmsd (`numpy.ndarray` of float64).
        rotation (`numpy.ndarray` of float64, shape (n, 3, 3)): maps molecule
            coordinates onto the template frame, about the centroids.
        centres (`numpy.ndarray` of float64, shape (n, 2, 3)): molecule and
            template centroids.
        atom_offset (`numpy.ndarray` of int64, n + 1): hit ``i``'s matched
            atoms are ``atoms[atom_offset[i]:atom_offset[i + 1]]``.
        atoms (`numpy.ndarray` of int32): molecule atom indices, in template
            atom order.
    """

    __slots__ = ("molecule", "template", "ordinal", "rmsd", "rotation", "centres", "atom_offset", "atoms",
                 "_jess", "_molecules", "_device")

    def __init__(self, data, jess, molecules, device=None):
        n = data["count"]
        self.molecule = data["structure"]
        self.template = data["template"]
        self.ordinal = data["ordinal"]
        self.rmsd = data["rmsd"]
        self.rotation = data["rotation"].reshape(n, 3, 3)
        self.centres = data["centres"].reshape(n, 2, 3)
        self.atom_offset = data["atom_offset"]
        self.atoms = data["atoms"]
        self._jess = jess
        self._molecules = molecules
        self._device = device  # (device result, device structures) of the query

    def superposed_atoms(self):
        """The matched atoms of every hit in its template's frame: an
        (atoms, 3) array aligned with `atoms` -- what ``Hit.atoms()`` gives
        hit by hit -- computed on the GPU from the query's device results."""
        if self._device is None:
            raise RuntimeError("the device results of this query are no longer held")
        result, structures = self._device
        return result.superposed(structures)

    def __len__(self):
        return len(self.rmsd)

    def molecule_offsets(self) -> np.ndarray:
        """Row offsets per molecule: the hits of molecule ``m`` are rows
        ``offsets[m]:offsets[m + 1]``."""
        return np.searchsorted(self.molecule, np.arange(len(self._molecules) + 1), side="left")

    def hit(self, i: int) -> "Hit":
        """Row ``i`` as a `Hit` object."""
        mol = self._molecules[int(self.molecule[i])]
        a0, a1 = int(self.atom_offset[i]), int(self.atom_offset[i + 1])
        hit = Hit.__new__(Hit)
        hit.rmsd = float(self.rmsd[i])
        hit._rotation = self.rotation[i].reshape(9).copy()
        hit._centre = self.centres[i].copy()
        hit._atoms = mol._atoms[self.atoms[a0:a1]].copy()
        hit._template = self._jess._templates[int(self.template[i])]
        hit._molecule = mol
        return hit


# --- Jess ---------------------------------------------------------------------


class Jess:
    """A handle to run template searches over a list of templates (``_jess.pyx:2623-2869``)."""

    def __init__(self, templates=()):
        self._templates = tuple(templates)
        for t in self._templates:
            if not isinstance(t, Template):
                raise TypeError(f"expected Template, found {type(t).__name__}")
        self._packed = None
        self._device = None

    def __len__(self):
        return len(self._templates)

    def __bool__(self):
        return len(self._templates) > 0

    def __getitem__(self, index):
        if isinstance(index, slice):
            return type(self)(self._templates[index])
        index = int(index)
        n = len(self._templates)
        if index < 0:
            index += n
        if index < 0 or index >= n:
            raise IndexError(index)
        return self._templates[index]

    def __copy__(self):
        return self.copy()

    def __reduce__(self):
        return type(self), (self._templates,)

    def __eq__(self, other):
        if not isinstance(other, Jess):
            return NotImplemented
        return self._templates == other._templates

    def __hash__(self):
        return hash((Jess, self._templates))

    def __sizeof__(self):
        return object.__sizeof__(self) + sum(t.__sizeof__() for t in self._templates)

    def copy(self) -> "Jess":
        return type(self)(self._templates)

    def _packed_templates(self):
        if self._packed is None:
            from ._pack import pack_templates

            self._packed = pack_templates(self._templates)
        return self._packed

    def _device_templates(self):
        if self._device is None:
            from . import _native

            self._device = _native.Templates(self._packed_templates())
        return self._device

    def query(self, molecule, rmsd_threshold, distance_cutoff, max_dynamic_distance, *,
              max_candidates=None, ignore_chain=None, best_match=False, reorder=True):
        if not isinstance(molecule, Molecule):
            raise TypeError(f"expected Molecule, found {type(molecule).__name__}")
        if ignore_chain is True:
            warnings.warn(
                "`ignore_chain` parameter expects string parameters to specificy the mode since "
                "PyJess v0.7.0. Use `ignore_chain='atoms'` instead of `ignore_chain=True`",
                DeprecationWarning, 2)
            ignore_chain = "atoms"
        elif ignore_chain is False:
            warnings.warn(
                "`ignore_chain` parameter expects string parameters to specificy the mode since "
                "PyJess v0.7.0. Use `ignore_chain=None` instead of `ignore_chain=False`",
                DeprecationWarning, 2)
            ignore_chain = None
        return Query(self, molecule, rmsd_threshold, distance_cutoff, max_dynamic_distance,
                     max_candidates, ignore_chain, best_match, reorder)

    def query_many(self, molecules, rmsd_threshold, distance_cutoff, max_dynamic_distance, *,
                   max_candidates=None, ignore_chain=None, best_match=False, reorder=True,
                   precision="fp32"):
        """Search many molecules in one batched device query.

        Returns one list of hits per molecule, each identical to
        ``list(self.query(molecule, ...))``.  ``precision`` selects the
        distance-test arithmetic: ``"fp32"`` (FP32 with a guard band and FP64
        recheck) or ``"fp64"``.
        """
        from . import _native

        molecules = list(molecules)
        q = Query(self, Molecule(), rmsd_threshold, distance_cutoff, max_dynamic_distance,
                  max_candidates, ignore_chain, best_match, reorder)
        mode = {"fp32": _native.MODE_BATCHED_FP32, "fp64": _native.MODE_BATCHED_FP64,
                "plain": _native.MODE_PLAIN_FP64}[precision]
        result = _native.query(self._device_templates(), _native.structures_for(molecules),
                               q._params(mode))
        per = _materialize(result, self, molecules)
        for s, ws in enumerate(result.warnings_by_structure(len(molecules))):
            for _ in ws:
                warnings.warn("Jess returned a superposition matrix with NaN values", UserWarning, 2)
        return per

    def query_arrays(self, molecules, rmsd_threshold, distance_cutoff, max_dynamic_distance, *,
                     max_candidates=None, ignore_chain=None, best_match=False, reorder=True,
                     precision="fp32") -> HitArrays:
        """`query_many` with the hits returned as NumPy columns (`HitArrays`)
        instead of `Hit` objects; the same search, hits and order."""
        from . import _native

        molecules = list(molecules)
        q = Query(self, Molecule(), rmsd_threshold, distance_cutoff, max_dynamic_distance,
                  max_candidates, ignore_chain, best_match, reorder)
        mode = {"fp32": _native.MODE_BATCHED_FP32, "fp64": _native.MODE_BATCHED_FP64,
                "plain": _native.MODE_PLAIN_FP64}[precision]
        structures = _native.structures_for(molecules)
        result = _native.query(self._device_templates(), structures, q._params(mode))
        for s, ws in enumerate(result.warnings_by_structure(len(molecules))):
            for _ in ws:
                warnings.warn("Jess returned a superposition matrix with NaN values", UserWarning, 2)
        return HitArrays(result.arrays(), self, molecules, device=(result, structures))
