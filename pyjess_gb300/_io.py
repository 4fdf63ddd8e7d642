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


def _header_fields(lines):
    """(id, date, name) from HEADER lines, as `parse_pdb` reads them."""
    id_ = date = name = None
    for line in lines:
        if id_ is None:
            id_ = line[62:66].strip() or None
        if date is None:
            text = line[50:59].strip()
            if text:
                date = datetime.datetime.strptime(text, "%d-%b-%y").date()
        if name is None:
            name = line[10:50].strip() or None
    return id_, date, name


def _header_lines(text: str, end: int):
    """The lines of text[:end] that start with HEADER."""
    starts = [0] if text.startswith("HEADER") and end > 0 else []
    i = text.find("\nHEADER", 0, end)
    while i >= 0:
        starts.append(i + 1)
        i = text.find("\nHEADER", i + 1, end)
    out = []
    for s in starts:
        e = text.find("\n", s)
        out.append(text[s:e if e >= 0 else len(text)])
    return out


def parse_pdb_text(text: str, *, ignore_endmdl=False, skip_hetatm=False):
    """`parse_pdb` over a whole text, the atom records read by the native
    reader of libpjg (one call, no per-atom Python work).  Texts it does not
    take (non-ASCII, unusual field forms, mmCIF) and machines without the
    library go through `parse_pdb`, which gives the same records."""
    if text.isascii():
        try:
            from . import _native

            flags = (_native.PDB_IGNORE_ENDMDL if ignore_endmdl else 0) | (_native.PDB_SKIP_HETATM if skip_hetatm
                                                                             else 0)
            fast = _native.parse_pdb_records(text.encode("ascii"), flags, ATOM_DTYPE)
        except (OSError, RuntimeError):
            fast = None
        if fast is not None:
            records, end = fast
            return (records, *_header_fields(_header_lines(text, end)))
    return parse_pdb(io.StringIO(text), ignore_endmdl=ignore_endmdl, skip_hetatm=skip_hetatm)


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
            text = f.read()
        if not isinstance(text, str):
            text = text.decode()
        records, id_, date, name = parse_pdb_text(
            text, ignore_endmdl=self.ignore_endmdl, skip_hetatm=self.skip_hetatm
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


# ---------------------------------------------------------------------------
# mmCIF input.  The reference reads mmCIF through the gemmi module
# (``CIFMoleculeParser``, ``src/pyjess/_io.py:106-233``), which is not
# available here; this is a reader of the CIF syntax the atom records need
# (data blocks, tag-value pairs, ``loop_`` tables, quoted and semicolon
# text values, comments) followed by the reference's column mapping.  Values
# are kept as raw tokens, quotes included, as gemmi's table rows are; the
# mapping strips them where the reference does.

_CIF_TOKEN = __import__("re").compile(
    r"""'(?:[^']|'(?=\S))*'(?=\s|$)|"(?:[^"]|"(?=\S))*"(?=\s|$)|#.*|\S+""")


class CIFBlock:
    """One ``data_`` block: single values by tag and ``loop_`` tables."""

    def __init__(self, name: str):
        self.name = name
        self.values: dict = {}
        self.loops: list = []  # (tags, rows)

    def find_value(self, tag: str):
        return self.values.get(tag.lower())

    def find(self, prefix: str, columns):
        """Rows of the columns `prefix + c` (a leading ``?`` marks an optional
        column): a list of rows (None for an absent optional column), or
        None when a required column is missing."""
        prefix = prefix.lower()
        names = [(c[1:] if c.startswith("?") else c, c.startswith("?")) for c in columns]
        for tags, rows in self.loops:
            pos = {t: i for i, t in enumerate(tags)}
            if not any(t.startswith(prefix) for t in tags):
                continue
            idx = []
            for c, optional in names:
                i = pos.get(prefix + c.lower())
                if i is None and not optional:
                    return None
                idx.append(i)
            return [[None if i is None else row[i] for i in idx] for row in rows]
        # a category written as single values is a one-row table
        row = []
        for c, optional in names:
            v = self.values.get(prefix + c.lower())
            if v is None and not optional:
                return None
            row.append(v)
        return [row]


def read_cif(text: str) -> typing.List[CIFBlock]:
    """The data blocks of a CIF text."""
    blocks: typing.List[CIFBlock] = []
    tokens: typing.List[str] = []
    lines = text.splitlines()
    i = 0
    while i < len(lines):
        line = lines[i]
        if line.startswith(";"):
            # text field: up to the next line starting with ';'
            body = [line[1:]]
            i += 1
            while i < len(lines) and not lines[i].startswith(";"):
                body.append(lines[i])
                i += 1
            tokens.append("\n".join(body).strip())
            i += 1
            continue
        for m in _CIF_TOKEN.finditer(line):
            tok = m.group(0)
            if tok.startswith("#"):
                break
            tokens.append(tok)
        i += 1

    block = None
    k = 0
    while k < len(tokens):
        tok = tokens[k]
        low = tok.lower()
        if low.startswith("data_"):
            block = CIFBlock(tok[5:])
            blocks.append(block)
            k += 1
        elif block is None:
            raise ValueError("CIF text without a data block")
        elif low == "loop_":
            k += 1
            tags = []
            while k < len(tokens) and tokens[k].startswith("_"):
                tags.append(tokens[k].lower())
                k += 1
            values = []
            while k < len(tokens) and not tokens[k].startswith("_") and \
                    tokens[k].lower() not in ("loop_",) and not tokens[k].lower().startswith("data_"):
                values.append(tokens[k])
                k += 1
            if tags:
                if len(values) % len(tags):
                    raise ValueError(f"loop of {tags[0]}: {len(values)} values for {len(tags)} columns")
                n = len(tags)
                block.loops.append((tags, [values[j:j + n] for j in range(0, len(values), n)]))
        elif tok.startswith("_"):
            if k + 1 >= len(tokens):
                raise ValueError(f"tag {tok} without a value")
            block.values[low] = tokens[k + 1]
            k += 2
        else:
            raise ValueError(f"unexpected CIF token {tok!r}")
    return blocks


class CIFMoleculeParser:
    """Parse a molecule from mmCIF text (``src/pyjess/_io.py:106-233``)."""

    _PRIMARY_COLUMNS = [
        "id", "type_symbol", "label_atom_id", "label_alt_id", "label_comp_id", "label_asym_id",
        "label_seq_id", "?pdbx_PDB_ins_code", "Cartn_x", "Cartn_y", "Cartn_z", "occupancy",
        "B_iso_or_equiv", "?pdbx_formal_charge", "?group_PDB", "pdbx_PDB_model_num",
    ]
    _AUTH_COLUMNS = [
        "id", "type_symbol", "auth_atom_id", "label_alt_id", "auth_comp_id", "auth_asym_id",
        "auth_seq_id", "?pdbx_PDB_ins_code", "Cartn_x", "Cartn_y", "Cartn_z", "occupancy",
        "B_iso_or_equiv", "?pdbx_formal_charge", "?group_PDB", "pdbx_PDB_model_num",
    ]

    def __init__(self, id=None, date=None, name=None, use_author=False, skip_hetatm=False,
                 ignore_endmdl=False):
        self.id = id
        self.date = date
        self.name = name
        self.use_author = use_author
        self.skip_hetatm = skip_hetatm
        self.ignore_endmdl = ignore_endmdl

    def _load_block(self, blocks, molecule_type):
        from ._jess import Atom

        if len(blocks) != 1:
            raise ValueError(f"expected one data block in the CIF text, found {len(blocks)}")
        block = blocks[0]
        table = block.find("_atom_site.", self._AUTH_COLUMNS if self.use_author else self._PRIMARY_COLUMNS)
        if not table:
            raise ValueError("missing columns in CIF files")
        atoms = []
        max_residue_number = 0
        for row in table:
            # column 15 is the model number: the first model only, unless
            # ENDMDL is ignored
            if not self.ignore_endmdl and row[15] != "1":
                break
            if row[14] != "ATOM" and (row[14] != "HETATM" or self.skip_hetatm):
                continue
            if row[6] == "." and row[14] == "HETATM":
                warnings.warn(
                    "HETATM line found without residue number. Consider parsing with use_author=True to "
                    "use author-defined residue numbers, or skip_hetatm=True to disable parsing of HETATM "
                    "altogether.", UserWarning, stacklevel=3)
                residue_number = max_residue_number
                max_residue_number += 1
            else:
                residue_number = int(row[6])
                max_residue_number = max(residue_number, max_residue_number)
            atoms.append(Atom(
                serial=int(row[0]),
                element=row[1],
                name=row[2].strip('"'),
                altloc=" " if row[3] == "." else row[3],
                residue_name=row[4],
                chain_id=row[5],
                residue_number=residue_number,
                insertion_code=" " if row[7] is None or row[7] == "?" else row[7],
                x=float(row[8]),
                y=float(row[9]),
                z=float(row[10]),
                occupancy=0.0 if row[11] == "." else float(row[11]),
                temperature_factor=0.0 if row[12] == "." else float(row[12]),
                charge=0 if row[13] is None or row[13] == "?" else int(row[13]),
            ))
        id_ = block.name if self.id is None else self.id
        entry_id = block.find_value("_entry.id")
        keywords = block.find_value("_struct_keywords.pdbx_keywords")
        title = block.find_value("_struct.title")
        name = keywords or title or entry_id
        name = name.strip("'") if name else None
        date = None
        revisions = block.find("_pdbx_audit_revision_history.", ["revision_date"])
        if revisions:
            # the earliest revision is the deposition
            date = min(datetime.datetime.strptime(r[0], "%Y-%m-%d") for r in revisions).date()
        return molecule_type(
            atoms,
            id=id_,
            date=self.date if self.date is not None else date,
            name=self.name if self.name is not None else name,
        )

    def loads(self, text, molecule_type):
        return self._load_block(read_cif(text), molecule_type)

    def load(self, file, molecule_type):
        if hasattr(file, "read"):
            return self.loads(file.read(), molecule_type)
        with open(file) as f:
            return self.loads(f.read(), molecule_type)
