"""The native PDB reader (pjg_parse_pdb) against the general Python reader:
the same atom records, header fields and errors on the reference's
fixtures and on edited texts (HETATM and ENDMDL options, charges, blank
fields, short and long lines, line endings, mmCIF tags), and the fallback
to the general reader for forms the native one does not take."""

import io

import numpy as np
import pytest

from pyjess_gb300 import _io


def _both(text, **kw):
    fast = _io.parse_pdb_text(text, **kw)
    slow = _io.parse_pdb(io.StringIO(text), **kw)
    return fast, slow


def _same(text, **kw):
    (fr, *fh), (sr, *sh) = _both(text, **kw)
    assert fr.dtype == sr.dtype
    assert fr.tobytes() == sr.tobytes()
    assert fh == sh
    return fr


def _native_took(text, **kw):
    from pyjess_gb300 import _native
    from pyjess_gb300._records import ATOM_DTYPE

    flags = (_native.PDB_IGNORE_ENDMDL if kw.get("ignore_endmdl") else 0) | \
        (_native.PDB_SKIP_HETATM if kw.get("skip_hetatm") else 0)
    return _native.parse_pdb_records(text.encode("ascii"), flags, ATOM_DTYPE) is not None


@pytest.mark.parametrize("name", ["1AMY.pdb", "5ayx.EF.pdb"])
@pytest.mark.parametrize("kw", [{}, {"skip_hetatm": True}, {"ignore_endmdl": True}])
def test_fixtures_identical(golden, name, kw):
    text = (golden / name).read_text()
    rec = _same(text, **kw)
    assert len(rec) > 0
    assert _native_took(text, **kw)


ATOM = "ATOM      1  N   ALA A   1      11.104   6.134  -6.504  1.00  0.00           N  \n"
HET = "HETATM  100 FE   HEM A 200      -1.500  22.250   3.125  0.50 10.00          FE2+\n"


def test_models_endmdl_and_header():
    text = ("HEADER    HYDROLASE                               02-JAN-99   1ABC              \n"
            "MODEL        1\n" + ATOM + "ENDMDL\n" + "MODEL        2\n" + ATOM.replace("11.104", "12.104") +
            "ENDMDL\nHEADER    OTHER                                   03-FEB-00   2XYZ\n")
    r1 = _same(text)
    r2 = _same(text, ignore_endmdl=True)
    assert len(r1) == 1 and len(r2) == 2
    (_, id_, date, name), _ = _both(text)
    assert (id_, date.year, name) == ("1ABC", 1999, "HYDROLASE")


@pytest.mark.parametrize("edit", [
    lambda l: l,                                                # plain
    lambda l: l.replace("  N  \n", "  N1-\n"),                  # charge n-
    lambda l: l.replace("  N  \n", "  N-1\n"),                  # signed charge
    lambda l: l.replace("  N  \n", "  NXX\n"),                  # unparsable charge -> 0
    lambda l: l.replace("  N  \n", "  N+ \n"),                  # lone sign -> 0
    lambda l: l.replace("1.00  0.00", "          "),             # blank occupancy / B
    lambda l: l[:54] + "\n",                                     # minimal record
    lambda l: l.rstrip("\n") + "  trailing columns beyond eighty\n",
    lambda l: l.replace("\n", "\r\n"),                           # CRLF (text mode reads LF)
    lambda l: l.replace("   1  ", "      ", 1),                  # blank serial
    lambda l: l.replace("11.104", "11.1e0"),                     # exponent
    lambda l: l.replace("11.104", "1_1.10"),                     # Python float syntax only
    lambda l: l.replace("11.104", "-0.000"),                     # negative zero
    lambda l: l.replace("ALA", "A\tA"),                          # tab in a name
])
def test_record_forms(edit):
    _same(edit(ATOM) + HET + edit(ATOM))


def test_short_record_raises_the_same_error():
    text = ATOM + ATOM[:50] + "\n"
    with pytest.raises(ValueError, match="Failed to parse atom"):
        _io.parse_pdb(io.StringIO(text))
    with pytest.raises(ValueError, match="Failed to parse atom"):
        _io.parse_pdb_text(text)


def test_bad_coordinate_raises_the_same_error():
    text = ATOM.replace("11.104", "  abcd  ")
    with pytest.raises(ValueError):
        _io.parse_pdb_text(text)


def test_mmcif_tag_is_rejected():
    with pytest.raises(ValueError, match="mmCIF"):
        _io.parse_pdb_text(ATOM + "data_1ABC\n")


def test_many_structures_round_trip(golden):
    """Molecule.load through the native reader equals the general reader's
    molecule atom for atom."""
    from pyjess_gb300 import Molecule

    m = Molecule.load(str(golden / "1AMY.pdb"))
    text = (golden / "1AMY.pdb").read_text()
    recs, *_ = _io.parse_pdb(io.StringIO(text))
    assert len(m) == len(recs)
    assert np.array_equal(np.array([a.serial for a in m]), recs["serial"])
