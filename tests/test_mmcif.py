"""mmCIF input (`Molecule.load(format="cif")`, format detection) against the
reference's own mmCIF tests (``src/pyjess/tests/test_molecule.py:253-360``)
and its 1AMY.cif / 1AMY.pdb fixtures, plus the CIF syntax the reader handles."""

import io
import itertools
import textwrap
import warnings

import pytest


def _load(golden, name, **kw):
    from pyjess_gb300 import Molecule

    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        return Molecule.load(str(golden / name), **kw)


def _same_atom(a, b, hetero=False):
    if not hetero:
        assert (a.serial, a.chain_id, a.residue_number) == (b.serial, b.chain_id, b.residue_number)
    assert (a.name, a.altloc, a.residue_name, a.insertion_code, a.element) == \
           (b.name, b.altloc, b.residue_name, b.insertion_code, b.element)
    for f in ("x", "y", "z", "occupancy", "temperature_factor", "charge"):
        assert getattr(a, f) == pytest.approx(getattr(b, f), abs=1e-5)


def test_cif_dump(golden):
    cif = _load(golden, "1AMY.cif", format="cif")
    expected = textwrap.dedent(
        """
        HEADER    HYDROLASE (O-GLYCOSYL)                  13-MAY-95   1AMY
        ATOM      1  N   GLN A   1       6.240  48.686  17.460  1.00 27.79           N
        ATOM      2  CA  GLN A   1       5.440  49.851  17.773  1.00 16.62           C
        ATOM      3  C   GLN A   1       6.628  50.721  18.086  1.00 14.24           C
        ATOM      4  O   GLN A   1       7.313  50.396  19.052  1.00 11.61           O
        ATOM      5  CB  GLN A   1       4.588  49.715  19.030  1.00 18.54           C
        """
    ).strip()
    assert cif[0:5].dumps().strip() == expected


def test_cif_vs_pdb(golden):
    cif = _load(golden, "1AMY.cif", format="cif")
    pdb = _load(golden, "1AMY.pdb", format="pdb")
    assert pdb[0:5] == cif[0:5]
    assert pdb[0:5].dumps(write_header=False).strip() == cif[0:5].dumps(write_header=False).strip()


@pytest.mark.parametrize("fmt", ["cif", "detect"])
def test_load_mmcif_after_comments(golden, fmt):
    from pyjess_gb300 import Molecule

    text = "# this is a comment line \n# and a second comment line \n" + (golden / "1AMY.cif").read_text()
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        assert len(Molecule.load(io.StringIO(text), format=fmt)) == 3339
        assert len(Molecule.loads(text, format=fmt)) == 3339


def test_load_consistency_no_skip_hetatm(golden):
    pdb = _load(golden, "1AMY.pdb", format="pdb")
    cif = _load(golden, "1AMY.cif", format="cif")
    assert len(cif) == len(pdb) == 3339
    for a, b in itertools.islice(zip(pdb, cif), 3184):
        _same_atom(a, b)
    for a, b in itertools.islice(zip(pdb, cif), 3184, 3339):
        _same_atom(a, b, hetero=True)


def test_hetatm_without_residue_number_warns(golden):
    from pyjess_gb300 import Molecule

    with pytest.warns(UserWarning, match="HETATM line found without residue number"):
        Molecule.load(str(golden / "1AMY.cif"), format="cif")
    cif = _load(golden, "1AMY.cif", format="cif", skip_hetatm=True)
    assert len(cif) == 3184


def test_use_author_numbers_match_pdb(golden):
    pdb = _load(golden, "1AMY.pdb", format="pdb")
    cif = _load(golden, "1AMY.cif", format="cif", use_author=True)
    assert len(cif) == len(pdb)
    for a, b in zip(pdb, cif):
        assert (a.residue_number, a.chain_id, a.name, a.residue_name) == \
               (b.residue_number, b.chain_id, b.name, b.residue_name)


def test_detect_pdb(golden):
    from pyjess_gb300 import Molecule

    assert len(Molecule.load(str(golden / "1AMY.pdb"))) == 3339


def test_cif_syntax():
    from pyjess_gb300._io import read_cif

    text = textwrap.dedent(
        """\
        # leading comment
        data_TEST
        _entry.id   TEST   # trailing comment
        _struct.title
        ;A title written
        over two lines
        ;
        loop_
        _atom_site.id
        _atom_site.label_atom_id
        _atom_site.note
        1 "O5'" 'it''s fine'
        2 CA    plain
        """
    )
    (block,) = read_cif(text)
    assert block.name == "TEST"
    assert block.find_value("_entry.id") == "TEST"
    assert block.find_value("_struct.title") == "A title written\nover two lines"
    rows = block.find("_atom_site.", ["id", "label_atom_id", "note", "?missing"])
    assert rows == [["1", '"O5\'"', "'it''s fine'", None], ["2", "CA", "plain", None]]
    assert block.find("_atom_site.", ["id", "missing"]) is None


def test_cif_errors():
    from pyjess_gb300 import Molecule

    with pytest.raises(ValueError):
        Molecule.loads("data_X\ndata_Y\n", format="cif")
    with pytest.raises(ValueError, match="missing columns"):
        Molecule.loads("data_X\n_entry.id X\n", format="cif")


@pytest.mark.parametrize("use_author", [False, True])
@pytest.mark.parametrize("skip_hetatm", [False, True])
def test_load_consistency(golden, use_author, skip_hetatm):
    """The four PDB/mmCIF consistency cases of the reference: ATOM records
    identical, HETATM records identical but for serial, chain and residue
    number (label columns number hetero groups differently)."""
    pdb = _load(golden, "1AMY.pdb", format="pdb", skip_hetatm=skip_hetatm)
    cif = _load(golden, "1AMY.cif", format="cif", use_author=use_author, skip_hetatm=skip_hetatm)
    n = 3184 if skip_hetatm else 3339
    assert len(cif) == len(pdb) == n
    for a, b in itertools.islice(zip(pdb, cif), 3184):
        _same_atom(a, b)
    for a, b in itertools.islice(zip(pdb, cif), 3184, n):
        _same_atom(a, b, hetero=True)
