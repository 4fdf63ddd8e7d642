"""Host-side API: parsing, encoding, dumps, pickling, equality.

Modelled on the reference's unit tests (src/pyjess/tests/test_template_atom.py,
test_template.py, test_atom.py, test_molecule.py); no GPU needed.
"""

import io
import pickle
import textwrap

import numpy as np
import pytest

from pyjess_gb300 import Atom, Jess, Mat4, Molecule, Template, TemplateAtom

TEMPLATE = textwrap.dedent(
    """
    ATOM      0  NZ  LYS A1030       1.431  -9.717  -1.722
    ATOM      0  CG  ASP A1132       0.000   0.000   0.000
    ATOM      0  OD1 ASP A1132       0.595   1.085   0.000
    ATOM      0  OD2 ASP A1132       0.609  -1.111   0.000
    ATOM      1  NE  ARG A1136       3.953   0.597  -1.721 K
    ATOM      0  CG  ASN A1137       0.736  -1.869  -4.261
    ATOM      0  OD1 ASN A1137       1.760  -2.435  -4.344
    ATOM      0  ND2 ASN A1137       0.264  -1.477  -3.134
    ATOM      0  CG  ASP A1150      -0.010  -5.408  -2.070
    ATOM      0  OD1 ASP A1150      -0.587  -5.769  -1.153
    ATOM      0  OD2 ASP A1150       1.085  -5.212  -2.011
    """
).strip()


def make_tatom(**kw):
    d = dict(atom_names=["NE"], residue_names=["ARG"], chain_id="A", residue_number=1,
             x=0.0, y=0.0, z=0.0, match_mode=0)
    d.update(kw)
    return TemplateAtom(**d)


class TestTemplateAtom:
    def test_load(self):
        atom = TemplateAtom.loads("ATOM      1  NE  ARG A1136       3.953   0.597  -1.721 K")
        assert atom.match_mode == 1
        assert atom.atom_names == ("NE",)
        assert atom.residue_names == ("ARG", "LYS")
        assert atom.chain_id == "A"
        assert atom.residue_number == 1136
        assert (atom.x, atom.y, atom.z) == (3.953, 0.597, -1.721)

    def test_invalid_match_code(self):
        with pytest.raises(ValueError):
            make_tatom(match_mode=2000)
        with pytest.raises(ValueError):
            make_tatom(match_mode=-10)
        with pytest.raises(ValueError):
            TemplateAtom.loads("ATOM    200  NE  ARG A1136       3.953   0.597  -1.721 K")

    def test_invalid_residue_name(self):
        with pytest.raises(ValueError):
            make_tatom(residue_names=["something"])

    def test_eq_hash(self):
        a, b = make_tatom(), make_tatom()
        assert a == b and hash(a) == hash(b) and a is not b
        assert a != make_tatom(x=1.0)

    def test_consistency(self):
        loaded = TemplateAtom.loads("ATOM      1  NE  ARG A1136       3.953   0.597  -1.721 K")
        created = TemplateAtom(chain_id=loaded.chain_id, residue_number=loaded.residue_number,
                               x=loaded.x, y=loaded.y, z=loaded.z,
                               residue_names=loaded.residue_names, atom_names=loaded.atom_names,
                               distance_weight=loaded.distance_weight, match_mode=loaded.match_mode)
        assert loaded == created

    def test_repr_pickle_roundtrip(self):
        atom = make_tatom()
        assert eval(repr(atom)) == atom
        assert pickle.loads(pickle.dumps(atom)) == atom

    def test_dumps(self):
        atom = TemplateAtom(chain_id="A", residue_number=1136, x=3.953, y=0.597, z=-1.721,
                            residue_names=["ARG", "LYS"], atom_names=["NE"],
                            distance_weight=0.0, match_mode=1)
        assert atom.dumps() == "ATOM      1  NE  ARG A1136       3.953   0.597  -1.721 K     0.00"

    def test_dumps_roundtrip(self):
        atom = make_tatom()
        t = atom.dumps()
        assert t[20:22] == " A"
        assert TemplateAtom.loads(t) == atom

    def test_distance_weight_column(self, golden):
        tpl = Template.load(str(golden / "4.1.2.tpl"))
        assert [a.distance_weight for a in tpl] == [0.53] * 3 + [2.08] * 3 + [2.35] * 3
        assert tpl[0].residue_names == ("THR", "THR")


class TestTemplate:
    def test_loads(self):
        tpl = Template.loads(TEMPLATE)
        assert len(tpl) == 11 and tpl.dimension == 5
        assert tpl[0].residue_names == ("LYS",)
        assert tpl[1].atom_names == ("CG",)
        assert tpl[2].residue_number == 1132
        assert tpl[-1].residue_number == 1150

    def test_id(self):
        assert Template.loads(TEMPLATE).id is None
        assert Template.loads("REMARK PDB_ID 2bw4\n" + TEMPLATE).id == "2bw4"

    def test_slicing_copy_eq_hash_pickle(self):
        t1 = Template.loads(TEMPLATE, id="tpl1")
        assert len(t1[1:4]) == 3
        t2 = Template.loads(TEMPLATE, id="tpl1")
        assert t1 == t2 and hash(t1) == hash(t2)
        assert t1 != Template.loads(TEMPLATE, id="tpl3")
        assert t1.copy() == t1
        assert pickle.loads(pickle.dumps(t1)) == t1
        assert Template.loads(t1.dumps()) == t1

    def test_empty(self):
        assert len(Template()) == 0 and not Template()

    def test_dimension_multiple_chains(self, golden):
        assert Template.load(str(golden / "1sur.qry")).dimension == 4

    def test_load_error(self, tmp_path):
        with pytest.raises(FileNotFoundError):
            Template.load("/some/nonsensical/file")


class TestAtomMolecule:
    LINE = "ATOM   2285  CA  THR A 293     -19.300 -20.307 -16.357  1.00  8.39           C"

    def test_atom_loads(self):
        atom = Atom.loads(self.LINE)
        assert atom.serial == 2285 and atom.name == "CA" and atom.residue_name == "THR"
        assert atom.chain_id == "A" and atom.residue_number == 293
        assert (atom.x, atom.y, atom.z) == (-19.300, -20.307, -16.357)
        assert atom.element == "C"
        assert atom.dumps() == self.LINE + "\n"

    def test_atom_init_and_errors(self):
        atom = Atom(serial=1, name="CA", residue_name="THR", chain_id="A", residue_number=3,
                    x=1.0, y=2.0, z=3.0)
        assert atom == Atom(**{k: v for k, v in atom._state().items()})
        assert pickle.loads(pickle.dumps(atom)) == atom
        for kw in (dict(name="ABCDE"), dict(residue_name="ABCD"), dict(chain_id="ABC")):
            base = dict(serial=1, name="CA", residue_name="THR", chain_id="A", residue_number=3,
                        x=1.0, y=2.0, z=3.0)
            base.update(kw)
            with pytest.raises(ValueError):
                Atom(**base)

    def test_molecule_load(self, amy, ayx):
        assert len(amy) == 3339 and amy.id == "1AMY"
        assert amy[0].serial == 1 and amy[0].name == "N" and amy[0].residue_name == "GLN"
        assert ayx[0].chain_id == "E"
        noh = Molecule.load(str(__import__("conftest").GOLDEN / "1AMY.pdb"), skip_hetatm=True)
        assert len(noh) == 3184

    def test_molecule_ops(self, amy):
        assert amy.copy() == amy
        assert len(amy[10:20]) == 10
        cons = amy.conserved(10.0)
        assert all(a.temperature_factor >= 10.0 for a in cons)
        m2 = pickle.loads(pickle.dumps(amy[:50]))
        assert m2 == amy[:50]
        text = amy[:5].dumps()
        assert Molecule.loads(text).id == "1AMY"

    def test_transform(self, amy):
        ident = Mat4([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 1, 0], [0, 0, 0, 1]])
        shift = Mat4([[1, 0, 0, 1], [0, 1, 0, 2], [0, 0, 1, 3], [0, 0, 0, 1]])
        assert amy[:3].transform(ident) == amy[:3]
        moved = amy[0].transform(shift)
        assert moved.x == pytest.approx(amy[0].x + 1) and moved.z == pytest.approx(amy[0].z + 3)
        assert np.asarray(shift @ ident).tolist() == np.asarray(shift).tolist()


class TestJessHost:
    def test_empty(self):
        j = Jess()
        assert len(j) == 0 and not j
        assert Jess() == Jess() and hash(Jess()) == hash(Jess())

    def test_getitem_copy(self, t133, t412):
        j = Jess([t133, t412])
        assert j[0] is t133 and j[-1] is t412
        assert len(j[:1]) == 1 and len(j[2:]) == 0
        assert j.copy() == j
        assert pickle.loads(pickle.dumps(j)) == j

    def test_query_argument_errors(self, t133, amy):
        j = Jess([t133])
        with pytest.raises(ValueError):
            j.query(amy, 2, 2, 2, max_candidates=-1)
        with pytest.raises(ValueError):
            j.query(amy, 2, 2, 2, ignore_chain="all")
        with pytest.warns(DeprecationWarning):
            q = j.query(amy, 2, 2, 2, ignore_chain=True)
        assert q.ignore_chain == "atoms"
