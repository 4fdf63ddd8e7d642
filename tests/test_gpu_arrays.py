"""`Jess.query_arrays`: the hits of `Jess.query_many` as NumPy columns."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("best", [False, True])
def test_query_arrays_matches_query_many(t133, t412, amy, ayx, best):
    from pyjess_gb300 import Jess

    jess = Jess([t133, t412])
    mols = [amy, ayx, amy[:1500]]
    many = jess.query_many(mols, 2, 4, 4, best_match=best)
    arr = jess.query_arrays(mols, 2, 4, 4, best_match=best)
    flat = [(m, h) for m, hits in enumerate(many) for h in hits]
    assert len(arr) == len(flat) > 0
    offsets = arr.molecule_offsets()
    assert [offsets[m + 1] - offsets[m] for m in range(len(mols))] == [len(h) for h in many]
    for i, (m, h) in enumerate(flat):
        assert arr.rmsd[i] == h.rmsd
        assert int(arr.molecule[i]) == m
        assert jess[int(arr.template[i])] is h.template()
        assert np.array_equal(arr.rotation[i].reshape(9), h._rotation)
        assert np.array_equal(arr.centres[i], h._centre)
        a0, a1 = arr.atom_offset[i], arr.atom_offset[i + 1]
        got = arr.hit(i)
        assert [a.serial for a in got.atoms(False)] == [a.serial for a in h.atoms(False)]
        assert got.rmsd == h.rmsd and got.dumps() == h.dumps()
        assert a1 - a0 == len(h.template())


def test_query_arrays_empty():
    from pyjess_gb300 import Jess, Molecule

    arr = Jess().query_arrays([Molecule()], 2, 2, 2)
    assert len(arr) == 0 and list(arr.molecule_offsets()) == [0, 0]


def test_superposed_atoms_match_host_transform(t133, t412, amy, ayx):
    """HitArrays.superposed_atoms (the device transform of every hit's
    matched atoms) against Hit.atoms(transform=True) on the host."""
    from pyjess_gb300 import Jess

    jess = Jess([t133, t412])
    mols = [amy, ayx]
    arr = jess.query_arrays(mols, 2, 4, 4)
    xyz = arr.superposed_atoms()
    assert xyz.shape == (len(arr.atoms), 3) and len(arr) > 0
    worst = 0.0
    for i in range(len(arr)):
        hit = arr.hit(i)
        host = np.array([[a.x, a.y, a.z] for a in hit.atoms(transform=True)])
        a0, a1 = arr.atom_offset[i], arr.atom_offset[i + 1]
        worst = max(worst, float(np.abs(xyz[a0:a1] - host).max()))
    assert worst < 1e-12, worst
    # the transformed atoms reproduce each hit's rmsd against its template
    for i in range(0, len(arr), 7):
        tpl = np.array([[a.x, a.y, a.z] for a in jess[int(arr.template[i])]])
        a0, a1 = arr.atom_offset[i], arr.atom_offset[i + 1]
        rmsd = np.sqrt(((xyz[a0:a1] - tpl) ** 2).sum() / len(tpl))
        assert abs(rmsd - arr.rmsd[i]) < 1e-9
