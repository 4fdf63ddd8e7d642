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
