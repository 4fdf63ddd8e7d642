"""The seeded synthetic workloads: deterministic, with the stated shapes."""

import numpy as np


def test_config3_is_deterministic_and_shaped():
    from pyjess_gb300 import workloads as W

    a = W.config(3, n_structures=6, n_templates=20)
    b = W.config(3, n_structures=6, n_templates=20)
    assert np.array_equal(a.structures.xyz, b.structures.xyz)
    assert np.array_equal(a.templates.xyz, b.templates.xyz)
    assert a.structures.n_structures == 6 and a.templates.n_templates == 20
    # templates: 3 atoms a residue, 2-8 residues
    counts = np.diff(a.templates.atom_offset)
    assert counts.min() >= 6 and counts.max() <= 24 and (counts % 3 == 0).all()
    # coordinates rounded to 0.001 A, as PDB files are, except in the
    # adversarial structures (10% of config 3: here structure 0), whose
    # moved atoms sit within 1e-6 A of annulus boundaries
    x = a.structures.xyz[a.structures.atom_offset[1]:]
    assert np.allclose(x, np.round(x, 3), atol=1e-9)


def test_shards_are_independent_draws():
    from pyjess_gb300 import workloads as W

    a = W.config(3, n_structures=4, n_templates=5, shard=1)
    b = W.config(3, n_structures=4, n_templates=5, shard=2)
    c = W.config(3, n_structures=4, n_templates=5)
    assert not np.array_equal(a.structures.xyz[:10], b.structures.xyz[:10])
    assert not np.array_equal(a.structures.xyz[:10], c.structures.xyz[:10])
    assert a.structures.n_structures == b.structures.n_structures == 4
