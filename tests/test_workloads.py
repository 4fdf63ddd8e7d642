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


def test_template_subset_repacks():
    from oracle import oracle
    from pyjess_gb300 import workloads as W

    wl = W.config(3, n_structures=3, n_templates=12)
    t = wl.templates
    whole = t.subset(range(t.n_templates))
    for f in ("atom_offset", "code", "res_seq", "chain", "xyz", "dist_weight", "name_offset", "names",
              "resname_offset", "resnames", "dim"):
        assert np.array_equal(getattr(whole, f), getattr(t, f)), f
    # a subset searches like the same templates inside the whole set
    part = t.subset([7, 2, 9])
    r = oracle.query(part, wl.structures, **wl.params)["hits"]
    ref = oracle.query(t, wl.structures, **wl.params)["hits"]
    mine = sorted((int(s), [7, 2, 9][int(k)], int(o)) for s, k, o in zip(r["structure"], r["template"], r["ordinal"]))
    full = sorted((int(s), int(k), int(o)) for s, k, o in zip(ref["structure"], ref["template"], ref["ordinal"])
                  if int(k) in (7, 2, 9))
    assert mine == full


def test_adversarial_structures_concentrate_boundary_tests():
    """The adversarial structures' moved atoms put candidate-pair distances
    within 1e-6 A of annulus boundaries far more often than in ordinary
    structures (oracle counts of every annulus test)."""
    from oracle import oracle
    from pyjess_gb300 import workloads as W

    wl = W.config(3, n_structures=40, n_templates=400)
    assert wl.n_adversarial == 4
    adv = oracle.query(wl.templates, wl.structures.subset(range(4)), threads=4, **wl.params)["boundary"]
    ordn = oracle.query(wl.templates, wl.structures.subset(range(4, 40)), threads=4, **wl.params)["boundary"]
    assert adv["tests"] > 0 and ordn["tests"] > 0
    assert adv["near"] / adv["tests"] > 10 * max(ordn["near"], 1) / ordn["tests"]
