"""The CPU oracle against the reference's own golden vectors.

These pins are what make the oracle trustworthy as the parity reference:
- ``1AMY+1.3.3.txt``: Jess's output for template 1.3.3 on 1AMY,
  ``query(mol, 2, 4, 4, reorder=False)``, 156 hits in scanner order
  (reference test ``test_jess.py:228-274``), and the same hit set with
  ``reorder=True`` (``test_jess.py:276-334``);
- the module doctest of ``_jess.pyx:45-70``: templates [1.3.3, 4.1.2] on 1AMY
  with (2, 2, 2) give 13 hits in reorder=True order, best match 1.071, and
  the first hit's PDB dump (``_jess.pyx:2651-2662``);
- ``test_jess.py:336-372``: 4.1.2 on 5ayx.EF with (3, 3, 3) gives 0 / 2 / 7
  hits for ignore_chain None / "residues" / "atoms".
"""

import pytest

from helpers import oracle_hits, parse_block

DOCTEST_RMSD = "1.4386 1.4877 1.4376 1.5284 1.4863 1.4369 1.4790 1.1414 1.0755 1.1973 1.1353 1.0711 1.1494".split()

DOCTEST_DUMP = """REMARK 1AMY 1.439 2om2 Det= 1.0 log(E)~ 1.11
ATOM    729  CA  THR A  94      34.202 -24.426   8.851  1.00  2.00           C
ATOM    732  CB  THR A  94      35.157 -23.467   8.101  1.00  4.66           C
ATOM    733  OG1 THR A  94      36.338 -23.247   8.871  1.00  9.85           O
ATOM    746  CD  GLU A  96      41.454 -29.509   8.013  1.00 24.05           C
ATOM    748  OE2 GLU A  96      42.536 -29.680   7.441  1.00 34.44           O
ATOM    747  OE1 GLU A  96      41.212 -28.521   8.708  1.00 18.56           O
ATOM    437  CZ  ARG A  55      44.471 -26.619  10.181  1.00  8.51           C
ATOM    436  NE  ARG A  55      44.334 -27.346  11.290  1.00  9.05           N
ATOM    438  NH1 ARG A  55      43.590 -26.751   9.179  1.00 13.17           N
ENDMDL
"""


def check_block(hit, block, transform_check=True):
    query_id, rmsd, det, loge, atom_lines = parse_block(block)
    assert query_id == "1AMY"
    assert hit.rmsd == pytest.approx(rmsd, abs=5e-4)
    assert hit.determinant == pytest.approx(det, abs=0.05)
    assert hit.log_evalue == pytest.approx(loge, abs=0.0051)
    atoms = hit.atoms()
    assert len(atoms) == len(atom_lines)
    for atom, line in zip(atoms, atom_lines):
        assert atom.serial == int(line[7:12])
        assert atom.name == line[13:17].strip()
        assert atom.residue_name == line[17:21].strip()
        assert atom.chain_id == line[21:23].strip()
        assert atom.residue_number == int(line[23:27])
        assert atom.x == pytest.approx(float(line[31:39]), abs=5e-4)
        assert atom.y == pytest.approx(float(line[39:47]), abs=5e-4)
        assert atom.z == pytest.approx(float(line[47:55]), abs=5e-4)
        assert atom.occupancy == pytest.approx(float(line[55:61]), abs=5e-4)
        assert atom.temperature_factor == pytest.approx(float(line[61:67]), abs=5e-4)


def test_mcsa_query_no_reorder(t133, amy, golden_blocks):
    from pyjess_gb300 import Jess

    jess = Jess([t133])
    hits, _ = oracle_hits(jess, [amy], rmsd_threshold=2, distance_cutoff=4,
                          max_dynamic_distance=4, reorder=False)
    hits = hits[0]
    assert len(hits) == len(golden_blocks) == 156
    for hit, block in zip(hits, golden_blocks):
        assert hit.template() is t133
        check_block(hit, block)


def test_mcsa_query_reorder(t133, amy, golden_blocks):
    from pyjess_gb300 import Jess

    jess = Jess([t133])
    hits, _ = oracle_hits(jess, [amy], rmsd_threshold=2, distance_cutoff=4,
                          max_dynamic_distance=4, reorder=True)
    hits = hits[0]
    assert len(hits) == 156
    by_serials = {}
    for block in golden_blocks:
        lines = block.strip().splitlines()
        by_serials[tuple(int(l.split()[1]) for l in lines[1:-1])] = block
    for hit in hits:
        check_block(hit, by_serials[tuple(a.serial for a in hit.atoms(False))])


def test_kd_child_order_is_pinned(t133, amy, golden_blocks):
    """Visiting the left subtree first gives the same set in another order."""
    from pyjess_gb300 import Jess

    jess = Jess([t133])
    golden_serials = [tuple(int(l[6:11]) for l in b.strip().splitlines()[1:-1]) for b in golden_blocks]
    for right_first, same_order in ((1, True), (0, False)):
        hits, _ = oracle_hits(jess, [amy], rmsd_threshold=2, distance_cutoff=4,
                              max_dynamic_distance=4, reorder=False, kd_right_first=right_first)
        serials = [tuple(a.serial for a in h.atoms(False)) for h in hits[0]]
        assert set(serials) == set(golden_serials)
        assert (serials == golden_serials) is same_order
    from oracle import oracle

    oracle.lib().oracle_set_kd_right_first(oracle.KD_RIGHT_FIRST)


def test_doctest_order_and_dump(t133, t412, amy):
    from pyjess_gb300 import Jess

    jess = Jess([t133, t412])
    hits, _ = oracle_hits(jess, [amy], rmsd_threshold=2, distance_cutoff=2, max_dynamic_distance=2)
    hits = hits[0]
    assert [h.template().id for h in hits] == ["2om2"] * 13
    assert len(hits) == len(DOCTEST_RMSD)
    for hit, prefix in zip(hits, DOCTEST_RMSD):
        assert repr(hit.rmsd).startswith(prefix)
    assert hits[0].dumps(format="pdb") == DOCTEST_DUMP
    best, _ = oracle_hits(jess, [amy], rmsd_threshold=2, distance_cutoff=2, max_dynamic_distance=2,
                          best_match=True)
    assert len(best[0]) == 1
    assert repr(best[0][0].rmsd).startswith("1.071")


@pytest.mark.parametrize("mode,expected", [(0, 0), (1, 2), (2, 7)])
def test_ignore_chain_counts(t412, ayx, mode, expected):
    from pyjess_gb300 import Jess

    jess = Jess([t412])
    hits, _ = oracle_hits(jess, [ayx], rmsd_threshold=3, distance_cutoff=3, max_dynamic_distance=3,
                          ignore_chain=mode)
    assert len(hits[0]) == expected
    if mode == 1:
        for hit in hits[0]:
            atoms = hit.atoms(transform=False)
            for i in range(1, len(atoms)):
                if atoms[i - 1].residue_number == atoms[i].residue_number:
                    assert atoms[i - 1].chain_id == atoms[i].chain_id


def test_max_candidates_and_best_match_automaton(t133, amy):
    """The literal Query.__next__ replay: max_candidates cuts a template's
    stream, best_match keeps the first minimum; duplicated templates each
    report their own best (reference test_jess.py:134-226 semantics)."""
    from pyjess_gb300 import Jess

    jess = Jess([t133])
    full, _ = oracle_hits(jess, [amy], rmsd_threshold=2, distance_cutoff=4, max_dynamic_distance=4)
    n = len(full[0])
    for m in (0, 1, 2, 5, 50, 100000):
        cut, _ = oracle_hits(jess, [amy], rmsd_threshold=2, distance_cutoff=4, max_dynamic_distance=4,
                             max_candidates=m)
        assert 1 <= len(cut[0]) <= n
        if m >= 100000:
            assert len(cut[0]) == n
    jess3 = Jess([t133, t133, t133])
    best, _ = oracle_hits(jess3, [amy], rmsd_threshold=2, distance_cutoff=4, max_dynamic_distance=4,
                          best_match=True)
    assert len(best[0]) == 3
    low = min(h.rmsd for h in full[0])
    for hit in best[0]:
        assert hit.rmsd == low
