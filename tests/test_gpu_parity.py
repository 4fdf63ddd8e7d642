"""GPU parity: libpjg against the CPU oracle and the reference's golden vectors.

Bar: the ordered hit list of every structure is identical (template,
stream ordinal and every matched atom, in the reference's order); RMSD within
RMSD_TOL of the FP64 oracle; rotations within ROT_TOL; the search counters
(pairs, partial assignments, complete assignments, algorithmic bytes) equal
the oracle's instrumented counts.
"""

import numpy as np
import pytest

from helpers import hit_keys, parse_block

pytestmark = pytest.mark.gpu

RMSD_TOL = 1e-9    # Angstrom, GPU quaternion solver vs oracle Jacobi (FP64)
# Rotation entries.  Where the covariance is well conditioned
# (s3/s1 > 1e-3) the GPU quaternion rotation and the oracle's polar
# decomposition agree to ROT_TOL.  For near-coplanar assignments the polar
# formula (like the reference's, undefined at rank < 3) loses accuracy, so
# there the GPU rotation is checked against an SVD Kabsch solution instead,
# and everywhere it must reproduce the reported rmsd when applied.
ROT_TOL = 1e-7

MODES = ("fp32", "fp64", "plain")


def gpu_query(ptemplates, pstructures, mode="fp32", **kw):
    from pyjess_gb300 import _native
    from pyjess_gb300._abi import QueryParams

    P = QueryParams(
        rmsd_threshold=kw["rmsd_threshold"], distance_cutoff=kw["distance_cutoff"],
        max_dynamic_distance=kw["max_dynamic_distance"],
        max_candidates=-1 if kw.get("max_candidates") is None else kw["max_candidates"],
        ignore_chain=kw.get("ignore_chain", 0), best_match=int(kw.get("best_match", False)),
        reorder=int(kw.get("reorder", True)),
        mode={"fp32": _native.MODE_BATCHED_FP32, "fp64": _native.MODE_BATCHED_FP64,
              "plain": _native.MODE_PLAIN_FP64}[mode])
    res = _native.query(_native.Templates(ptemplates), _native.Structures(pstructures), P)
    return res


def check_rotations(g, r, ptemplates, pstructures, limit=5000):
    """GPU rotations: proper, optimal (they reproduce the reported rmsd),
    equal to the oracle's where the fit is well conditioned and to an SVD
    Kabsch rotation elsewhere (see ROT_TOL)."""
    for i in range(min(g["count"], limit)):
        R = g["rotation"][i].reshape(3, 3)
        assert abs(np.linalg.det(R) - 1.0) < 1e-9
        s, t = int(g["structure"][i]), int(g["template"][i])
        a0, a1 = g["atom_offset"][i], g["atom_offset"][i + 1]
        mol = pstructures.xyz[pstructures.atom_offset[s] + g["atoms"][a0:a1]]
        tpl = ptemplates.xyz[ptemplates.atom_offset[t]:ptemplates.atom_offset[t + 1]]
        c = g["centres"][i]
        fit = (mol - c[:3]) @ R.T + c[3:]
        rmsd = np.sqrt(((fit - tpl) ** 2).sum() / len(tpl))
        assert abs(rmsd - g["rmsd"][i]) < 1e-7, (i, rmsd, g["rmsd"][i])
        if len(tpl) < 3:
            continue
        a, b = mol - mol.mean(0), tpl - tpl.mean(0)
        U, sv, Vt = np.linalg.svd(a.T @ b)
        cond = sv[2] / sv[0] if sv[0] > 0 else 0.0
        if cond > 1e-3:
            assert np.abs(R - r["rotation"][i].reshape(3, 3)).max() <= ROT_TOL
        elif cond > 1e-9:
            d = np.sign(np.linalg.det(Vt.T @ U.T))
            Rk = Vt.T @ np.diag([1, 1, d]) @ U.T
            assert np.abs(R - Rk).max() <= 1e-12 / cond + 1e-9


def svd_rmsd(mol, tpl):
    a, b = mol - mol.mean(0), tpl - tpl.mean(0)
    M = a.T @ b
    sv = np.linalg.svd(M, compute_uv=False)
    lam = sv[0] + sv[1] + (sv[2] if np.linalg.det(M) > 0 else -sv[2])
    e = (a * a).sum() + (b * b).sum() - 2 * lam
    return np.sqrt(max(e, 0.0) / len(a)), sv


def check_rmsd(g, r, ptemplates, pstructures):
    """|rmsd_gpu - rmsd_oracle| <= RMSD_TOL.  The oracle, like the reference,
    takes singular values as square roots of the eigenvalues of M^T M, which
    loses accuracy when the smallest singular value is tiny (s3/s1 < 1e-5:
    near-coplanar atom sets); there the GPU value must instead be within
    RMSD_TOL of an SVD of M itself.  Returns the largest GPU-oracle gap."""
    err = np.abs(g["rmsd"] - r["rmsd"])
    for i in np.flatnonzero(err > RMSD_TOL):
        s, t = int(g["structure"][i]), int(g["template"][i])
        a0, a1 = g["atom_offset"][i], g["atom_offset"][i + 1]
        mol = pstructures.xyz[pstructures.atom_offset[s] + g["atoms"][a0:a1]]
        tpl = ptemplates.xyz[ptemplates.atom_offset[t]:ptemplates.atom_offset[t + 1]]
        exact, sv = svd_rmsd(mol, tpl)
        assert sv[2] < 1e-5 * sv[0], (i, err[i], sv)
        assert abs(g["rmsd"][i] - exact) <= RMSD_TOL, (i, g["rmsd"][i], exact)
    return float(err.max())


def compare(ptemplates, pstructures, mode="fp32", check_stats=True, **kw):
    from oracle import oracle

    ref = oracle.query(ptemplates, pstructures, threads=8, **kw)
    res = gpu_query(ptemplates, pstructures, mode=mode, **kw)
    g = res.arrays()
    r = ref["hits"]
    assert hit_keys(g) == hit_keys(r)
    if r["count"]:
        check_rmsd(g, r, ptemplates, pstructures)
        assert np.abs(g["centres"] - r["centres"]).max() <= 1e-9
        check_rotations(g, r, ptemplates, pstructures)
    gw = res.warnings()
    assert list(gw[0]) == list(ref["warnings"][0]) and list(gw[1]) == list(ref["warnings"][1])
    if check_stats and kw.get("max_candidates") is None:
        gs, os_ = res.stats(), ref["stats"]
        for key in ("pairs", "candidate_entries", "partials", "complete", "bytes_candidates",
                    "bytes_expansion"):
            assert gs[key] == os_[key], (key, gs[key], os_[key])
    return res, ref


# --- reference golden vectors through the public API -------------------------


@pytest.mark.parametrize("reorder", [False, True])
def test_golden_1amy(t133, amy, golden_blocks, reorder):
    from pyjess_gb300 import Jess

    jess = Jess([t133])
    hits = list(jess.query(amy, 2, 4, 4, reorder=reorder))
    assert len(hits) == 156
    serials = [tuple(a.serial for a in h.atoms(False)) for h in hits]
    golden = [tuple(int(l[6:11]) for l in b.strip().splitlines()[1:-1]) for b in golden_blocks]
    if not reorder:
        assert serials == golden
    else:
        assert sorted(serials) == sorted(golden)
    by = dict(zip(golden, golden_blocks))
    for hit, key in zip(hits, serials):
        _, rmsd, det, loge, lines = parse_block(by[key])
        assert hit.rmsd == pytest.approx(rmsd, abs=5e-4)
        assert hit.determinant == pytest.approx(det, abs=0.05)
        assert hit.log_evalue == pytest.approx(loge, abs=0.0051)
        for atom, line in zip(hit.atoms(), lines):
            assert atom.x == pytest.approx(float(line[31:39]), abs=5e-4)
            assert atom.y == pytest.approx(float(line[39:47]), abs=5e-4)
            assert atom.z == pytest.approx(float(line[47:55]), abs=5e-4)


def test_golden_doctest(t133, t412, amy):
    from test_oracle_golden import DOCTEST_DUMP, DOCTEST_RMSD
    from pyjess_gb300 import Jess

    jess = Jess([t133, t412])
    hits = list(jess.query(amy, 2, 2, 2))
    assert [h.template().id for h in hits] == ["2om2"] * 13
    for hit, prefix in zip(hits, DOCTEST_RMSD):
        assert repr(hit.rmsd)[:6] == prefix[:6] or abs(hit.rmsd - float(prefix)) < 1e-4
    assert hits[0].dumps() == DOCTEST_DUMP
    best = list(jess.query(amy, 2, 2, 2, best_match=True))
    assert len(best) == 1 and round(best[0].rmsd, 3) == 1.071


@pytest.mark.parametrize("ignore,expected", [(None, 0), ("residues", 2), ("atoms", 7)])
def test_golden_ignore_chain(t412, ayx, ignore, expected):
    from pyjess_gb300 import Jess

    assert len(list(Jess([t412]).query(ayx, 3, 3, 3, ignore_chain=ignore))) == expected


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("reorder", [False, True])
def test_golden_vs_oracle_all_modes(t133, t412, amy, mode, reorder):
    from pyjess_gb300 import Jess
    from pyjess_gb300._pack import pack_molecules

    jess = Jess([t133, t412, t133])
    compare(jess._packed_templates(), pack_molecules([amy]), mode=mode, rmsd_threshold=2,
            distance_cutoff=4, max_dynamic_distance=4, reorder=reorder)


@pytest.mark.parametrize("mc", [0, 1, 3, 10])
@pytest.mark.parametrize("best", [False, True])
def test_automaton_max_candidates(t133, t412, amy, mc, best):
    from pyjess_gb300 import Jess
    from pyjess_gb300._pack import pack_molecules

    jess = Jess([t133, t412, t133])
    compare(jess._packed_templates(), pack_molecules([amy]), rmsd_threshold=2, distance_cutoff=4,
            max_dynamic_distance=4, max_candidates=mc, best_match=best)


# --- synthetic workloads --------------------------------------------------------


@pytest.mark.parametrize("mode", MODES)
def test_config0(mode):
    from pyjess_gb300 import workloads as W

    wl = W.config(0)
    compare(wl.templates, wl.structures, mode=mode, **wl.params)


@pytest.mark.parametrize("mode", MODES)
def test_config1_bit_exact_order(mode):
    from pyjess_gb300 import workloads as W

    wl = W.config(1)
    res, ref = compare(wl.templates, wl.structures, mode=mode, **wl.params)
    assert ref["hits"]["count"] > 100


@pytest.mark.parametrize("index", [2, 3])
@pytest.mark.parametrize("mode", ["fp32", "fp64"])
def test_config_batched_reduced(index, mode):
    from pyjess_gb300 import workloads as W

    wl = W.config(index, n_structures=40, n_templates=300)
    compare(wl.templates, wl.structures, mode=mode, **wl.params)


def test_config3_adversarial_guard_band():
    """Structures whose atoms sit within 1e-6 A of annulus boundaries: the
    FP32 filter must send them to the FP64 recheck and decide as the oracle."""
    from pyjess_gb300 import workloads as W

    wl = W.config(3, n_structures=20, n_templates=200)
    res, ref = compare(wl.templates, wl.structures, mode="fp32", **wl.params)
    assert res.stats()["fp64_rechecks"] > 0


@pytest.mark.parametrize("best", [False, True])
def test_config4_dense_reduced(best):
    from pyjess_gb300 import workloads as W

    wl = W.config(4, n_structures=3, n_templates=6, residues=(300, 500))
    p = dict(wl.params)
    p["max_candidates"] = 50
    compare(wl.templates, wl.structures, best_match=best, **p)


@pytest.mark.parametrize("ignore", [0, 1, 2])
def test_ignore_chain_synthetic(ignore):
    from pyjess_gb300 import workloads as W

    wl = W.config(2, n_structures=10, n_templates=100)
    compare(wl.templates, wl.structures, ignore_chain=ignore, **wl.params)


# --- edge cases -------------------------------------------------------------------


def test_empty_inputs(t133):
    from pyjess_gb300 import Jess, Molecule

    assert list(Jess().query(Molecule(), 2, 2, 4)) == []
    assert list(Jess([t133]).query(Molecule(), 2, 2, 4)) == []


def test_single_atom_and_tiny_templates(amy):
    """One-atom templates: the scanner skips the first seed and every
    superposition is degenerate (NaN rotation), so only warnings come out."""
    from pyjess_gb300 import Jess, Template, TemplateAtom
    from pyjess_gb300._pack import pack_molecules

    one = Template([TemplateAtom(chain_id="A", residue_number=1, x=0, y=0, z=0, residue_names=["SER"],
                                 atom_names=["OG"], match_mode=0)], id="one")
    jess = Jess([one])
    res, ref = compare(jess._packed_templates(), pack_molecules([amy[:400]]), rmsd_threshold=2,
                       distance_cutoff=2, max_dynamic_distance=2, check_stats=False)
    assert res.arrays()["count"] == 0
    assert len(res.warnings()[0]) == len(ref["warnings"][0]) > 0
    with pytest.warns(UserWarning):
        assert list(jess.query(amy[:400], 2, 2, 2)) == []


def test_no_candidates_skips_template(t133, amy):
    from pyjess_gb300 import Jess, Template, TemplateAtom
    from pyjess_gb300._pack import pack_molecules

    ghost = Template([TemplateAtom(chain_id="A", residue_number=1, x=0, y=0, z=0, residue_names=["XYZ"],
                                   atom_names=["QQ"], match_mode=0)] * 3, id="ghost")
    jess = Jess([t133, ghost])
    compare(jess._packed_templates(), pack_molecules([amy]), rmsd_threshold=2, distance_cutoff=4,
            max_dynamic_distance=4)


def test_query_many_matches_query(t133, t412, amy, ayx):
    from pyjess_gb300 import Jess

    jess = Jess([t133, t412])
    mols = [amy, ayx, amy[:1000]]
    many = jess.query_many(mols, 2, 3, 3)
    for mol, hits in zip(mols, many):
        single = list(jess.query(mol, 2, 3, 3))
        assert [tuple(a.serial for a in h.atoms(False)) for h in hits] == \
               [tuple(a.serial for a in h.atoms(False)) for h in single]
        assert [h.rmsd for h in hits] == [h.rmsd for h in single]


# --- kd leaf order on demand ----------------------------------------------------
#
# PJG_LEAF_LEVELS sets how many levels' lists are put in leaf order before
# the search; deeper lists are ordered when a pair first reaches them, the
# pair being suspended and resumed from its saved search state, or, when the
# state pool is full (PJG_STATE_POOL=0 forces it), replayed from its start
# skipping the rows it already emitted.  Small values force many
# suspensions; -1 orders every list up front.

POOLS = [None, "0"]


def set_pool(monkeypatch, pool):
    if pool is None:
        monkeypatch.delenv("PJG_STATE_POOL", raising=False)
    else:
        monkeypatch.setenv("PJG_STATE_POOL", pool)


@pytest.mark.parametrize("pool", POOLS)
@pytest.mark.parametrize("levels", [-1, 0, 1, 2, 9, 12])
def test_leaf_order_on_demand_config3(monkeypatch, levels, pool):
    from pyjess_gb300 import workloads as W

    monkeypatch.setenv("PJG_LEAF_LEVELS", str(levels))
    set_pool(monkeypatch, pool)
    wl = W.config(3, n_structures=30, n_templates=300)
    res, ref = compare(wl.templates, wl.structures, mode="fp32", **wl.params)
    st = res.stats()
    if levels in (0, 1):
        assert st["suspensions"] > 0 and st["search_rounds"] > 1
    if levels == -1:
        assert st["suspensions"] == 0 and st["search_rounds"] == st["chunks"]


@pytest.mark.parametrize("heavy", ["1", "0"])
def test_heavy_pairs_first(monkeypatch, heavy):
    """The costliest pairs taken first (done for chunks of at least eight
    times the heavy-pair target; PJG_HEAVY_PER_WARP=1 brings the target
    within reach of a 70 x 300 workload) or not: the oracle's hits and
    search counters either way."""
    from pyjess_gb300 import workloads as W

    monkeypatch.setenv("PJG_HEAVY_PER_WARP", "1")
    monkeypatch.setenv("PJG_HEAVY_FIRST", heavy)
    wl = W.config(3, n_structures=70, n_templates=300)
    compare(wl.templates, wl.structures, mode="fp32", **wl.params)


@pytest.mark.parametrize("levels", [3, 10])
def test_leaf_order_up_front_levels_without_reorder(monkeypatch, levels):
    """Template atoms taken in their own order (reorder=False) with 3 and
    10 levels put in leaf order before the search (the second deeper than
    the level demand keeps in registers): the oracle's hits."""
    from pyjess_gb300 import workloads as W

    monkeypatch.setenv("PJG_LEAF_LEVELS", str(levels))
    wl = W.config(3, n_structures=20, n_templates=200)
    compare(wl.templates, wl.structures, mode="fp32", reorder=False, **wl.params)


@pytest.mark.parametrize("pool", POOLS)
@pytest.mark.parametrize("levels", [4, 1])
def test_list_sharing(monkeypatch, levels, pool):
    """Requested lists of one structure with the same atoms share one leaf
    order (the default; PJG_LIST_SHARING=0 orders every list itself).  The
    workload's templates list extra residue names in random order, so lists
    share by equal sequences and by equal sets in another order; both runs
    give the oracle's hits, bit for bit the same arrays."""
    from pyjess_gb300 import workloads as W

    monkeypatch.setenv("PJG_LEAF_LEVELS", str(levels))
    set_pool(monkeypatch, pool)
    wl = W.config(3, n_structures=30, n_templates=300)
    res, _ = compare(wl.templates, wl.structures, mode="fp32", **wl.params)
    st = res.stats()
    assert 0 < st["leaf_shared"] < st["leaf_lists"]
    monkeypatch.setenv("PJG_LIST_SHARING", "0")
    res0, _ = compare(wl.templates, wl.structures, mode="fp32", **wl.params)
    st0 = res0.stats()
    assert st0["leaf_shared"] == 0 and st0["leaf_lists"] == st["leaf_lists"]
    a, b = res.arrays(), res0.arrays()
    assert a["count"] == b["count"]
    for k in a:
        if k != "count":
            assert np.array_equal(a[k], b[k]), k


@pytest.mark.parametrize("pool", POOLS)
@pytest.mark.parametrize("levels", [0, 1])
@pytest.mark.parametrize("best", [False, True])
def test_leaf_order_on_demand_cut(monkeypatch, levels, best, pool):
    """max_candidates cut (applied inside the search in non-best mode) and
    best_match across suspended and resumed (or replayed) pairs."""
    from pyjess_gb300 import workloads as W

    monkeypatch.setenv("PJG_LEAF_LEVELS", str(levels))
    set_pool(monkeypatch, pool)
    wl = W.config(4, n_structures=3, n_templates=6, residues=(300, 500))
    p = dict(wl.params)
    p["max_candidates"] = 50
    compare(wl.templates, wl.structures, best_match=best, **p)


@pytest.mark.parametrize("pool", POOLS)
@pytest.mark.parametrize("levels", [0, 1])
@pytest.mark.parametrize("mode", MODES)
def test_leaf_order_on_demand_golden(monkeypatch, t133, t412, amy, levels, mode, pool):
    from pyjess_gb300 import Jess
    from pyjess_gb300._pack import pack_molecules

    monkeypatch.setenv("PJG_LEAF_LEVELS", str(levels))
    set_pool(monkeypatch, pool)
    jess = Jess([t133, t412, t133])
    compare(jess._packed_templates(), pack_molecules([amy]), mode=mode, rmsd_threshold=2,
            distance_cutoff=4, max_dynamic_distance=4, reorder=False)


def test_leaf_order_on_demand_orders_fewer_entries(monkeypatch):
    from pyjess_gb300 import workloads as W

    wl = W.config(3, n_structures=20, n_templates=1000)
    monkeypatch.setenv("PJG_LEAF_LEVELS", "-1")
    full = gpu_query(wl.templates, wl.structures, **wl.params)
    monkeypatch.setenv("PJG_LEAF_LEVELS", "4")
    lazy = gpu_query(wl.templates, wl.structures, **wl.params)
    assert hit_keys(full.arrays()) == hit_keys(lazy.arrays())
    fs, ls = full.stats(), lazy.stats()
    assert ls["leaf_entries"] < fs["leaf_entries"]
    for key in ("partials", "complete", "bytes_expansion", "fp64_rechecks"):
        assert fs[key] == ls[key], key


@pytest.mark.parametrize("levels", [1, 4])
def test_leaf_arrays_grow(monkeypatch, levels):
    """Leaf-order arrays that start at one entry grow as lists are requested
    (before the search and between rounds); one structure per chunk."""
    from pyjess_gb300 import workloads as W

    monkeypatch.setenv("PJG_LEAF_LEVELS", str(levels))
    monkeypatch.setenv("PJG_LEAF_CAPACITY", "1")
    wl = W.config(3, n_structures=12, n_templates=300)
    compare(wl.templates, wl.structures, mode="fp32", **wl.params)
    monkeypatch.setenv("PJG_ENTRY_BUDGET", "1")
    res, _ = compare(wl.templates, wl.structures, mode="fp32", **wl.params)
    assert res.stats()["chunks"] == 12


def test_row_budget_split(monkeypatch):
    """A chunk whose complete rows exceed the row budget is redone on half
    its structures (down to one): the same hits and search counters as the
    oracle's."""
    from pyjess_gb300 import workloads as W

    monkeypatch.setenv("PJG_ROW_BUDGET", "50")
    wl = W.config(3, n_structures=12, n_templates=300)
    res, ref = compare(wl.templates, wl.structures, mode="fp32", **wl.params)
    st = res.stats()
    assert st["row_splits"] > 0 and st["chunks"] > 1


def test_large_result_copy_out():
    """Results of several MiB come back through the threaded copy (one host
    thread per MiB, each touching then copying its range of the caller's
    arrays): every field matches the oracle, and a second copy of the same
    results is identical."""
    from pyjess_gb300 import workloads as W

    wl = W.config(3, n_structures=60, n_templates=600)
    res, ref = compare(wl.templates, wl.structures, mode="fp32", **wl.params)
    a = res.arrays()
    nbytes = sum(v.nbytes for k, v in a.items() if hasattr(v, "nbytes"))
    assert nbytes > (4 << 20), nbytes
    res._arrays = None
    b = res.arrays()
    for k in a:
        if hasattr(a[k], "nbytes"):
            assert np.array_equal(a[k], b[k]), k


def test_rmsd_max_error_per_config(capsys):
    """Largest |rmsd_gpu - rmsd_oracle| per configuration (reduced sizes for
    configs 2-4), printed, and within RMSD_TOL wherever the oracle's formula
    is well conditioned (check_rmsd)."""
    from pyjess_gb300 import workloads as W

    cases = [
        ("config 0", W.config(0), {}),
        ("config 1", W.config(1), {}),
        ("config 2 (40 x 300)", W.config(2, n_structures=40, n_templates=300), {}),
        ("config 3 (40 x 300)", W.config(3, n_structures=40, n_templates=300), {}),
        ("config 4 (3 x 6, best_match=False)", W.config(4, n_structures=3, n_templates=6, residues=(300, 500)),
         {"max_candidates": 50}),
        ("config 4 (3 x 6, best_match=True)", W.config(4, n_structures=3, n_templates=6, residues=(300, 500)),
         {"max_candidates": 50, "best_match": True}),
    ]
    lines = []
    for label, wl, extra in cases:
        p = dict(wl.params)
        p.update(extra)
        res, ref = compare(wl.templates, wl.structures, mode="fp32", **p)
        g = res.arrays()
        err = float(np.abs(g["rmsd"] - ref["hits"]["rmsd"]).max()) if g["count"] else 0.0
        lines.append(f"{label}: {g['count']} hits, identical; max |rmsd - oracle| = {err:.3g} A")
    with capsys.disabled():
        print("\n" + "\n".join(lines))
