"""Full-size parity: the benchmarked workload against the CPU oracle.

Config 3 at the size the benchmark times (2,000 structures x 5,000
templates = 10 M pairs, FP32-guarded search with FP64 recheck) through
`pjg_query`, and the oracle on all host cores.  Bar, as in
test_gpu_parity.py: identical hit lists (structure, template, stream
ordinal, every atom, in order), identical NaN-rotation warnings, RMSD within
RMSD_TOL of the oracle (or of an SVD where the oracle's method is
ill-conditioned), centroids within 1e-9, rotations within ROT_TOL where the
fit is well conditioned (else within an SVD-Kabsch rotation) and optimal
everywhere.  Every comparison is vectorised; the few rows outside a
tolerance get the per-row SVD check.
"""

import os

import numpy as np
import pytest

from test_gpu_parity import RMSD_TOL, ROT_TOL, gpu_query, svd_rmsd

pytestmark = pytest.mark.gpu


def _hit_coords(h, ptemplates, pstructures, sel):
    """Molecule and template coordinates of hits `sel`: (rows, per-hit
    atom counts, mol xyz, tpl xyz), atoms of consecutive hits concatenated."""
    a0 = h["atom_offset"][sel]
    n = h["atom_offset"][sel + 1] - a0
    rows = np.repeat(np.arange(len(sel)), n)
    k = np.arange(n.sum()) - np.repeat(np.cumsum(n) - n, n)
    s = h["structure"][sel][rows].astype(np.int64)
    t = h["template"][sel][rows].astype(np.int64)
    mol = pstructures.xyz[pstructures.atom_offset[s] + h["atoms"][a0[rows] + k]]
    tpl = ptemplates.xyz[ptemplates.atom_offset[t] + k]
    return rows, n, mol, tpl


def compare_full(g, r, ptemplates, pstructures, chunk=1 << 19):
    """Vectorised form of test_gpu_parity.compare for millions of hits;
    returns a summary dict."""
    assert g["count"] == r["count"]
    for key in ("structure", "template", "ordinal", "atom_offset", "atoms"):
        assert np.array_equal(g[key], r[key]), key
    out = {"hits": int(g["count"]), "svd_rmsd_rows": 0, "svd_rotation_rows": 0, "max_rmsd_err": 0.0}
    if not g["count"]:
        return out
    err = np.abs(g["rmsd"] - r["rmsd"])
    out["max_rmsd_err"] = float(err.max())
    bad = np.flatnonzero(err > RMSD_TOL)
    for i in bad:
        _, _, mol, tpl = _hit_coords(g, ptemplates, pstructures, np.array([i]))
        exact, sv = svd_rmsd(mol, tpl)
        assert sv[2] < 1e-5 * sv[0], (i, err[i], sv)
        assert abs(g["rmsd"][i] - exact) <= RMSD_TOL, (i, g["rmsd"][i], exact)
    out["svd_rmsd_rows"] = int(len(bad))
    out["max_rmsd_err_outside_svd_rows"] = float(np.delete(err, bad).max()) if len(bad) < len(err) else 0.0
    assert np.abs(g["centres"] - r["centres"]).max() <= 1e-9
    R = g["rotation"].reshape(-1, 3, 3)
    assert np.abs(np.linalg.det(R) - 1.0).max() < 1e-9
    # optimal: the rotation reproduces the reported rmsd (every hit, in chunks)
    for c0 in range(0, g["count"], chunk):
        sel = np.arange(c0, min(c0 + chunk, g["count"]))
        rows, n, mol, tpl = _hit_coords(g, ptemplates, pstructures, sel)
        c = g["centres"][sel][rows]
        fit = np.einsum("nij,nj->ni", R[sel][rows], mol - c[:, :3]) + c[:, 3:]
        d2 = np.bincount(rows, weights=((fit - tpl) ** 2).sum(1), minlength=len(sel))
        rm = np.sqrt(d2 / n)
        worst = np.abs(rm - g["rmsd"][sel]).max()
        assert worst < 1e-7, (c0, worst)
    # equal to the oracle's rotation, except where the fit is ill-conditioned
    rerr = np.abs(g["rotation"] - r["rotation"]).max(1)
    for i in np.flatnonzero(rerr > ROT_TOL):
        _, _, mol, tpl = _hit_coords(g, ptemplates, pstructures, np.array([i]))
        if len(tpl) < 3:
            continue
        a, b = mol - mol.mean(0), tpl - tpl.mean(0)
        U, sv, Vt = np.linalg.svd(a.T @ b)
        cond = sv[2] / sv[0] if sv[0] > 0 else 0.0
        assert cond <= 1e-3, (i, rerr[i], cond)
        if cond > 1e-9:
            d = np.sign(np.linalg.det(Vt.T @ U.T))
            Rk = Vt.T @ np.diag([1, 1, d]) @ U.T
            assert np.abs(R[i] - Rk).max() <= 1e-12 / cond + 1e-9
        out["svd_rotation_rows"] += 1
    return out


def test_config3_full_size_identical_to_oracle():
    """The benchmarked workload itself: 10 M pairs, every hit."""
    from oracle import oracle
    from pyjess_gb300 import workloads

    wl = workloads.config(3)
    assert wl.pairs == 10_000_000
    res = gpu_query(wl.templates, wl.structures, mode="fp32", **wl.params)
    g = res.arrays()
    ref = oracle.query(wl.templates, wl.structures, threads=os.cpu_count() or 1, **wl.params)
    summary = compare_full(g, ref["hits"], wl.templates, wl.structures)
    gw = res.warnings()
    assert np.array_equal(gw[0], ref["warnings"][0]) and np.array_equal(gw[1], ref["warnings"][1])
    gs, os_ = res.stats(), ref["stats"]
    for key in ("pairs", "candidate_entries", "partials", "complete", "bytes_candidates", "bytes_expansion"):
        assert gs[key] == os_[key], (key, gs[key], os_[key])
    print(f"\nconfig 3 full size ({wl.pairs} pairs): {summary['hits']} hits identical to the oracle; "
          f"max |rmsd - oracle| = {summary['max_rmsd_err']:.3g} A "
          f"({summary['max_rmsd_err_outside_svd_rows']:.3g} A outside the {summary['svd_rmsd_rows']} "
          f"ill-conditioned rows checked against an SVD); {summary['svd_rotation_rows']} rotations checked "
          f"against SVD-Kabsch; {gs['fp64_rechecks']} FP64 rechecks; {len(gw[0])} warnings")


def test_config4_full_size_structures_best_match_strided():
    """Config 4 at its full structure sizes (2,000-5,000 residues), all 500
    permissive templates, max_candidates 10,000, best_match=True: every
    50th structure, searched together on the GPU and by the oracle."""
    from oracle import oracle
    from pyjess_gb300 import workloads

    wl = workloads.config(4)
    sub = wl.structures.subset(list(range(0, wl.structures.n_structures, 50)))
    p = dict(wl.params)
    assert p["max_candidates"] == 10000
    res = gpu_query(wl.templates, sub, mode="fp32", best_match=True, **p)
    g = res.arrays()
    ref = oracle.query(wl.templates, sub, threads=os.cpu_count() or 1, best_match=True, **p)
    summary = compare_full(g, ref["hits"], wl.templates, sub)
    gw = res.warnings()
    assert np.array_equal(gw[0], ref["warnings"][0]) and np.array_equal(gw[1], ref["warnings"][1])
    print(f"\nconfig 4 full-size structures, best_match=True ({sub.n_structures} x {wl.templates.n_templates}): "
          f"{summary['hits']} hits identical to the oracle; max |rmsd - oracle| = {summary['max_rmsd_err']:.3g} A")
