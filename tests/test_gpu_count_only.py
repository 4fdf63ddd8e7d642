"""Count-only queries (pjg_query_params.count_only): the same hit, atom and
warning counts and search counters as the query that keeps its hits, on
the dense-hit workload (permissive templates) in both best_match modes,
against the oracle's counts; copying hits out of a count-only result is
refused."""

import os

import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("best", [False, True])
def test_count_only_matches_materialised(best):
    from oracle import oracle
    from pyjess_gb300 import _native, workloads as W
    from pyjess_gb300._abi import QueryParams

    wl = W.config(4, n_structures=3, n_templates=6, residues=(300, 500))
    p = dict(wl.params)
    p["max_candidates"] = 50

    def params(count_only):
        return QueryParams(rmsd_threshold=p["rmsd_threshold"], distance_cutoff=p["distance_cutoff"],
                           max_dynamic_distance=p["max_dynamic_distance"], max_candidates=p["max_candidates"],
                           ignore_chain=0, best_match=int(best), reorder=1, mode=_native.MODE_BATCHED_FP32,
                           count_only=count_only)

    tpl, sts = _native.Templates(wl.templates), _native.Structures(wl.structures)
    full = _native.query(tpl, sts, params(0))
    counted = _native.query(tpl, sts, params(1))
    L = _native.load()
    assert L.pjg_results_count(counted.handle) == L.pjg_results_count(full.handle) > 0
    assert L.pjg_results_atom_count(counted.handle) == L.pjg_results_atom_count(full.handle)
    assert L.pjg_results_warning_count(counted.handle) == L.pjg_results_warning_count(full.handle)
    a, b = full.stats(), counted.stats()
    for k in ("pairs", "partials", "complete", "passing", "hits", "bytes_expansion"):
        assert a[k] == b[k], k
    ref = oracle.query(wl.templates, wl.structures, threads=os.cpu_count() or 1, best_match=best, **p)
    assert L.pjg_results_count(counted.handle) == ref["hits"]["count"]
    with pytest.raises(RuntimeError, match="count-only"):
        counted.arrays()
