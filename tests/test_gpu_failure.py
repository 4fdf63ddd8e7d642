"""Failure paths on the GPU, in forms that fault, trap or hang nothing.

The search kernel carries a wall-time budget (PJG_KERNEL_BUDGET_S, read at
each query): every warp checks the global timer in its work loop and stops
once the budget is spent, the kernel returns on its own, and the host
reports PJG_ERR_TIMEOUT.  The test makes the budget run out with a tiny
value, then checks that the library (same process, same context) still
answers a normal query with the oracle's hits.
"""

import os

import pytest

from helpers import hit_keys
from test_gpu_parity import check_rmsd

pytestmark = pytest.mark.gpu


def _query(wl):
    from pyjess_gb300 import _native
    from pyjess_gb300._abi import QueryParams

    P = QueryParams(rmsd_threshold=wl.params["rmsd_threshold"], distance_cutoff=wl.params["distance_cutoff"],
                    max_dynamic_distance=wl.params["max_dynamic_distance"], max_candidates=-1, ignore_chain=0,
                    best_match=0, reorder=1, mode=_native.MODE_BATCHED_FP32)
    return _native.query(_native.Templates(wl.templates), _native.Structures(wl.structures), P)


def test_time_budget_returns_timeout_and_library_stays_usable(monkeypatch):
    from oracle import oracle
    from pyjess_gb300 import workloads

    wl = workloads.config(3, n_structures=20, n_templates=300)
    monkeypatch.setenv("PJG_KERNEL_BUDGET_S", "1e-6")
    with pytest.raises(RuntimeError, match="timeout"):
        _query(wl)
    monkeypatch.delenv("PJG_KERNEL_BUDGET_S")
    res = _query(wl).arrays()
    ref = oracle.query(wl.templates, wl.structures, threads=os.cpu_count() or 1, **wl.params)["hits"]
    assert res["count"] == ref["count"] > 0
    assert hit_keys(res) == hit_keys(ref)
    check_rmsd(res, ref, wl.templates, wl.structures)
