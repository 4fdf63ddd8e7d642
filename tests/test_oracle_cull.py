"""The oracle's culling-scheme counts (instrumentation of its kd range
queries, not part of the reference's algorithm): for each query on a list of
64 or more points, the points a search would load by 32-leaf block culling
and by uniform grids, against the points in the join box and the results.
They leave the hits unchanged and satisfy the containments the schemes
imply."""

import os

from oracle import oracle
from pyjess_gb300 import workloads as W


def test_cull_counts():
    wl = W.config(3, n_structures=4, n_templates=200)
    threads = min(8, os.cpu_count() or 1)
    r = oracle.query(wl.templates, wl.structures, threads=threads, cull_stats=True, **wl.params)
    plain = oracle.query(wl.templates, wl.structures, threads=threads, **wl.params)
    assert r["hits"]["count"] == plain["hits"]["count"]
    assert (r["hits"]["atoms"] == plain["hits"]["atoms"]).all()
    assert "cull" not in plain
    c = r["cull"]
    assert c["queries"] > 0
    # results lie in the join box; block culling loads every point of the
    # blocks the box meets, so at least those inside it, and at most all
    assert 0 < c["children"] <= c["in_box"] <= c["block_loaded"] <= c["points"]
    assert c["blocks_hit"] * 32 >= c["block_loaded"] >= c["blocks_hit"]
    # the 8-leaf sub-blocks that meet the box lie in the blocks that do
    assert c["in_box"] <= c["sub_loaded"] <= c["block_loaded"] and c["sub_hit"] <= 4 * c["blocks_hit"]
    # sibling groups: every query belongs to exactly one, and a group's
    # union box meets at least one block (each member's results lie in it)
    assert c["group_members"] == c["queries"] and 0 < c["groups"] <= c["queries"]
    assert c["groups"] <= c["group_blocks_hit"] <= 32 * c["group_loaded"]
    cells = [c["grid"][g]["cells"] for g in oracle.CULL_GRID]
    for g in oracle.CULL_GRID:
        assert c["in_box"] <= c["grid"][g]["loaded"] <= c["points"]
    assert cells == sorted(cells, reverse=True)
