"""The autotuner on the GPU: tuning knobs through the C ABI, a tuning run on
a small sample, and the tuned configuration's hits identical to the
oracle's."""

import os

import pytest

from helpers import hit_keys
from test_gpu_parity import check_rmsd

pytestmark = pytest.mark.gpu


def test_tuning_abi_defaults_and_range_checks():
    from pyjess_gb300 import _native, tune

    _native.set_tuning(None)
    assert _native.get_tuning() == tune.DEFAULTS
    _native.set_tuning({"block_min": 96, "pair_grain": 2})
    assert _native.get_tuning() == dict(tune.DEFAULTS, block_min=96, pair_grain=2)
    for bad in ({"tile_cap": 16}, {"pair_grain": 65}, {"leaf_levels": -2}, {"leaf_rank_max": 257},
                {"leaf_reach": -2}):
        with pytest.raises(RuntimeError, match="invalid"):
            _native.set_tuning(bad)
    # a rejected call changes nothing
    assert _native.get_tuning() == dict(tune.DEFAULTS, block_min=96, pair_grain=2)
    _native.set_tuning(None)
    assert "GB" in _native.device_name() or _native.device_name()


@pytest.mark.parametrize("tuning", [dict(leaf_levels=1, block_min=32, pair_grain=8, tile_cap=1024, leaf_rank_max=64,
                                         leaf_reach=1),
                                    dict(leaf_levels=-1, block_min=192, pair_grain=2, tile_cap=8192),
                                    dict(leaf_levels=6, block_min=48, pair_grain=4, leaf_rank_max=128, leaf_reach=2),
                                    dict(leaf_levels=2, leaf_reach=1)])
def test_every_tuning_gives_the_oracle_hits(tuning):
    from oracle import oracle
    from pyjess_gb300 import _native, workloads
    from test_gpu_parity import gpu_query

    wl = workloads.config(3, n_structures=30, n_templates=300)
    ref = oracle.query(wl.templates, wl.structures, threads=os.cpu_count() or 1, **wl.params)
    try:
        _native.set_tuning(tuning)
        res = gpu_query(wl.templates, wl.structures, mode="fp32", **wl.params)
        g = res.arrays()
    finally:
        _native.set_tuning(None)
    assert hit_keys(g) == hit_keys(ref["hits"])
    check_rmsd(g, ref["hits"], wl.templates, wl.structures)
    gs = res.stats()
    for key in ("pairs", "candidate_entries", "partials", "complete", "bytes_expansion"):
        assert gs[key] == ref["stats"][key], key


def test_autotune_sample_and_cache(tmp_path):
    from oracle import oracle
    from pyjess_gb300 import _native, tune, workloads
    from test_gpu_parity import gpu_query

    wl = workloads.config(3, n_structures=40, n_templates=300)
    path = tmp_path / "tuning.json"
    entry, source = tune.ensure(wl.templates, wl.structures, wl.params, tune=True, path=path,
                                sample_pairs=6000, passes=1, repeats=1)
    assert source == "tuned" and entry["ms"] <= entry["default_ms"]
    again, source2 = tune.ensure(wl.templates, wl.structures, wl.params, path=path)
    assert source2 == "cache" and again["tuning"] == entry["tuning"]
    try:
        tune.apply(entry)
        g = gpu_query(wl.templates, wl.structures, mode="fp32", **wl.params).arrays()
    finally:
        _native.set_tuning(None)
    ref = oracle.query(wl.templates, wl.structures, threads=os.cpu_count() or 1, **wl.params)["hits"]
    assert hit_keys(g) == hit_keys(ref)
