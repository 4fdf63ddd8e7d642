"""The autotuner's host logic on the CPU: shape keys, the JSON cache,
coordinate descent and the check that a tuned configuration keeps the hits
(with a stand-in runner instead of the GPU)."""

import json

import numpy as np
import pytest

from pyjess_gb300 import tune


def _workload(ns=6, nt=5):
    from pyjess_gb300 import workloads

    return workloads.config(3, n_structures=ns, n_templates=nt)


def test_shape_key_tracks_workload_and_options():
    wl = _workload()
    k = tune.shape_key(wl.templates, wl.structures, wl.params)
    assert k == tune.shape_key(wl.templates, wl.structures, dict(wl.params))
    assert k != tune.shape_key(wl.templates, wl.structures, dict(wl.params, best_match=True))
    assert k != tune.shape_key(wl.templates, wl.structures, dict(wl.params, max_candidates=10))
    assert k != tune.shape_key(wl.templates, wl.structures, dict(wl.params, distance_cutoff=3.0))
    wl2 = _workload(ns=24)
    assert k != tune.shape_key(wl2.templates, wl2.structures, wl2.params)


def test_cache_roundtrip_and_bad_files(tmp_path):
    path = tmp_path / "tuning.json"
    assert tune.load_cache(path) == {}
    entry = {"tuning": dict(tune.DEFAULTS, block_min=96), "ms": 1.0}
    tune.store("GPU A", "key1", entry, path)
    tune.store("GPU B", "key1", {"tuning": dict(tune.DEFAULTS)}, path)
    assert tune.lookup("GPU A", "key1", path)["tuning"]["block_min"] == 96
    assert tune.lookup("GPU A", "key2", path) is None
    assert tune.lookup("GPU C", "key1", path) is None
    # malformed entries are ignored, not trusted
    data = json.loads(path.read_text())
    data["GPU A"]["key3"] = {"tuning": {"block_min": "x"}}
    data["GPU A"]["key4"] = {"no": "tuning"}
    path.write_text(json.dumps(data))
    assert tune.lookup("GPU A", "key3", path) is None
    assert tune.lookup("GPU A", "key4", path) is None
    path.write_text("{not json")
    assert tune.load_cache(path) == {}
    assert tune.lookup("GPU A", "key1", path) is None


def test_cache_path_from_environment(tmp_path, monkeypatch):
    monkeypatch.setenv(tune.CACHE_ENV, str(tmp_path / "c.json"))
    assert tune.cache_path() == tmp_path / "c.json"
    monkeypatch.delenv(tune.CACHE_ENV)
    assert tune.cache_path() == tune.DEFAULT_CACHE


def test_sample_indices():
    assert tune.sample_indices(10, 5000, 10**9) == list(range(10))
    idx = tune.sample_indices(2000, 5000, 1_000_000)
    assert len(idx) == 200 and idx[0] == 0 and idx[1] == 10
    assert tune.sample_indices(1, 5000, 10) == [0]


def test_coordinate_descent_finds_separable_optimum():
    target = {"leaf_levels": 2, "block_min": 96, "pair_grain": 4, "tile_cap": 2048, "leaf_rank_max": 128,
              "leaf_reach": 2}

    def cost(cfg):
        return sum(abs(tune.SPACE[k].index(cfg[k]) - tune.SPACE[k].index(target[k])) for k in target) + 1.0

    best, t, trials = tune.coordinate_descent(cost)
    assert best == target and t == 1.0
    # every configuration timed once
    assert len({tuple(sorted(c.items())) for c, _ in trials}) == len(trials)


class FakeRunner:
    def __init__(self, best, change_hits=False):
        self.best, self.change_hits = best, change_hits

    def time(self, cfg):
        return 10.0 - 5.0 * all(cfg[k] == v for k, v in self.best.items())

    def hits(self, cfg):
        n = 3 + (1 if self.change_hits and cfg != tune.DEFAULTS else 0)
        return {"count": n, "rmsd": np.arange(n, dtype=float)}


def test_autotune_with_stand_in_runner():
    wl = _workload()
    entry = tune.autotune(wl.templates, wl.structures, wl.params, runner=FakeRunner({"block_min": 128}))
    assert entry["tuning"] == dict(tune.DEFAULTS, block_min=128)
    assert entry["ms"] == 5.0 and entry["default_ms"] == 10.0


def test_autotune_rejects_a_configuration_that_changes_hits():
    wl = _workload()
    with pytest.raises(RuntimeError, match="changed the hits"):
        tune.autotune(wl.templates, wl.structures, wl.params, runner=FakeRunner({"pair_grain": 4}, True))
