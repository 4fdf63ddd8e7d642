"""Autotuner of the GPU search's execution knobs (``pjg_tuning``).

A batched query moves work between its kernels through a few knobs that
change no result: how many levels of candidate lists get their kd leaf
order before the search (the rest on demand, at the price of suspending
and resuming the pairs that reach them), the list length from which the
search expands one parent at a time with block culling, the frontier tile
capacity, how many pairs a search warp takes from the work queue at once,
and the longest list ordered by the rank method.  The best values depend on
the GPU and on the shape of the workload (template sizes, structure sizes,
distance cutoff), so they are measured, not fixed.

`autotune` times ``pjg_query`` (device time, CUDA events) on a strided sample
of the workload's structures against all of its templates, for the candidate
values of one knob at a time with the others held at the best found so far
(coordinate descent, two passes), keeps the fastest configuration, checks
that it returns exactly the hits of the default configuration on the sample,
and stores it in a JSON cache keyed by the GPU's name and the workload's
shape key.  `ensure` returns the cached entry for a workload, tuning on a
miss when asked to, and `apply` sets it for the queries that follow.

The reference has nothing to tune: its search is one CPU thread per query.
"""

from __future__ import annotations

import json
import math
import os
import pathlib
import time

import numpy as np

DEFAULTS = {"leaf_levels": 4, "block_min": 64, "tile_cap": 4096, "pair_grain": 1, "leaf_rank_max": 256,
            "leaf_reach": -1}
# candidate values per knob, searched in this order
SPACE = {
    "leaf_reach": [-1, 1, 2, 3],
    "leaf_levels": [1, 2, 3, 4, 5, 6, -1],
    "block_min": [32, 48, 64, 96, 128, 192],
    "pair_grain": [1, 2, 4, 8],
    "tile_cap": [1024, 2048, 4096, 8192],
    "leaf_rank_max": [64, 128, 192, 256],
}
CACHE_ENV = "PJG_TUNING_CACHE"
DEFAULT_CACHE = pathlib.Path(__file__).resolve().with_name("tuning.json")


def cache_path(path=None) -> pathlib.Path:
    if path is not None:
        return pathlib.Path(path)
    env = os.environ.get(CACHE_ENV)
    return pathlib.Path(env) if env else DEFAULT_CACHE


def _bucket(x: int) -> int:
    """Power-of-two bucket of a count (0 for 0)."""
    return 0 if x <= 0 else 1 << int(round(math.log2(x)))


def shape_key(ptemplates, pstructures, params: dict) -> str:
    """Key of the workload's shape: template count and median size,
    structure count and median size (buckets), distance cutoff, and the
    query options that change the search (best_match, max_candidates)."""
    na = np.diff(np.asarray(ptemplates.atom_offset))
    ns = np.diff(np.asarray(pstructures.atom_offset))
    med_t = int(np.median(na)) if len(na) else 0
    med_s = int(np.median(ns)) if len(ns) else 0
    mc = params.get("max_candidates")
    return (f"T{_bucket(ptemplates.n_templates)}-n{med_t}-S{_bucket(pstructures.n_structures)}"
            f"-N{_bucket(med_s)}-r{float(params['distance_cutoff']):g}"
            f"-b{int(bool(params.get('best_match', False)))}-m{-1 if mc is None else int(mc)}")


def load_cache(path=None) -> dict:
    """The cache as a dict (empty when the file is missing or unreadable)."""
    p = cache_path(path)
    try:
        with open(p) as f:
            data = json.load(f)
        return data if isinstance(data, dict) else {}
    except (OSError, ValueError):
        return {}


def save_cache(cache: dict, path=None) -> pathlib.Path:
    """Write the cache atomically (temporary file, then rename)."""
    p = cache_path(path)
    tmp = p.with_name(p.name + f".tmp{os.getpid()}")
    with open(tmp, "w") as f:
        json.dump(cache, f, indent=1, sort_keys=True)
        f.write("\n")
    os.replace(tmp, p)
    return p


def lookup(gpu: str, key: str, path=None):
    """The cached entry for (gpu, key), or None."""
    entry = load_cache(path).get(gpu, {}).get(key)
    if not isinstance(entry, dict) or "tuning" not in entry:
        return None
    t = entry["tuning"]
    if set(t) != set(DEFAULTS) or not all(isinstance(v, int) for v in t.values()):
        return None
    return entry


def store(gpu: str, key: str, entry: dict, path=None) -> pathlib.Path:
    cache = load_cache(path)
    cache.setdefault(gpu, {})[key] = entry
    return save_cache(cache, path)


def sample_indices(n_structures: int, n_templates: int, sample_pairs: int) -> list:
    """Every k-th structure, so that the sample holds about `sample_pairs`
    pairs with all templates (all structures when the workload is smaller)."""
    want = max(1, min(n_structures, int(round(sample_pairs / max(1, n_templates)))))
    stride = max(1, n_structures // want)
    return list(range(0, n_structures, stride))[:want]


def coordinate_descent(time_of, space=SPACE, start=DEFAULTS, passes=2):
    """Minimise `time_of(config)` one knob at a time.  Returns (best config,
    its time, every trial as (config, time)); each config is timed once."""
    seen = {}

    def timed(cfg):
        k = tuple(sorted(cfg.items()))
        if k not in seen:
            seen[k] = time_of(dict(cfg))
        return seen[k]

    best = dict(start)
    best_t = timed(best)
    for _ in range(passes):
        changed = False
        for knob, values in space.items():
            for v in values:
                if v == best[knob]:
                    continue
                cfg = dict(best, **{knob: v})
                t = timed(cfg)
                if t < best_t:
                    best, best_t, changed = cfg, t, True
        if not changed:
            break
    trials = [(dict(k), t) for k, t in seen.items()]
    return best, best_t, trials


class _NativeRunner:
    """Times pjg_query on the device for a given tuning."""

    def __init__(self, ptemplates, pstructures, params, repeats):
        from . import _native
        from ._abi import QueryParams

        self._native = _native
        self.templates = _native.Templates(ptemplates)
        self.structures = _native.Structures(pstructures)
        mc = params.get("max_candidates")
        self.P = QueryParams(rmsd_threshold=params["rmsd_threshold"], distance_cutoff=params["distance_cutoff"],
                             max_dynamic_distance=params["max_dynamic_distance"],
                             max_candidates=-1 if mc is None else int(mc), ignore_chain=int(params.get("ignore_chain", 0)),
                             best_match=int(bool(params.get("best_match", False))),
                             reorder=int(params.get("reorder", True)), mode=_native.MODE_BATCHED_FP32,
                             guard_band=1e-4)
        self.repeats = repeats

    def time(self, tuning: dict) -> float:
        self._native.set_tuning(tuning)
        self._native.query(self.templates, self.structures, self.P)  # warm-up
        return min(self._native.query(self.templates, self.structures, self.P).stats()["ms_total"]
                   for _ in range(self.repeats))

    def hits(self, tuning: dict) -> dict:
        self._native.set_tuning(tuning)
        return self._native.query(self.templates, self.structures, self.P).arrays()


def same_hits(a: dict, b: dict) -> bool:
    if a["count"] != b["count"]:
        return False
    return all(np.array_equal(a[k], b[k]) for k in a if k != "count")


def autotune(ptemplates, pstructures, params: dict, *, sample_pairs: int = 1_000_000, passes: int = 2,
             repeats: int = 2, runner=None) -> dict:
    """Tune on a strided sample of `pstructures` (all templates); returns the
    cache entry {"tuning", "ms", "default_ms", "trials", "sample", "when"}.
    Raises RuntimeError if the tuned configuration's hits on the sample
    differ from the defaults' (the knobs must not change any result)."""
    from . import _native

    idx = sample_indices(pstructures.n_structures, ptemplates.n_templates, sample_pairs)
    sub = pstructures.subset(idx) if len(idx) < pstructures.n_structures else pstructures
    run = runner or _NativeRunner(ptemplates, sub, params, repeats)
    previous = _native.get_tuning() if runner is None else None
    t0 = time.perf_counter()
    try:
        best, best_ms, trials = coordinate_descent(run.time, passes=passes)
        default_ms = [t for c, t in trials if c == DEFAULTS][0]
        if best != DEFAULTS and not same_hits(run.hits(best), run.hits(DEFAULTS)):
            raise RuntimeError(f"tuned configuration {best} changed the hits of the sample")
    finally:
        if previous is not None:
            _native.set_tuning(previous)
    return {
        "tuning": best,
        "ms": best_ms,
        "default_ms": default_ms,
        "trials": len(trials),
        # every configuration timed: the knobs that differ from the
        # defaults, and its device milliseconds
        "timed": [[{k: v for k, v in c.items() if v != DEFAULTS[k]}, round(t, 3)] for c, t in trials],
        "sample": f"{len(idx)} of {pstructures.n_structures} structures x {ptemplates.n_templates} templates",
        "tune_s": round(time.perf_counter() - t0, 1),
        "when": time.strftime("%Y-%m-%dT%H:%M:%SZ", time.gmtime()),
    }


def ensure(ptemplates, pstructures, params: dict, *, tune: bool = False, path=None, **kw):
    """The tuning for this GPU and workload: (entry, source) with source
    "cache", "tuned" (measured now and stored) or "default" (no entry and
    `tune` false; entry None)."""
    from . import _native

    gpu = _native.device_name()
    key = shape_key(ptemplates, pstructures, params)
    entry = lookup(gpu, key, path)
    if entry is not None:
        return entry, "cache"
    if not tune:
        return None, "default"
    entry = autotune(ptemplates, pstructures, params, **kw)
    store(gpu, key, entry, path)
    return entry, "tuned"


def apply(entry) -> dict:
    """Set `entry`'s tuning (None: the defaults) for the queries that follow."""
    from . import _native

    _native.set_tuning(None if entry is None else entry["tuning"])
    return _native.get_tuning()
