"""Benchmark: template x structure pairs per second on one GB300.

Workload (config 3 of the synthetic suite): 5,000 synthetic templates (Zipf 2-8 residues x
3 atoms) against 2,000 synthetic structures (lognormal lengths, median 350
residues, 1-4 chains, 200 adversarial structures with distances within
1e-6 A of annulus boundaries) = 10,000,000 pairs per step, batched,
FP32-guarded distance tests with FP64 recheck.

  value       pairs/s of pjg_query with templates and structures already
              resident on the device (device time from CUDA events on the
              query's stream)
  e2e         the same metric through the C ABI with host buffers: per step
              pjg_templates_create + pjg_structures_create (H2D), pjg_query,
              pjg_results_copy (D2H), wall clock
  roofline    k_search (the expansion kernel): algorithmic expansion bytes /
              kernel time against the measured HBM copy bandwidth
  cpu_baseline  the CPU oracle (a port of the reference's algorithm) on the
              host cores, on a bounded sample of the same workload

`--impl reference` times that CPU implementation alone on this workload
(bounded sample per step).  Under torchrun (N>1) every rank runs its own
config-3 instance (independent pairs: weak scaling, no data-path
collective); the step time is the maximum over ranks (gloo all-reduce) and
rank 0 prints one JSON line.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "template·structure pairs/s on 1 GB300: batched+FP32-guarded vs plain, same hits"
UNIT = "pairs/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--config", type=int, default=3, choices=[2, 3],
                    help="workload: 3 (default, 2,000 x 5,000) or 2 (1,000 x 2,000)")
    ap.add_argument("--structures", type=int, default=0, help="structures (0: the configuration's)")
    ap.add_argument("--templates", type=int, default=0, help="templates (0: the configuration's)")
    ap.add_argument("--cpu-stride", type=int, default=31,
                    help="the CPU arms time every k-th structure (all templates)")
    ap.add_argument("--plain-structures", type=int, default=-1,
                    help="structures run through the plain FP64 per-structure path (-1: all, 0: none)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--tune", action="store_true",
                    help="run the autotuner when the tuning cache has no entry for this GPU and workload "
                         "(else the cached entry, or the defaults, are used)")
    ap.add_argument("--default-tuning", action="store_true", help="ignore the tuning cache")
    ap.add_argument("--ingest-files", type=int, default=200,
                    help="PDB files read back for the ingestion measurement (0: skip)")
    ap.add_argument("--search-profile", action="store_true",
                    help="run the search-profile build of the library and print k_search's event counts "
                         "and section cycles (not a bench line)")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = max(mx, float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return json.load(f), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def workload(args, rank=0, world=1):
    """This rank's share of a multi-GPU run: rank 0 takes the configuration
    itself, rank r an independent instance drawn with the same distributions
    (weak scaling: the pairs of every rank are independent, no data-path
    collective)."""
    from pyjess_gb300 import workloads as W

    return W.config(args.config, n_structures=args.structures or None, n_templates=args.templates or None,
                    shard=rank if world > 1 else 0)


def max_over_ranks(value, dist):
    """The largest `value` over all ranks (gloo all-reduce), or `value`."""
    if dist is None:
        return value
    import torch

    t = torch.tensor([float(value)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def cpu_structures(wl, stride):
    """The CPU arms' sample: every `stride`-th structure (ordinary and
    adversarial ones in the set's proportions) against every template."""
    return list(range(0, wl.structures.n_structures, max(1, stride)))


def cpu_sample(wl, idx, threads):
    """Time the CPU oracle on structures `idx` x all templates; returns
    (pairs/s, seconds, pairs, hits, boundary counts of the adversarial and
    of the ordinary structures of the sample).  The two groups run as two
    oracle calls, timed together."""
    from oracle import oracle

    groups = [[i for i in idx if i < wl.n_adversarial], [i for i in idx if i >= wl.n_adversarial]]
    dt, hits, boundary = 0.0, 0, []
    for g in groups:
        if not g:
            boundary.append({"tests": 0, "near": 0})
            continue
        sub = wl.structures.subset(g)
        t0 = time.perf_counter()
        r = oracle.query(wl.templates, sub, threads=threads, **wl.params)
        dt += time.perf_counter() - t0
        hits += r["hits"]["count"]
        boundary.append(r["boundary"])
    pairs = wl.templates.n_templates * len(idx)
    return pairs / dt, dt, pairs, hits, boundary


def sample_text(wl, idx, stride):
    pairs = len(idx) * wl.templates.n_templates
    n_adv = wl.n_adversarial
    return (f"every {stride}th structure ({len(idx)} of {wl.structures.n_structures}, "
            f"{sum(1 for i in idx if i < n_adv)} of them adversarial) x {wl.templates.n_templates} templates = "
            f"{pairs} pairs per step; pairs/s of the sample stands for the whole set")


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    wl = workload(args)
    threads = os.cpu_count() or 1
    idx = cpu_structures(wl, args.cpu_stride)
    vals = []
    for i in range(args.warmup + args.steps):
        v, dt, pairs, hits, _ = cpu_sample(wl, idx, threads)
        if i >= args.warmup:
            vals.append(v)
    value = statistics.median(vals)
    sample = sample_text(wl, idx, args.cpu_stride)
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 0,
        "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": wl.name, "pairs": wl.pairs, "sample": sample},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "notes": "the reference's C core cannot be built (empty vendor/jess submodule); the oracle port "
                 "restating its algorithm runs on all host cores",
    }))


def pdb_text(ps, s: int) -> str:
    """PDB ATOM records of packed structure `s` (the columns the reader takes)."""
    a0, a1 = int(ps.atom_offset[s]), int(ps.atom_offset[s + 1])
    dec = lambda b: bytes(b).replace(b"_", b" ").replace(b"\0", b" ").decode()
    lines = []
    for i in range(a0, a1):
        x, y, z = ps.xyz[i]
        ch = bytes(ps.chain[i]).decode()
        lines.append(f"ATOM  {int(ps.serial[i]):5d} {dec(ps.name[i])} {dec(ps.resname[i])[:3]}{ch}"
                     f"{int(ps.res_seq[i]):4d}    {x:8.3f}{y:8.3f}{z:8.3f}  1.00  0.00          "
                     f"{dec(ps.name[i]).strip()[:1]:>2}  \n")
    return "".join(lines) + "END\n"


def ingestion(wl, tpl, P, n_files: int, threads: int):
    """Structure ingestion in front of the query: `n_files` structures
    written as PDB files, read back with Molecule.load (the native record
    reader, on `threads` host threads), packed and uploaded
    (pjg_structures_create), then queried.  The general Python reader is
    timed on a few of the files for comparison."""
    import concurrent.futures
    import tempfile

    from pyjess_gb300 import Molecule, _io, _native
    from pyjess_gb300._pack import pack_molecules

    idx = list(range(wl.n_adversarial, min(wl.structures.n_structures, wl.n_adversarial + n_files)))
    with tempfile.TemporaryDirectory() as d:
        paths = []
        for s in idx:
            path = os.path.join(d, f"s{s}.pdb")
            with open(path, "w") as f:
                f.write(pdb_text(wl.structures, s))
            paths.append(path)
        atoms = int(sum(wl.structures.atom_offset[s + 1] - wl.structures.atom_offset[s] for s in idx))
        t0 = time.perf_counter()
        with concurrent.futures.ThreadPoolExecutor(max_workers=threads) as pool:
            mols = list(pool.map(Molecule.load, paths))
        t1 = time.perf_counter()
        packed = pack_molecules(mols)
        t2 = time.perf_counter()
        sts = _native.Structures(packed)
        t3 = time.perf_counter()
        res = _native.query(tpl, sts, P)
        q_ms = res.stats()["ms_total"]
        k = min(10, len(paths))
        t4 = time.perf_counter()
        for path in paths[:k]:
            with open(path) as f:
                _io.parse_pdb(f)
        py_ms = (time.perf_counter() - t4) / k * 1e3
    n = len(paths)
    return {"structures": n, "atoms": atoms, "threads": threads,
            "load_ms_per_structure": (t1 - t0) / n * 1e3, "atoms_per_s": atoms / (t1 - t0),
            "pack_ms": (t2 - t1) * 1e3, "structures_create_ms": (t3 - t2) * 1e3, "query_ms": q_ms,
            "python_reader_ms_per_structure": py_ms,
            "note": "Molecule.load of PDB files (native record reader) on host threads, then pack_molecules and "
                    "pjg_structures_create, against the device query of the same structures x all templates"}


def query_params(wl, mode, guard_band=1e-4):
    from pyjess_gb300._abi import QueryParams

    return QueryParams(rmsd_threshold=wl.params["rmsd_threshold"], distance_cutoff=wl.params["distance_cutoff"],
                       max_dynamic_distance=wl.params["max_dynamic_distance"], max_candidates=-1, ignore_chain=0,
                       best_match=0, reorder=1, mode=mode, guard_band=guard_band)


def same_arrays(a, b):
    """Every field of two hit-array dicts equal (bit for bit)."""
    import numpy as np

    if a["count"] != b["count"]:
        return False
    return all(np.array_equal(a[k], b[k]) for k in a if k != "count")


def search_profile(args):
    """k_search's event counts and section cycles on this workload, from the
    search-profile build of the library (one query after one warm-up)."""
    import tempfile

    variant = os.environ.get("PJG_PROF_VARIANT", "prof")
    os.environ["PJG_LIB_VARIANT"] = variant
    from pyjess_gb300 import _build, _native

    _build.build(variant=variant)
    _native.init(dist_env()[2])
    wl = workload(args)
    tpl = _native.Templates(wl.templates)
    sts = _native.Structures(wl.structures)
    P = query_params(wl, _native.MODE_BATCHED_FP32)
    _native.query(tpl, sts, P).arrays()
    with tempfile.NamedTemporaryFile("r", suffix=".jsonl") as f:
        os.environ["PJG_PROF_OUT"] = f.name
        st = _native.query(tpl, sts, P).stats()
        prof = json.loads(f.read().strip().splitlines()[-1])
    pairs_run = prof["pairs"] - prof["empty"]
    derived = {
        "cycles_per_pair_run": prof["cyc_pair"] / max(1, pairs_run),
        "share_setup": prof["cyc_setup"] / max(1, prof["cyc_pair"]),
        "share_seed": prof["cyc_seed"] / max(1, prof["cyc_pair"]),
        "share_block": prof["cyc_block"] / max(1, prof["cyc_pair"]),
        "share_product": prof["cyc_prod"] / max(1, prof["cyc_pair"]),
        "share_emit": prof["cyc_emit"] / max(1, prof["cyc_pair"]),
        "share_block_chain": prof["cyc_chain"] / max(1, prof["cyc_pair"]),
        "share_block_batch": prof["cyc_batch"] / max(1, prof["cyc_pair"]),
        "share_control": prof["cyc_ctrl"] / max(1, prof["cyc_pair"]),
        "share_suspend": prof["cyc_susp"] / max(1, prof["cyc_pair"]),
        "blocks_hit_per_tested": prof["blocks_hit"] / max(1, prof["blocks_tested"]),
        "inbox_per_leaf_loaded": prof["leaves_inbox"] / max(1, 32 * prof["blocks_hit"]),
        "children_per_block_test": prof["child_block"] / max(1, prof["batch_lanes"]),
        "lanes_per_batch": prof["batch_lanes"] / max(1, prof["batches"]),
        "children_per_product_test": prof["child_prod"] / max(1, prof["prod_lanes"]),
        "lanes_per_product_batch": prof["prod_lanes"] / max(1, prof["prod_batches"]),
        "block_visits_per_partial": prof["block_visits"] / max(1, st["partials"]),
        # the launches' tails (queue empty to last warp out) against the
        # expansion time, and the longest single pair (at 2.07 GHz)
        "tail_share_of_expansion": prof.get("tail_ns", 0) / max(1.0, st["ms_expansion"] * 1e6),
        "longest_pair_us": prof.get("pair_max_cyc", 0) / 2070.0,
    }
    lo = prof.get("leaf_order")
    if lo:
        cyc = max(1, lo["cyc_list"])
        derived["leaf_order"] = {
            "warp_cycles_per_entry": lo["cyc_list"] / max(1, lo["entries"]),
            **{f"share_{k}": lo[f"cyc_{k}"] / cyc for k in ("load", "sort", "count", "seg", "write")},
            "sort_words_per_node": lo["sort_words"] / max(1, lo["sort_nodes"]),
            "count_pairs_per_entry": lo["count_pairs"] / max(1, lo["entries"]),
            "class_cycles_per_entry": [c / max(1, e) for c, e in zip(lo["class_cycles"], lo["class_entries"])],
            "class_entry_share": [e / max(1, lo["entries"]) for e in lo["class_entries"]],
        }
    print(json.dumps({"search_profile": prof, "derived": derived, "workload": wl.name,
                      "partials": st["partials"], "complete": st["complete"],
                      "ms_expansion_profile_build": st["ms_expansion"]}))


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.search_profile:
        return search_profile(args)
    rank, world, local = dist_env()
    import __graft_entry__

    __graft_entry__.build()
    from pyjess_gb300 import _native

    _native.init(local)
    dist = None
    if world > 1:
        import torch.distributed as dist_mod

        dist_mod.init_process_group("gloo")
        dist = dist_mod
    t0 = time.time()
    wl = workload(args, rank, world)
    gen_s = time.time() - t0
    P = query_params(wl, _native.MODE_BATCHED_FP32)
    # execution tuning: the cached entry for this GPU and workload shape
    # (autotuned on a sample of the workload when --tune finds none)
    from pyjess_gb300 import tune

    if args.default_tuning:
        entry, source = None, "default"
    else:
        entry, source = tune.ensure(wl.templates, wl.structures, wl.params, tune=args.tune)
    tuning = {"values": tune.apply(entry), "source": source,
              "key": tune.shape_key(wl.templates, wl.structures, wl.params)}
    if entry is not None:
        tuning.update({k: entry[k] for k in ("sample", "ms", "default_ms") if k in entry})
    tpl = _native.Templates(wl.templates)
    sts = _native.Structures(wl.structures)

    # ---- device-resident timing
    for _ in range(args.warmup):
        res = _native.query(tpl, sts, P)
        res.arrays()
    if dist:
        dist.barrier()
    step_ms, stats, launches = [], [], 0
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            res = _native.query(tpl, sts, P)
            st = res.stats()
            stats.append(st)
            step_ms.append(st["ms_total"])
            launches += st["launches"]
            arr = res.arrays()
    total_ms = max_over_ranks(sum(step_ms), dist)
    pairs_step = wl.pairs
    value = pairs_step * world * args.steps / (total_ms / 1e3)
    s0 = stats[-1]
    hits_per_s = s0["hits"] * world * args.steps / (total_ms / 1e3)

    # ---- roofline of the expansion kernel (k_search)
    peaks, peak_kind = measured_peaks()
    exp_ms = sum(s["ms_expansion"] for s in stats)
    exp_bytes = sum(s["bytes_expansion"] for s in stats)
    achieved = exp_bytes / (exp_ms / 1e3) / 1e9 if exp_ms > 0 else 0.0
    peak = float(peaks["hbm_gbs"])
    traffic, issue = None, None
    tpath = os.path.join(ROOT, "profiles", "k_search_traffic.json")
    if os.path.exists(tpath):
        with open(tpath) as f:
            tr = json.load(f)
        # the resource that binds k_search: issue slots (ncu, same capture)
        if tr.get("issue_active_frac") is not None:
            issue = {"frac": tr["issue_active_frac"], "frac_first_round": tr.get("issue_active_frac_first_round"),
                     "warp_inst_per_partial": tr.get("warp_inst_per_partial"),
                     "source": "ncu smsp__issue_active.avg.pct_of_peak_sustained_active and sm__inst_executed.sum "
                               "of the k_search launches of a 20 x 5,000 query (profiles/k_search_traffic.json)"}
        # DRAM bytes per algorithmic expansion byte, measured by ncu over the
        # k_search launches of one query of a smaller case, times the
        # expansion bytes of an average launch of this workload
        if tr.get("dram_per_expansion_byte"):
            launches_k = max(1, sum(s["search_rounds"] for s in stats))
            traffic = tr["dram_per_expansion_byte"] * exp_bytes / launches_k

    # ---- plain FP64 per-structure path (the method the batched path is
    # measured against) over the structures asked for (default: all), its
    # hits compared field by field with the batched query's
    plain = None
    if args.plain_structures != 0 and rank == 0:
        ns = wl.structures.n_structures
        k = ns if args.plain_structures < 0 else min(args.plain_structures, ns)
        Pp = query_params(wl, _native.MODE_PLAIN_FP64)
        if k == ns:
            ssub, batched = sts, arr
        else:
            ssub = _native.Structures(wl.structures.subset(list(range(k))))
            batched = _native.query(tpl, ssub, P).arrays()
        rp = _native.query(tpl, ssub, Pp)
        ms = rp.stats()["ms_total"]
        plain = {"value": wl.templates.n_templates * k / (ms / 1e3), "unit": UNIT, "structures": k,
                 "ms": ms, "identical_to_batched": same_arrays(rp.arrays(), batched),
                 "compared": "every field of every hit (structure, template, ordinal, atoms, rmsd, rotation, "
                             "centres), bit for bit"}
        del rp

    # ---- end to end through the C ABI with host buffers
    e2e = None
    if not args.no_e2e:
        h2d = wl.structures.nbytes() + sum(getattr(wl.templates, f).nbytes for f in (
            "atom_offset", "code", "res_seq", "chain", "xyz", "dist_weight", "name_offset", "names",
            "resname_offset", "resnames", "dim"))
        times, d2h = [], 0
        phases = {"templates_create": 0.0, "structures_create": 0.0, "query": 0.0, "results_copy": 0.0}
        for i in range(args.warmup + args.steps):
            t1 = time.perf_counter()
            tp2 = _native.Templates(wl.templates)
            t2 = time.perf_counter()
            st2 = _native.Structures(wl.structures)
            t3 = time.perf_counter()
            r2 = _native.query(tp2, st2, P)
            t4 = time.perf_counter()
            a2 = r2.arrays()
            t5 = time.perf_counter()
            del tp2, st2
            dt = time.perf_counter() - t1
            if i >= args.warmup:
                times.append(dt)
                for k, v in zip(phases, (t2 - t1, t3 - t2, t4 - t3, t5 - t4)):
                    phases[k] += 1e3 * v / args.steps
            d2h = sum(v.nbytes for k, v in a2.items() if hasattr(v, "nbytes"))
        tot = max_over_ranks(sum(times), dist)
        e2e = {"value": pairs_step * world * args.steps / tot, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h), "phases_ms": {k: round(v, 1) for k, v in phases.items()}}

    # ---- CPU baseline (rank 0, N=1): the same strided sample as the
    # reference arm, median of three runs
    cpu, boundary = None, None
    if rank == 0 and world == 1 and not args.no_cpu:
        threads = os.cpu_count() or 1
        idx = cpu_structures(wl, args.cpu_stride)
        runs = [cpu_sample(wl, idx, threads) for _ in range(3)]
        v = statistics.median(r[0] for r in runs)
        cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": sample_text(wl, idx, args.cpu_stride) + f" (median of 3 runs of "
                                                                  f"{statistics.median(r[1] for r in runs):.1f} s)"}
        # adversarial structures: share of the candidate-pair distance tests
        # (the kd range queries' annulus tests, counted by the oracle on the
        # sample) within 1e-6 A of an annulus boundary, against the ordinary
        # structures of the same sample
        adv, ordn = runs[0][4]
        if wl.n_adversarial:
            boundary = {
                "adversarial_structures": wl.n_adversarial,
                "near_boundary_fraction_adversarial": adv["near"] / max(1, adv["tests"]),
                "near_boundary_fraction_ordinary": ordn["near"] / max(1, ordn["tests"]),
                "tests_adversarial": adv["tests"], "tests_ordinary": ordn["tests"],
                "measured_on": "the CPU sample's structures (oracle counts of every annulus test)"}

    ingest = None
    if rank == 0 and args.ingest_files > 0:
        ingest = ingestion(wl, tpl, P, args.ingest_files, os.cpu_count() or 1)

    if rank != 0:
        return
    line = {
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": total_ms / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32+f64",
        "data": "synthetic",
        "config": {"workload": wl.name, "pairs_per_gpu": pairs_step, "structures": wl.structures.n_structures,
                   "templates": wl.templates.n_templates, "atoms": wl.structures.n_atoms,
                   "params": wl.params, "l2": "inputs and candidate lists larger than L2 (no flush)",
                   "adversarial": wl.notes, "adversarial_boundary": boundary,
                   "generation_s": round(gen_s, 1)},
        "hits_per_s": hits_per_s,
        "hits_per_step": s0["hits"],
        "plain_fp64": plain,
        "batched_over_plain": value / plain["value"] if plain else None,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak if peak else None, "traffic": traffic,
                     "kernel": "k_search", "peak_kind": peak_kind, "issue_slots": issue,
                     "bytes_expansion_per_step": exp_bytes / args.steps,
                     "ms_expansion_per_step": exp_ms / args.steps},
        "stage_ms": {"candidates": s0["ms_candidates"], "expansion": s0["ms_expansion"],
                     "superposition": s0["ms_superposition"], "total": s0["ms_total"]},
        "counters": {k: s0[k] for k in ("pairs", "candidate_entries", "partials", "complete", "passing", "hits",
                                        "fp64_rechecks", "leaf_lists", "leaf_entries", "leaf_shared", "leaf_sorted",
                                        "leaf_exact", "suspensions", "search_rounds", "chunks", "row_splits")},
        "cpu_baseline": cpu,
        "ingestion": ingest,
        "e2e": e2e,
        "gpu_launches": launches,
        "tuning": tuning,
        "clocks": clocks.summary(),
    }
    print(json.dumps(line))


if __name__ == "__main__":
    main()
