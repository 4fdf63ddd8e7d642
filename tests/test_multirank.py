"""The multi-GPU bench path's host logic with two gloo ranks on the CPU:
each rank draws its own instance of the workload (independent pairs, weak
scaling) and the step time is the maximum over ranks."""

import os
import socket

import pytest


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import argparse

    import numpy as np
    import torch.distributed as dist

    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        args = argparse.Namespace(config=3, structures=3, templates=4)
        wl = bench.workload(args, rank, world)
        out[rank] = {
            "max": bench.max_over_ranks(10.0 + rank, dist),
            "atoms": int(wl.structures.n_atoms),
            "first_xyz": np.asarray(wl.structures.xyz[:4]).tolist(),
            "n_structures": int(wl.structures.n_structures),
            "n_templates": int(wl.templates.n_templates),
        }
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(2, port, out), nprocs=2, join=True)
        r0, r1 = out[0], out[1]
    assert r0["max"] == r1["max"] == 11.0
    assert r0["n_structures"] == r1["n_structures"] == 3
    assert r0["n_templates"] == r1["n_templates"] == 4
    assert r0["first_xyz"] != r1["first_xyz"]


def test_single_rank_is_config3():
    import argparse

    import bench
    from pyjess_gb300 import workloads as W

    args = argparse.Namespace(config=3, structures=3, templates=4)
    a = bench.workload(args, 0, 1)
    b = W.config(3, n_structures=3, n_templates=4)
    assert (a.structures.xyz == b.structures.xyz).all()
    assert bench.max_over_ranks(5.0, None) == 5.0


def test_search_profile_fields_the_bench_line_reads():
    """The committed k_search capture holds what the bench line's roofline
    reports: DRAM bytes per expansion byte and the issue-slot fraction."""
    import json
    import pathlib

    tr = json.loads((pathlib.Path(__file__).resolve().parents[1] / "profiles" / "k_search_traffic.json").read_text())
    assert 1.0 < tr["dram_per_expansion_byte"] < 10.0
    assert 0.0 < tr["issue_active_frac"] <= tr["issue_active_frac_first_round"] <= 1.0
    assert tr["warp_inst_per_partial"] == round(tr["inst_executed"] / tr["partials"], 1)
    timed = [l for l in tr["launches"] if l["query"] == "timed"]
    assert sum(l["dram_bytes_read"] + l["dram_bytes_write"] for l in timed) == tr["dram_bytes"]
