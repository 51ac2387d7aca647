"""bench.py's multi-GPU path (replicas only) on CPU ranks over gloo, world size 2.

Each rank times its own replica; the job's time is the slowest rank's (an all-reduce MAX)
and the value counts every rank's particles.  The reference arm runs on rank 0 only.
"""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

from conftest import REPO

sys.path.insert(0, str(REPO))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, times, out):
    import torch.distributed as dist

    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    t = bench.max_over_ranks(dist, times[rank], device="cpu")
    v = bench.replica_value(world, 1_000_000, 10, t)
    dist.barrier()
    dist.destroy_process_group()
    out.put((rank, t, v))


def test_replica_time_is_the_slowest_rank_and_value_counts_all_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    times = [0.050, 0.062]
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, times, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t, v in res:
        assert t == pytest.approx(0.062)
        assert v == pytest.approx(2 * 1_000_000 * 10 / 0.062)


def test_single_process_needs_no_collective():
    import bench

    assert bench.max_over_ranks(None, 0.25) == 0.25
    assert bench.replica_value(1, 1000, 4, 0.5) == 8000.0


def test_reference_arm_runs_on_rank_zero_only():
    import argparse

    import bench

    args = argparse.Namespace(workload="dam_break_10k", steps=1, warmup=0, gpus=2)
    assert bench.bench_reference(args, world=2, rank=1) == 0  # returns at once, no work


def test_reference_arm_line_carries_the_contract_keys(built, capsys):
    """The reference arm's JSON line on a small workload (rank 0, CPU): its own metric and
    unit, a cpu_baseline describing the run, and an e2e with no host<->device bytes."""
    import argparse
    import json

    import bench

    args = argparse.Namespace(workload="dam_break_10k", steps=1, warmup=0, gpus=1)
    assert bench.bench_reference(args, world=1, rank=0) == 0
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    assert line["metric"] == bench.METRIC and line["unit"] == bench.UNIT
    assert line["value"] > 0 and line["higher_is_better"] is True
    assert line["config"]["workload"] == "dam_break_10k"
    cb = line["cpu_baseline"]
    assert cb["value"] == line["value"] and cb["kind"] == "port" and cb["cores"] >= 1
    assert cb["sample"]
    assert line["e2e"] == {"value": line["value"], "unit": bench.UNIT,
                           "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
