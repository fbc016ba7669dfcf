"""CPU: the multi-GPU bookkeeping of bench.py on two gloo ranks.

The path has no data exchange (replicas only): each rank renders its own
copy of the workload and the job's time is the slowest rank's.  These tests
run that reduction on two CPU processes (gloo, 127.0.0.1) and check that the
reference arm does no work on ranks other than 0.
"""

from __future__ import annotations

import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, results):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    os.environ["RANK"] = str(rank)
    os.environ["WORLD_SIZE"] = str(world)
    sys.path.insert(0, ROOT)
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        results[rank] = bench.max_over_ranks(10.0 + 5.0 * rank)
        if rank != 0:
            class Args:
                steps = 1
                warmup = 0
            results[world + rank] = bench.run_reference_arm(Args())
    finally:
        dist.destroy_process_group()


def test_slowest_rank_sets_the_time_and_reference_arm_runs_on_rank0_only():
    world = 2
    manager = mp.get_context("spawn").Manager()
    results = manager.dict()
    mp.start_processes(_worker, args=(world, _free_port(), results), nprocs=world, start_method="spawn")
    assert results[0] == 15.0 and results[1] == 15.0
    assert results[world + 1] == 0


def test_single_process_value_is_unchanged():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks(3.5) == 3.5


def test_gpus_flag_starts_one_replica_per_gpu():
    """bench.py --gpus N without a launcher starts N processes itself
    (RANK / LOCAL_RANK / WORLD_SIZE, a 127.0.0.1 rendezvous); here the
    replicas only rendezvous over gloo and reduce, with no GPU work."""
    import json
    import subprocess

    result = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--gpus", "2", "--dry-run"],
                            capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert result.returncode == 0, result.stderr[-2000:]
    lines = [json.loads(line) for line in result.stdout.splitlines() if line.startswith("{")]
    assert sorted(line["rank"] for line in lines) == [0, 1]
    assert all(line["world"] == 2 and line["local_rank"] == line["rank"] for line in lines)
    assert all(line["max_over_ranks"] == 2.0 and line["master"] == "127.0.0.1" for line in lines)
