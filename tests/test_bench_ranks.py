"""The multi-rank host logic of bench.py on CPU: world_size-2 gloo ranks on
127.0.0.1. Each rank times its own replica; the job's time is the slowest
rank's (MAX all-reduce), the whole-job rate counts every rank's substeps, and
the reference arm runs on rank 0 alone."""
import os
import socket
import sys
import types

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


def _free_port():
    with socket.socket() as so:
        so.bind(("127.0.0.1", 0))
        return so.getsockname()[1]


def _rank(rank, world, port, times, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = bench.max_over_ranks(times[rank], dist, "cpu")
    out[rank] = (ms, bench.job_rate(world, ms / 10))
    dist.barrier()
    dist.destroy_process_group()


def test_job_time_is_the_slowest_rank_and_rate_counts_every_rank():
    world, times = 2, [12.5, 31.0]
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, _free_port(), times, out), nprocs=world, join=True)
        res = dict(out)
    for r in range(world):
        ms, rate = res[r]
        assert ms == max(times)
        # 10 steps in 31 ms on the slower rank, 2 replicas: 645 substeps/s
        assert rate == pytest.approx(world * 1e3 / (max(times) / 10))


def test_single_rank_needs_no_process_group():
    assert bench.max_over_ranks(7.25) == 7.25
    assert bench.job_rate(1, 2.0) == 500.0


def test_reference_arm_runs_on_rank_zero_only(monkeypatch):
    """Under torchrun the other ranks exit 0 without touching the workload."""
    monkeypatch.setenv("RANK", "1")
    args = types.SimpleNamespace(workload="block", solver=None, steps=1, warmup=3)
    assert bench.run_reference(args) == 0
