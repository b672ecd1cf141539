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


def test_batched_roofline_takes_the_sweep_share_of_the_step():
    """batch_roofline: the dominant kernel's time is the event-timed step minus
    the other kernels' event-timed share, over its launches per step; its
    algorithmic bytes are (80 B/tet + 28 B/vertex) per sweep over the whole
    batch."""
    n = 4
    prof = {"project_gs": (2.5, n), "predict": (0.02, n), "finalize": (0.03, n)}
    s = types.SimpleNamespace(profile_steps=lambda k: prof, params=types.SimpleNamespace(gs_variant=4))
    b = types.SimpleNamespace(T=1000, V=300, iters=20)
    r = bench.batch_roofline(s, b, 2.05, n)
    assert r["kernel"] == "project_gs" and r["launches_per_step"] == 1
    assert abs(r["avg_launch_ms"] - 2.0) < 1e-12
    per_launch = (80.0 * 1000 + 28.0 * 300) * 20
    assert abs(r["algorithmic_bytes_per_launch"] - per_launch) < 1e-6
    assert abs(r["achieved"] - per_launch / 2.0e-3 / 1e9) < 1e-9
    assert abs(r["frac"] - r["achieved"] / r["peak"]) < 1e-12
    # a step whose dominant kernel is not the sweep has no sweep roofline
    s2 = types.SimpleNamespace(profile_steps=lambda k: {"detect": (9.0, n), "project_gs": (0.1, n)},
                               params=s.params)
    assert bench.batch_roofline(s2, b, 2.0, n) is None
