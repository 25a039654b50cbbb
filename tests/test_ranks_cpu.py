"""The benchmark's multi-rank path on CPU ranks (gloo, world size 2).

The traversal shards by rays: every rank traces its own seeded rays with no
data-path collective ("replicas"). The only exchange is the timing: each
timing's maximum over the ranks sets the job's time, and the whole-job rate
counts every rank's rays. The reference arm runs on rank 0 alone.
"""
from __future__ import annotations

import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, out) -> None:
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r took 10 (r + 1) ms for the traversal and 1 + r s end to end
        got = bench.max_over_ranks([10.0 * (rank + 1), 1.0 + rank], dist, "cpu")
        out[rank] = got
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_timings_take_the_slowest_rank():
    ctx = mp.get_context("spawn")
    with ctx.Manager() as mgr:
        out = mgr.dict()
        mp.start_processes(_worker, args=(2, _free_port(), out), nprocs=2, start_method="spawn")
        assert out[0] == [20.0, 2.0] and out[1] == [20.0, 2.0]


def test_job_rate_counts_every_rank():
    import bench
    # 2 ranks x 16.8 M rays x 5 steps in 20 ms
    assert bench.job_rate(2, 1 << 24, 5, 0.020) == pytest.approx(2 * (1 << 24) * 5 / 0.020 / 1e6)
    assert bench.job_rate(1, 1 << 24, 1, 1.0) == pytest.approx((1 << 24) / 1e6)


def test_ranks_trace_different_rays():
    from devilray_gb300 import scenes
    a = scenes.incoherent_rays(1024, seed=0)
    b = scenes.incoherent_rays(1024, seed=1)
    assert a.shape == b.shape and not (a == b).all()


def test_reference_arm_runs_on_rank_zero_only(monkeypatch):
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("LOCAL_RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    # a non-zero rank exits 0 at once, before building any workload
    monkeypatch.setattr(bench, "build_workload", lambda rank: pytest.fail("rank 1 built a workload"))
    assert bench.run_reference(None) == 0
