"""Several GPUs run independent replicas (pairs are independent units; no
data is exchanged).  The only cross-rank step is the benchmark's timing
reduction: each timing's maximum over the ranks, and the job's rate = all
ranks' pairs over the slowest rank's time.  Checked here with two gloo
ranks on the CPU."""
from __future__ import annotations

import os
import socket

import pytest


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, port: int, q) -> None:
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=2)
    try:
        # rank 0 is slower on the batched steps, rank 1 on the end-to-end runs
        got = bench.replica_max(dist, [120.0 - 20.0 * rank, 300.0 + 50.0 * rank], "cpu")
        q.put((rank, got))
    finally:
        dist.destroy_process_group()


def test_timing_reduction_over_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = dict(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out[0] == out[1] == [120.0, 350.0]


def test_job_rate_counts_every_rank_over_the_slowest_time():
    import bench
    # two replicas, 320 pairs each, the slower one taking 160 ms
    assert bench.job_rate(2, 320, 160.0) == pytest.approx(4000.0)
    assert bench.job_rate(1, 320, 160.0) == pytest.approx(2000.0)


def test_stage_bandwidth_from_profiler_records():
    import bench
    prof = {"path_row": {"ms": 2.0, "launches": 4, "bytes": 8e9},
            "cost": {"ms": 4.0, "launches": 3, "bytes": 1e9},
            "p2table": {"ms": 0.0, "launches": 0, "bytes": 0.0}}
    got = bench.stage_bandwidth(prof, 8000.0)
    assert got == {"path_row": {"gbs": 4000.0, "frac": 0.5}, "cost": {"gbs": 250.0, "frac": 0.0312}}
