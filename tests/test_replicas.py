"""Host-side logic of the benchmark.  Several GPUs run independent
replicas (pairs are independent units; no data is exchanged): the only
cross-rank step is the timing reduction -- each timing's maximum over the
ranks, and the job's rate = all ranks' pairs over the slowest rank's time
-- checked here with two gloo ranks on the CPU.  The JSON line is assembled
from measurement records by a pure function, checked on made-up records."""
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


def _record(total_ms, prof=None, trials=None):
    """A record shaped like bench.measure()'s."""
    return dict(total_ms=total_ms, step_ms=[total_ms / 10] * 10, pair_ms=[1.3, 1.31, 1.32], launches=370,
                prof=prof or {}, prof_steps=1,
                clocks={"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": [], "samples": 20},
                e2e_total=8 * 13.7, e2e_steps=8, e2e_trials=trials)


def test_result_line_keeps_the_contract_keys():
    import argparse
    import bench
    args = argparse.Namespace(batch=32, steps=10, warmup=3, mode="batched", impl="mine")
    prof = {"path_row": {"ms": 2.8, "launches": 4, "bytes": 11.9e9},
            "cost": {"ms": 4.36, "launches": 3, "bytes": 1.6e9},
            "p2table": {"ms": 0.0, "launches": 0, "bytes": 0.0}}
    head = _record(132.7, prof, [13.7, 13.7, 19.6, 13.7, 13.7])
    out = bench.result_line(args, 1, head, _record(384.0), {"hbm_gbs": 6795.1, "source": "measured"}, 320)
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "e2e", "gpu_launches", "clocks", "roofline", "throughput"):
        assert k in out, k
    assert out["value"] == round(320 / 0.1327, 3)
    assert out["e2e"]["value"] == round(32 * 8 / (8 * 13.7 / 1e3), 3)
    assert set(out["e2e"]) >= {"value", "unit", "h2d_bytes_per_step", "d2h_bytes_per_step"}
    assert out["roofline"]["bound"] == "hbm" and 0 < out["roofline"]["frac"] < 1
    assert set(out["roofline"]) >= {"achieved", "peak", "unit", "frac", "traffic"}
    assert out["throughput"]["mpix_per_s"] == round(out["value"] * 1920 * 1080 / 1e6, 1)
    assert set(out["kernels_hbm"]) == {"path_row", "cost"}
    assert out["kernels_ms_per_step"]["path_row"] == 2.8
    # traffic: each aggregation kind's own bytes times its DRAM bytes per own byte
    assert out["roofline"]["traffic"] == round(bench.AGG_TRAFFIC_PER_OWN_BYTE["path_row"] * 11.9, 4)
    prof2 = dict(prof, tbw={"ms": 1.8, "launches": 1, "bytes": 7.0e9}, wta={"ms": 0.4, "launches": 3, "bytes": 2.0e9})
    out2 = bench.result_line(args, 1, _record(132.7, prof2), _record(384.0), {"hbm_gbs": 6795.1, "source": "measured"},
                             320)
    want = sum(bench.AGG_TRAFFIC_PER_OWN_BYTE[k] * prof2[k]["bytes"] for k in ("path_row", "wta", "tbw")) / 1e9
    assert out2["roofline"]["traffic"] == round(want, 4)
    assert "k_gtbw" in out2["roofline"]["kernel"] and out2["roofline"]["ms_per_step"] == round(2.8 + 0.4 + 1.8, 4)
    ref = bench.result_line(argparse.Namespace(batch=32, steps=10, warmup=3, mode="batched", impl="reference"), 1,
                            _record(4146.6), _record(4146.6), {"hbm_gbs": 6795.1, "source": "measured"}, 320)
    assert ref["impl"] == "reference" and "roofline" not in ref


def test_roofline_bytes_of_the_benchmark_pair():
    """The algorithmic bytes the roofline divides by, for one 1920x1080
    D=256 pyramid_levels=3 pair: levels 1920x1080, 960x540 and 480x270 with
    16 labels and the coarse 240x135 with 32; 4 B per voxel for the
    aggregation; both u8 views, the outputs and the pyramid on top."""
    import bench
    got = bench.alg_bytes(1920, 1080, bench.params_for(bench.CENSUS))
    px = [1920 * 1080, 960 * 540, 480 * 270, 240 * 135]
    vox = 16 * (px[0] + px[1] + px[2]) + 32 * px[3]
    assert got["voxels"] == vox == 44_582_400
    assert got["aggregation"] == 4 * vox
    total = 4 * vox + 2 * sum(px) + 10 * px[0] + 12 * sum(px[1:]) + sum(2 * px[i - 1] + 2 * px[i] for i in (1, 2, 3))
    assert got["total"] == total == 219_542_400
    assert bench.alg_bytes(1920, 1080, bench.params_for(bench.BT)) == got
