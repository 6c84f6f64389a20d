#!/usr/bin/env python3
"""Benchmark: 1080p D=256 stereo pairs per second on one GB300.

A step is one pass of the SGM hot path over a batch of `--batch` seeded
synthetic 1920x1080 pairs, D=256, pyramid_levels=3, adaptive P2 and 3x3
median on, disparity x16 + float disparity + confidence outputs, Census and
Birchfield-Tomasi pairs alternating (the 1080p D=256 configuration the
reference's headline metric is quoted on).

  value   pairs/s with the inputs resident in device memory (CUDA events on
          the compute stream, L2 flushed between steps outside the events)
  e2e     the same through the public API with pinned host buffers: per step
          the host->device copy of every pair's images, compute(), and the
          device->host copy of its three outputs, all inside the events
  roofline  the dominant kernel (the row pass: L->R + R->L + WTA + LR check)
          timed with CUDA events on its own stream via the library profiler,
          its algorithmic bytes / duration against the measured HBM peak

--impl reference runs the reference's own CUDA kernels (compiled from its
sources into oracle/_ref/ and launched by oracle/_build/libref_harness.so)
through the reference's StereoMatcher schedule, on the same workload.
Several GPUs (torchrun): independent replicas, one per GPU (pairs are
independent units; nothing is exchanged).
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

W, H, D, LEVELS = 1920, 1080, 256, 3
CENSUS, BT = 1, 0
METRIC = "1080p D=256 pairs/s"


def params_for(cost: int) -> dict:
    return dict(num_disparities=D, pyramid_levels=LEVELS, cost_mode=cost,
                p1=8 if cost == CENSUS else 300, p2=32 if cost == CENSUS else 2400,
                adaptive_p2=True, median_filter=True, lr_check=True, uniqueness_ratio=10,
                pyramid_coarse_disparities=128)


def peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return {"hbm_gbs": d.get("hbm_gbs", 6800.0), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []
        self.t = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            if self.t:
                self.t.join(timeout=2)

    def summary(self) -> dict:
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx = max(mx, float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def make_inputs(batch: int, seed0: int = 3000):
    from pyrsgm_gb300 import synth
    pairs = []
    for i in range(batch):
        left, right, _ = synth.make_pair(W, H, D - 1, 16, seed0 + i)
        pairs.append((left, right, CENSUS if i % 2 == 0 else BT))
    return pairs


# ---------------------------------------------------------------------------
# this library
# ---------------------------------------------------------------------------
class MineRunner:
    def __init__(self, pairs, dev):
        import torch
        import pyrsgm_gb300 as pg
        self.torch, self.pg = torch, pg
        self.matchers = {c: pg.StereoMatcher(W, H, pg.Params(**params_for(c))) for c in (CENSUS, BT)}
        self.costs = [c for _, _, c in pairs]
        self.L = [torch.from_numpy(l).to(dev) for l, _, _ in pairs]
        self.R = [torch.from_numpy(r).to(dev) for _, r, _ in pairs]
        self.d16 = [torch.empty((H, W), dtype=torch.int16, device=dev) for _ in pairs]
        self.d32 = [torch.empty((H, W), dtype=torch.float32, device=dev) for _ in pairs]
        self.cf = [torch.empty((H, W), dtype=torch.float32, device=dev) for _ in pairs]
        self.hL = [torch.from_numpy(l).pin_memory() for l, _, _ in pairs]
        self.hR = [torch.from_numpy(r).pin_memory() for _, r, _ in pairs]
        self.h16 = [torch.empty((H, W), dtype=torch.int16).pin_memory() for _ in pairs]
        self.h32 = [torch.empty((H, W), dtype=torch.float32).pin_memory() for _ in pairs]
        self.hcf = [torch.empty((H, W), dtype=torch.float32).pin_memory() for _ in pairs]

    def step(self, stream, pair_events=None):
        for i, c in enumerate(self.costs):
            self.matchers[c].compute_into(self.L[i], self.R[i], self.d16[i], self.d32[i], self.cf[i], stream)
            if pair_events is not None:
                pair_events[i].record(stream)

    def step_e2e(self, stream):
        for i, c in enumerate(self.costs):
            self.L[i].copy_(self.hL[i], non_blocking=True)
            self.R[i].copy_(self.hR[i], non_blocking=True)
            self.matchers[c].compute_into(self.L[i], self.R[i], self.d16[i], self.d32[i], self.cf[i], stream)
            self.h16[i].copy_(self.d16[i], non_blocking=True)
            self.h32[i].copy_(self.d32[i], non_blocking=True)
            self.hcf[i].copy_(self.cf[i], non_blocking=True)

    def launches(self) -> int:
        from pyrsgm_gb300._native import lib
        return int(lib().pyrsgm_gb300_launch_count())


# ---------------------------------------------------------------------------
# the reference's kernels (oracle/_ref) on the reference schedule
# ---------------------------------------------------------------------------
class ReferenceRunner:
    """StereoMatcher::compute of the reference (src/stereo_matcher.cpp:238-338)
    driving the reference kernels through the harness, all buffers
    preallocated as in its constructor (src/stereo_matcher.cpp:164-217)."""

    def __init__(self, pairs, dev):
        import torch
        from tests import _oracle
        self.torch = torch
        self.ref = _oracle.ref()
        self.costs = [c for _, _, c in pairs]
        self.geo = {c: _oracle.orc_geometry(W, H, **params_for(c)) for c in (CENSUS, BT)}
        self.val = {c: _oracle.orc_validate(**params_for(c)) for c in (CENSUS, BT)}
        self.ws = {c: [] for c in (CENSUS, BT)}
        self.pyr = {}
        for c in (CENSUS, BT):
            for li in self.geo[c]:
                ws = self.ref.ref_create_workspace()
                assert self.ref.ref_workspace_reserve(ws, li["width"], li["height"], li["num_labels"]) == 0
                self.ws[c].append(ws)
        g = self.geo[CENSUS]
        for lv in range(1, LEVELS + 1):
            li = g[lv]
            mk = lambda dt: torch.empty((li["height"], li["width"]), dtype=dt, device=dev)
            self.pyr[lv] = dict(L=mk(torch.uint8), R=mk(torch.uint8), d16=mk(torch.int16), cf=mk(torch.float32))
        self.L = [torch.from_numpy(l).to(dev) for l, _, _ in pairs]
        self.R = [torch.from_numpy(r).to(dev) for _, r, _ in pairs]
        self.d16 = [torch.empty((H, W), dtype=torch.int16, device=dev) for _ in pairs]
        self.d32 = [torch.empty((H, W), dtype=torch.float32, device=dev) for _ in pairs]
        self.cf = [torch.empty((H, W), dtype=torch.float32, device=dev) for _ in pairs]
        self.hL = [torch.from_numpy(l).pin_memory() for l, _, _ in pairs]
        self.hR = [torch.from_numpy(r).pin_memory() for _, r, _ in pairs]
        self.h16 = [torch.empty((H, W), dtype=torch.int16).pin_memory() for _ in pairs]
        self.h32 = [torch.empty((H, W), dtype=torch.float32).pin_memory() for _ in pairs]
        self.hcf = [torch.empty((H, W), dtype=torch.float32).pin_memory() for _ in pairs]

    def _one(self, i, st):
        c = self.costs[i]
        v, geo, ref = self.val[c], self.geo[c], self.ref
        a = (v["p2_alpha"], v["p2_beta"], v["p2_lower_mult"], v["p2_upper_mult"])
        prevL, prevR, pw = self.L[i], self.R[i], W
        for lv in range(1, LEVELS + 1):
            li, par = geo[lv], geo[lv - 1]
            P = self.pyr[lv]
            for s, d in ((prevL, P["L"]), (prevR, P["R"])):
                assert ref.ref_pyrdown_u8(s.data_ptr(), s.stride(0), par["width"], par["height"], d.data_ptr(),
                                          d.stride(0), li["width"], li["height"], st) == 0
            prevL, prevR = P["L"], P["R"]
        for lv in range(LEVELS, -1, -1):
            li = geo[lv]
            w, h = li["width"], li["height"]
            refine = li["refine"]
            Lt = self.L[i] if lv == 0 else self.pyr[lv]["L"]
            Rt = self.R[i] if lv == 0 else self.pyr[lv]["R"]
            o16 = self.d16[i] if lv == 0 else self.pyr[lv]["d16"]
            oc = self.cf[i] if lv == 0 else self.pyr[lv]["cf"]
            o32 = self.d32[i].data_ptr() if lv == 0 else None
            post = ((1 if v["lr_check"] else 0) | (2 if v["median_filter"] else 0)) if lv == 0 else 1
            par = self.pyr.get(lv + 1)
            pwid = geo[lv + 1]["width"] if refine else 0
            phei = geo[lv + 1]["height"] if refine else 0
            r = ref.ref_compute_level(self.ws[c][lv], Lt.data_ptr(), Rt.data_ptr(),
                                      par["d16"].data_ptr() if refine else None,
                                      par["cf"].data_ptr() if refine else None, o16.data_ptr(), o32, oc.data_ptr(),
                                      Lt.stride(0), Rt.stride(0), pwid * 2, pwid * 4, w * 2, w * 4, w * 4, w, h,
                                      pwid, phei, li["num_labels"], 0, li["max_disparity"], li["block_size"],
                                      v["p1"], v["p2"], v["uniqueness_ratio"], v["disp12_max_diff"],
                                      v["pre_filter_cap"], v["cost_mode"], post, v["num_paths"], 1 if refine else 0,
                                      v["pyramid_min_confidence"], v["adaptive_p2"], *a, st)
            assert r == 0, ref.ref_last_error()

    def step(self, stream, pair_events=None):
        st = stream.cuda_stream
        for i in range(len(self.costs)):
            self._one(i, st)
            if pair_events is not None:
                pair_events[i].record(stream)

    def step_e2e(self, stream):
        st = stream.cuda_stream
        for i in range(len(self.costs)):
            self.L[i].copy_(self.hL[i], non_blocking=True)
            self.R[i].copy_(self.hR[i], non_blocking=True)
            self._one(i, st)
            self.h16[i].copy_(self.d16[i], non_blocking=True)
            self.h32[i].copy_(self.d32[i], non_blocking=True)
            self.hcf[i].copy_(self.cf[i], non_blocking=True)

    def launches(self) -> int:
        return 0


# ---------------------------------------------------------------------------
def cpu_baseline(pairs, budget_s: float = 25.0) -> dict:
    """The oracle (CPU restatement of the reference path, OpenMP over rows /
    columns) on host cores, on a bounded sample of the same workload."""
    import numpy as np
    from tests import _oracle
    orc = _oracle.oracle()
    cores = os.cpu_count() or 1
    orc.orc_set_num_threads(cores)
    done, t0 = 0, time.perf_counter()
    for left, right, c in pairs:
        p = params_for(c)
        lut = _oracle.p2_table_libm(p["p2"], 3.041, 16.137, 0.601, 1.77)
        _oracle.orc_matcher(np.ascontiguousarray(left), np.ascontiguousarray(right), lut, **p)
        done += 1
        if time.perf_counter() - t0 > budget_s or done >= 2:
            break
    dt = time.perf_counter() - t0
    return {"value": round(done / dt, 4), "unit": "pairs/s", "cores": orc.orc_num_threads(), "kind": "port",
            "sample": f"{done} full 1920x1080 D=256 L3 pair(s) (Census first, then BT), adaptive P2 table from libm"}


def run(args) -> dict | None:
    import torch
    import torch.distributed as dist

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl" if args.impl == "mine" else "gloo")
    if args.impl == "reference" and rank != 0:
        return None
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    pairs = make_inputs(args.batch)
    Runner = MineRunner if args.impl == "mine" else ReferenceRunner
    if args.impl == "reference":
        from tests import _oracle
        if not _oracle.ref_available():
            print(json.dumps({"impl": "reference", "unavailable": "reference kernels (oracle/_ref) not built"}))
            return None
    runner = Runner(pairs, dev)
    stream = torch.cuda.Stream(device=dev)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)  # > 129 MB L2

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            runner.step(stream)
    torch.cuda.synchronize()

    # ---- device-resident throughput --------------------------------------
    lib = None
    if args.impl == "mine":
        from pyrsgm_gb300._native import lib as _lib
        lib = _lib()
        lib.pyrsgm_gb300_profile(1)
    n0 = runner.launches()
    step_ms, pair_ms = [], []
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            with torch.cuda.stream(stream):
                flush.fill_(1)
                ev = [torch.cuda.Event(enable_timing=True) for _ in range(args.batch + 1)]
                ev[0].record(stream)
                runner.step(stream, ev[1:])
            torch.cuda.synchronize()
            step_ms.append(ev[0].elapsed_time(ev[-1]))
            pair_ms += [ev[i].elapsed_time(ev[i + 1]) for i in range(args.batch)]
    torch.cuda.synchronize()
    launches = runner.launches() - n0
    prof = {}
    if lib is not None:
        names = ["pyrdown", "features", "labels", "cost", "path_tb", "path_row", "post", "p2table"]
        for k, nm in enumerate(names):
            ms, cnt, by = C.c_double(), C.c_longlong(), C.c_double()
            lib.pyrsgm_gb300_profile_read(k, C.byref(ms), C.byref(cnt), C.byref(by))
            prof[nm] = {"ms": ms.value, "launches": cnt.value, "bytes": by.value}
        lib.pyrsgm_gb300_profile(0)
    total_ms = sum(step_ms)
    if world > 1:
        t = torch.tensor([total_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    value = world * args.batch * args.steps / (total_ms / 1e3)

    # ---- end to end through the public API -------------------------------
    e2e_ms = []
    for _ in range(max(1, args.steps // 2)):
        with torch.cuda.stream(stream):
            flush.fill_(2)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            runner.step_e2e(stream)
            b.record(stream)
        torch.cuda.synchronize()
        e2e_ms.append(a.elapsed_time(b))
    e2e_total = sum(e2e_ms)
    if world > 1:
        t = torch.tensor([e2e_total], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_total = float(t.item())
    e2e_value = world * args.batch * len(e2e_ms) / (e2e_total / 1e3)

    if rank != 0:
        return None
    pk = peaks()
    out = {
        "metric": METRIC, "value": round(value, 3), "unit": "pairs/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int16", "data": "synthetic (seeded value-noise pairs, "
        "slanted-plane Voronoi ground truth; stands in for Middlebury)",
        "config": {"workload": "1920x1080 D=256 pyramid_levels=3, Census/BT alternating, adaptive P2, median, "
                   "disp16+disp32+conf", "pairs_per_step": args.batch, "width": W, "height": H,
                   "num_disparities": D, "pyramid_levels": LEVELS, "l2": "flushed (256 MB write) between steps",
                   "parallelism": f"replicas x{world}"},
        "latency_ms": {"p50": round(statistics.median(pair_ms), 4),
                       "p99": round(sorted(pair_ms)[max(0, int(len(pair_ms) * 0.99) - 1)], 4),
                       "unit": "per pair, back-to-back compute() on one stream"},
        "e2e": {"value": round(e2e_value, 3), "unit": "pairs/s",
                "h2d_bytes_per_step": args.batch * 2 * W * H,
                "d2h_bytes_per_step": args.batch * W * H * (2 + 4 + 4)},
        "gpu_launches": launches,
        "clocks": clk.summary(),
    }
    if args.impl == "mine":
        row = prof.get("path_row", {})
        achieved = (row["bytes"] / (row["ms"] / 1e3) / 1e9) if row.get("ms") else None
        out["roofline"] = {"kernel": "k_path_row (L->R + R->L + WTA + disp2 + LR check)", "bound": "hbm",
                           "achieved": round(achieved, 2) if achieved else None, "peak": pk["hbm_gbs"],
                           "unit": "GB/s", "frac": round(achieved / pk["hbm_gbs"], 4) if achieved else None,
                           "peak_source": pk["source"], "traffic": None,
                           "avg_launch_ms": round(row["ms"] / row["launches"], 5) if row.get("launches") else None}
        out["kernels_ms_per_step"] = {k: round(v["ms"] / args.steps, 4) for k, v in prof.items() if v["launches"]}
        if not args.no_cpu and world == 1:
            out["cpu_baseline"] = cpu_baseline(pairs)
    else:
        out["impl"] = "reference"
        out["reference_build"] = "reference src/sgm_kernels.cu + src/pyrdown.cu compiled unmodified for sm_103a"
        if not args.no_cpu and world == 1:
            out["cpu_baseline"] = cpu_baseline(pairs)
    return out


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--batch", type=int, default=8, help="pairs per step")
    ap.add_argument("--impl", choices=["mine", "reference"], default="mine")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    out = run(args)
    if out is not None:
        print(json.dumps(out))


if __name__ == "__main__":
    main()
