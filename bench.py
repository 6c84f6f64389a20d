#!/usr/bin/env python3
"""Benchmark: 1080p D=256 stereo pairs per second on one GB300.

A step is one pass of the SGM hot path over a batch of `--batch` seeded
synthetic 1920x1080 pairs, D=256, pyramid_levels=3, adaptive P2 and 3x3
median on, disparity x16 + float disparity + confidence outputs, Census and
Birchfield-Tomasi pairs alternating (the 1080p D=256 configuration the
reference's headline metric is quoted on).

  value   pairs/s with the inputs resident in device memory (CUDA events on
          the compute stream, L2 flushed between steps outside the events)
  e2e     the same through the public API with pinned host buffers: every
          step copies its pairs' images host->device, runs the engine and
          copies the three outputs device->host (each kind of image and
          output of a step in one page-locked arena, copied whole); two
          slots let one step's copies overlap its neighbours' compute, and
          the events span all steps, copies included
  roofline  the aggregation kernels of one step, each timed with CUDA events
          on its stream via the library profiler: the algorithmic bytes of
          the aggregation (4 B per voxel: the partial aggregated volume
          written and read once) over their summed duration, against the
          measured HBM peak; pipeline_roofline the same for the whole step

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


# Measured DRAM bytes (ncu dram__bytes_read.sum + dram__bytes_write.sum) per
# byte the aggregation kernels move by their own design, from the full
# captures of the 1080p-level launches of eight pairs
# (profiles/stage_kernels_1080p_8pairs.md): k_gtb 1066.8, k_grow 2147.6,
# k_wta 1834.9 and k_gtbw 1854.7 MB against 1111.5, 2222.9, 1791.6 and
# 1808.2 MB of their own bytes.  Every kernel streams its volumes once per
# launch, so the ratio carries over to a step by each kind's own bytes.
AGG_TRAFFIC_PER_OWN_BYTE = {"path_tb": 1066.8 / 1111.5, "path_row": 2147.6 / 2222.9, "wta": 1834.9 / 1791.6,
                            "tbw": 1854.7 / 1808.2}


def alg_bytes(width: int, height: int, params: dict) -> dict:
    """Algorithmic device-memory bytes of one pair: every level's partial
    aggregated volume written and read once as int16 (4 B per voxel; costs
    recomputed on chip), both u8 views read, the outputs (disp16 + disp32 +
    conf at level 0; disparity and confidence written and read by the child
    on the other levels) and the pyramid (parent views read, child views
    written).  'aggregation' is the volume term alone."""
    import pyrsgm_gb300 as pg
    info = pg.level_geometry(width, height, pg.Params(**params))
    agg = sum(4.0 * li.width * li.height * li.num_labels for li in info)
    px = [li.width * li.height for li in info]
    views = sum(2.0 * p for p in px)
    outs = 10.0 * px[0] + sum(12.0 * p for p in px[1:])
    pyr = sum(2.0 * px[l - 1] + 2.0 * px[l] for l in range(1, len(px)))
    return {"aggregation": agg, "total": agg + views + outs + pyr,
            "voxels": sum(float(li.width * li.height * li.num_labels) for li in info)}


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
                 "-lms", "50"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            # the timed region starts once nvidia-smi is sampling
            t_end = time.time() + 5.0
            while not self.lines and time.time() < t_end and self.proc.poll() is None:
                time.sleep(0.01)
            self.skip = len(self.lines)
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
        for ln in self.lines[getattr(self, "skip", 0):]:
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
        import numpy as np
        import torch
        import pyrsgm_gb300 as pg
        self.torch, self.pg = torch, pg
        self.matchers = {c: pg.StereoMatcher(W, H, pg.Params(**params_for(c))) for c in (CENSUS, BT)}
        self.costs = [c for _, _, c in pairs]
        n = len(pairs)
        # every image and output kind of a step in one arena (pair i at [i]),
        # on the device and page-locked on the host: the end-to-end steps copy
        # whole arenas, the engine gets per-pair views
        self.A = dict(L=torch.from_numpy(np.stack([l for l, _, _ in pairs])).to(dev),
                      R=torch.from_numpy(np.stack([r for _, r, _ in pairs])).to(dev),
                      d16=torch.empty((n, H, W), dtype=torch.int16, device=dev),
                      d32=torch.empty((n, H, W), dtype=torch.float32, device=dev),
                      cf=torch.empty((n, H, W), dtype=torch.float32, device=dev),
                      hL=torch.from_numpy(np.stack([l for l, _, _ in pairs])).pin_memory(),
                      hR=torch.from_numpy(np.stack([r for _, r, _ in pairs])).pin_memory(),
                      h16=torch.empty((n, H, W), dtype=torch.int16).pin_memory(),
                      h32=torch.empty((n, H, W), dtype=torch.float32).pin_memory(),
                      hcf=torch.empty((n, H, W), dtype=torch.float32).pin_memory())
        for k in ("L", "R", "d16", "d32", "cf", "hL", "hR", "h16", "h32", "hcf"):
            setattr(self, k, list(self.A[k].unbind(0)))

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


class BatchRunner(MineRunner):
    """All pairs of a step in one BatchEngine run (one launch per stage and
    kernel variant for the whole batch, replayed as a CUDA graph)."""

    def __init__(self, pairs, dev):
        super().__init__(pairs, dev)
        pg = self.pg
        # the 16/32/64-label kernel shape of each aggregation launch is
        # measured on the first (warm-up) run and recorded
        pg.set_autotune(True)
        self.engine = pg.BatchEngine(40 << 30)
        items = [dict(left=self.L[i], right=self.R[i], params=pg.Params(**params_for(c)), disp16=self.d16[i],
                      disp32=self.d32[i], conf=self.cf[i]) for i, c in enumerate(self.costs)]
        self.arr = pg.BatchEngine.make_pairs(items)

    def step(self, stream, pair_events=None):
        self.engine.run_pairs(self.arr, True, stream)
        if pair_events is not None:
            for e in pair_events:
                e.record(stream)

    def step_direct(self, stream):
        self.engine.run_pairs(self.arr, False, stream)

    def e2e_begin(self, stream):
        """Two slots of device inputs/outputs so that one step's copies overlap
        the other's compute: H2D on one stream, the engine on the compute
        stream, D2H on a third, ordered per slot by events."""
        torch, pg = self.torch, self.pg
        if getattr(self, "slots", None) is None:
            self.slots = []
            for k in range(2):
                if k == 0:
                    sl = dict(self.A, arr=self.arr)
                else:
                    sl = {key: (t.clone() if key in ("L", "R") else torch.empty_like(t)) if t.is_cuda
                          else (t.clone().pin_memory() if key in ("hL", "hR") else torch.empty_like(t).pin_memory())
                          for key, t in self.A.items()}
                    items = [dict(left=sl["L"][i], right=sl["R"][i], params=pg.Params(**params_for(c)),
                                  disp16=sl["d16"][i], disp32=sl["d32"][i], conf=sl["cf"][i])
                             for i, c in enumerate(self.costs)]
                    sl["arr"] = pg.BatchEngine.make_pairs(items)
                sl["free"] = torch.cuda.Event()
                sl["inp"] = torch.cuda.Event()
                sl["done"] = torch.cuda.Event()
                self.slots.append(sl)
            self.s_h2d = torch.cuda.Stream()
            self.s_d2h = torch.cuda.Stream()
            self.engine.run_pairs(self.slots[1]["arr"], True, stream)   # graph for the second slot
        start = torch.cuda.Event()
        start.record(stream)
        self.s_h2d.wait_event(start)
        self.s_d2h.wait_event(start)
        for sl in self.slots:
            sl["free"].record(self.s_d2h)

    def step_e2e(self, stream, k: int = 0):
        torch = self.torch
        sl = self.slots[k % 2]
        with torch.cuda.stream(self.s_h2d):
            self.s_h2d.wait_event(sl["free"])
            sl["L"].copy_(sl["hL"], non_blocking=True)
            sl["R"].copy_(sl["hR"], non_blocking=True)
            sl["inp"].record(self.s_h2d)
        stream.wait_event(sl["inp"])
        self.engine.run_pairs(sl["arr"], True, stream)
        sl["done"].record(stream)
        with torch.cuda.stream(self.s_d2h):
            self.s_d2h.wait_event(sl["done"])
            sl["h16"].copy_(sl["d16"], non_blocking=True)
            sl["h32"].copy_(sl["d32"], non_blocking=True)
            sl["hcf"].copy_(sl["cf"], non_blocking=True)
            sl["free"].record(self.s_d2h)

    def e2e_end(self, stream):
        stream.wait_stream(self.s_h2d)
        stream.wait_stream(self.s_d2h)


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
def cpu_baseline(pairs, budget_s: float = 20.0) -> dict:
    """The oracle (CPU restatement of the reference path, OpenMP over rows /
    columns) on host cores, on a bounded sample of the same workload: the
    step's pairs in order (Census and BT alternating) until `budget_s` has
    passed, with the spread of the per-pair times."""
    import numpy as np
    from tests import _oracle
    orc = _oracle.oracle()
    cores = os.cpu_count() or 1
    orc.orc_set_num_threads(cores)
    per = []
    t0 = time.perf_counter()
    for left, right, c in pairs:
        p = params_for(c)
        lut = _oracle.p2_table_libm(p["p2"], 3.041, 16.137, 0.601, 1.77)
        t = time.perf_counter()
        _oracle.orc_matcher(np.ascontiguousarray(left), np.ascontiguousarray(right), lut, **p)
        per.append(time.perf_counter() - t)
        if time.perf_counter() - t0 > budget_s:
            break
    dt = time.perf_counter() - t0
    s = sorted(per)
    return {"value": round(len(per) / dt, 4), "unit": "pairs/s", "cores": orc.orc_num_threads(), "kind": "port",
            "sample": f"{len(per)} full 1920x1080 D=256 L3 pairs (Census and BT alternating), adaptive P2 table "
                      f"from libm; {budget_s:.0f} s budget",
            "pair_s": {"min": round(s[0], 4), "median": round(s[len(s) // 2], 4), "max": round(s[-1], 4)}}


def measure(runner, args, stream, flush, dev, world, dist, profile: bool, pair_timing: bool) -> dict:
    """Warm up, then time args.steps device-resident steps (CUDA events on the
    compute stream, L2 flushed between steps outside the events) and
    args.steps // 2 end-to-end steps (host->device inputs, compute,
    device->host outputs inside the events)."""
    import torch
    lib = None
    graph = isinstance(runner, BatchRunner)
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            runner.step(stream)
    torch.cuda.synchronize()
    if profile:
        from pyrsgm_gb300._native import lib as _lib
        lib = _lib()
        if not graph:
            lib.pyrsgm_gb300_profile(1)  # events around every launch of the timed steps
    n0 = runner.launches()
    step_ms, pair_ms = [], []
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    # clocks are sampled from here to the end of the e2e runs
    clk = ClockSampler(torch.cuda.current_device())
    clk.__enter__()
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(1)
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(args.batch + 1)]
            ev[0].record(stream)
            runner.step(stream, ev[1:] if pair_timing else None)
            if not pair_timing:
                ev[-1].record(stream)
        torch.cuda.synchronize()
        step_ms.append(ev[0].elapsed_time(ev[-1]))
        if pair_timing:
            pair_ms += [ev[i].elapsed_time(ev[i + 1]) for i in range(args.batch)]
    torch.cuda.synchronize()
    launches = runner.launches() - n0
    prof = {}
    if lib is not None and graph:
        # graph replays bypass the launchers: time the same launches of one
        # step enqueued directly (events on the compute stream around each)
        lib.pyrsgm_gb300_profile(1)
        with torch.cuda.stream(stream):
            flush.fill_(3)
            runner.step_direct(stream)
        torch.cuda.synchronize()
    if lib is not None:
        for k, nm in enumerate(PROF_NAMES):
            ms, cnt, by = C.c_double(), C.c_longlong(), C.c_double()
            lib.pyrsgm_gb300_profile_read(k, C.byref(ms), C.byref(cnt), C.byref(by))
            prof[nm] = {"ms": ms.value, "launches": cnt.value, "bytes": by.value}
        lib.pyrsgm_gb300_profile(0)
    total_ms = sum(step_ms)
    e2e_ms = []
    if hasattr(runner, "e2e_begin"):
        # pipelined: step k's H2D and D2H overlap the compute of its neighbours;
        # the timed region spans all steps, copies included (the first step's
        # inputs and the last step's outputs are not overlapped: a run of 16
        # steps or more keeps that under 3 % of a step)
        n_e2e = max(16, args.steps)
        with torch.cuda.stream(stream):
            flush.fill_(2)
            runner.e2e_begin(stream)
            runner.step_e2e(stream, 0)   # untimed: settles both slots' graphs and pinned pages
            runner.e2e_end(stream)
        torch.cuda.synchronize()
        # five timed runs of n_e2e pipelined steps; the median run counts
        # (a host-side stall of some 30 ms hits about one run in three)
        trials = []
        for _ in range(5):
            with torch.cuda.stream(stream):
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                runner.e2e_begin(stream)
                for k in range(n_e2e):
                    runner.step_e2e(stream, k)
                runner.e2e_end(stream)
                b.record(stream)
            torch.cuda.synchronize()
            trials.append(a.elapsed_time(b) / n_e2e)
        e2e_ms = [sorted(trials)[2]] * n_e2e
    else:
        for _ in range(max(1, args.steps // 2)):
            with torch.cuda.stream(stream):
                flush.fill_(2)
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                runner.step_e2e(stream)
                b.record(stream)
            torch.cuda.synchronize()
            e2e_ms.append(a.elapsed_time(b))
    clk.__exit__(None, None, None)
    e2e_total = sum(e2e_ms)
    if world > 1:
        total_ms, e2e_total = replica_max(dist, [total_ms, e2e_total], dev)
    return dict(total_ms=total_ms, step_ms=step_ms, pair_ms=pair_ms, launches=launches, prof=prof,
                prof_steps=1 if graph else args.steps,
                clocks=clk.summary(), e2e_total=e2e_total, e2e_steps=len(e2e_ms),
                e2e_trials=[round(t, 4) for t in trials] if hasattr(runner, "e2e_begin") else None)


def serve_compare(pairs_pool, params_of, rate: float, n: int, seed: int = 5000, max_batch: int = 16,
                  streams: int = 2, budget: int = 40 << 30, queue: int = 64) -> dict:
    """n requests with Poisson arrivals at `rate` pairs/s, served (a) by the
    continuous-batching server and (b) by plain sequential compute() of one
    StereoMatcher per shape (one request at a time: H2D, compute, D2H).
    Latency = arrival -> outputs in host memory."""
    import numpy as np
    import torch
    import pyrsgm_gb300 as pg
    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, n))
    picks = rng.integers(0, len(pairs_pool), n)
    nout = max_batch * streams + queue   # output buffers: every request that can be waiting or in flight

    def pinned(shape, dtype):
        # page-locked host memory (cudaHostAlloc through torch), as the plain
        # baseline below uses: copied by DMA in place by the server
        return torch.empty(shape, dtype=dtype).pin_memory().numpy()

    def outputs_for(w, h):
        return [{"disp16": pinned((h, w), torch.int16), "disp32": pinned((h, w), torch.float32),
                 "conf": pinned((h, w), torch.float32)} for _ in range(nout)]

    shapes = {}
    for l, _, c in pairs_pool:
        shapes.setdefault((l.shape[1], l.shape[0]), None)
    outs = {s: outputs_for(*s) for s in shapes}
    # (a) server
    srv = pg.Server(budget, max_batch=max_batch, streams=streams, max_queue=nout - max_batch * streams)
    # the caller's reused image and output arrays are page-locked once (as the
    # plain loop below uses pinned buffers)
    # the pool's images in page-locked memory too
    host_pool = []
    for l, r, c in pairs_pool:
        pl, pr = pinned(l.shape, torch.uint8), pinned(r.shape, torch.uint8)
        pl[...] = l
        pr[...] = r
        host_pool.append((pl, pr, c))
    pairs_pool = host_pool
    # the server keeps plans of every shape and I/O buffers of every size
    # resident (an allocation inside the timed stream would stall the
    # lanes), then the pool runs in bursts
    counts = {}
    for l, _, c in pairs_pool:
        key = (l.shape[1], l.shape[0], c)
        counts[key] = counts.get(key, 0) + 1
    for key, cnt in counts.items():
        try:
            srv.reserve(key[0], key[1], params_of(key[2]), min(max_batch, 4 * cnt))
        except RuntimeError:   # the lanes' budget is full: later shapes allocate on first use
            break
    # warm-up: the pool in bursts for at least a second (every shape's
    # kernels loaded, the GPU out of its idle clocks)
    t_w = time.perf_counter()
    while True:
        ids = [srv.submit(l, r, params_of(c), outputs=outs[(l.shape[1], l.shape[0])][k % nout])[0]
               for k, (l, r, c) in enumerate(pairs_pool[:min(max_batch * streams, queue)])]
        for rid in ids:
            srv.wait(rid)
        if time.perf_counter() - t_w > 1.0:
            break
    srv.reset_stats()
    clk = ClockSampler(torch.cuda.current_device())
    clk.__enter__()
    refused = 0
    t0 = time.perf_counter()
    for i in range(n):
        dt = t0 + arrivals[i] - time.perf_counter()
        if dt > 0:
            time.sleep(dt)
        l, r, c = pairs_pool[picks[i]]
        try:
            srv.submit(l, r, params_of(c), outputs=outs[(l.shape[1], l.shape[0])][i % nout])
        except ValueError:
            refused += 1
    srv.drain()
    clk.__exit__(None, None, None)
    st = srv.stats()
    tl = srv.timeline()
    srv.close()
    served = {"pairs_per_s": round(st["pairs_per_s"], 2), "p50_ms": round(st["p50_ms"], 3),
              "p99_ms": round(st["p99_ms"], 3), "p999_ms": round(st["p999_ms"], 3),
              "mean_batch": round(st["mean_batch"], 2), "completed": int(st["completed"]), "refused": refused,
              "timeline_ms": {k: round(v, 3) for k, v in tl.items()}, "clocks": clk.summary()}
    # (b) plain sequential compute() on the same arrival stream
    dev = torch.device("cuda")
    matchers, bufs = {}, {}
    for l, _, c in pairs_pool:
        key = (l.shape[1], l.shape[0], c)
        if key not in matchers:
            w, h = key[0], key[1]
            matchers[key] = pg.StereoMatcher(w, h, params_of(c))
            bufs[(w, h)] = dict(L=torch.empty((h, w), dtype=torch.uint8, device=dev),
                                R=torch.empty((h, w), dtype=torch.uint8, device=dev),
                                d16=torch.empty((h, w), dtype=torch.int16, device=dev),
                                d32=torch.empty((h, w), dtype=torch.float32, device=dev),
                                cf=torch.empty((h, w), dtype=torch.float32, device=dev))
    pinned = [(torch.from_numpy(l).pin_memory(), torch.from_numpy(r).pin_memory()) for l, r, _ in pairs_pool]
    host_out = {s: (torch.empty((s[1], s[0]), dtype=torch.int16).pin_memory(),
                    torch.empty((s[1], s[0]), dtype=torch.float32).pin_memory(),
                    torch.empty((s[1], s[0]), dtype=torch.float32).pin_memory()) for s in shapes}
    st = torch.cuda.Stream()
    lat = []
    t0 = time.perf_counter()
    clock = 0.0
    for i in range(n):
        clock = max(clock, arrivals[i])
        now = time.perf_counter() - t0
        if now < clock:
            time.sleep(clock - now)
        k = picks[i]
        l, r, c = pairs_pool[k]
        w, h = l.shape[1], l.shape[0]
        b = bufs[(w, h)]
        with torch.cuda.stream(st):
            b["L"].copy_(pinned[k][0], non_blocking=True)
            b["R"].copy_(pinned[k][1], non_blocking=True)
            matchers[(w, h, c)].compute_into(b["L"], b["R"], b["d16"], b["d32"], b["cf"], st)
            ho = host_out[(w, h)]
            ho[0].copy_(b["d16"], non_blocking=True)
            ho[1].copy_(b["d32"], non_blocking=True)
            ho[2].copy_(b["cf"], non_blocking=True)
        st.synchronize()
        done = time.perf_counter() - t0
        lat.append((done - arrivals[i]) * 1e3)
        clock = done
    lat.sort()
    plain = {"pairs_per_s": round(n / (clock - arrivals[0]), 2), "p50_ms": round(_pct(lat, 0.5), 3),
             "p99_ms": round(_pct(lat, 0.99), 3), "p999_ms": round(_pct(lat, 0.999), 3)}
    for m in matchers.values():
        m.close()
    return {"rate_pairs_per_s": rate, "requests": n, "max_batch": max_batch, "streams": streams,
            "server": served, "plain_sequential": plain}


def replica_max(dist, values, device) -> list:
    """Each timing's maximum over the ranks: the slowest replica bounds the
    job (replicas exchange nothing else)."""
    import torch
    t = torch.tensor(values, dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.tolist()]


def job_rate(world: int, units_per_rank: float, max_ms: float) -> float:
    """Whole-job throughput: the units of every rank over the slowest rank's time."""
    return world * units_per_rank / (max_ms / 1e3)


# profiled stages of the aggregation and the kernels behind them
AGG_STAGES = ("path_tb", "path_row", "wta", "tblr", "rlw", "tbw")
AGG_KERNELS = {"path_tb": "k_gtb/k_path_tb", "path_row": "k_grow/k_path_row", "wta": "k_wta",
               "tblr": "k_tblr", "rlw": "k_rlw", "tbw": "k_gtbw"}
PROF_NAMES = ["pyrdown", "features", "labels", "cost", "path_tb", "path_row", "post", "p2table", "wta", "tblr",
              "rlw", "tbw"]


def stage_bandwidth(prof: dict, peak_gbs: float) -> dict:
    """Algorithmic bytes over measured time for each profiled stage, in GB/s
    and as a fraction of the HBM peak (the issue-bound stages stay low)."""
    out = {}
    for k, v in prof.items():
        if v.get("launches") and v.get("ms", 0) > 0 and v.get("bytes", 0) > 0:
            gbs = v["bytes"] / (v["ms"] / 1e3) / 1e9
            out[k] = {"gbs": round(gbs, 1), "frac": round(gbs / peak_gbs, 4)}
    return out


def _pct(v, q):
    s = sorted(v)
    return s[max(0, min(len(s) - 1, int(round(q * (len(s) - 1)))))]


def result_line(args, world: int, headline: dict, plain: dict, pk: dict, npairs: int) -> dict:
    """The JSON line of a run from its measurements (`measure()` records of
    the headline and the plain per-pair runs, the HBM peak)."""
    value = job_rate(world, npairs, headline["total_ms"])
    e2e_value = job_rate(world, args.batch * headline["e2e_steps"], headline["e2e_total"])
    out = {
        "metric": METRIC, "value": round(value, 3), "unit": "pairs/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(headline["total_ms"] / args.steps, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int16",
        "data": "synthetic (seeded value-noise pairs, slanted-plane Voronoi ground truth; stands in for Middlebury)",
        "config": {"workload": "1920x1080 D=256 pyramid_levels=3, Census/BT alternating, adaptive P2, median, "
                   "disp16+disp32+conf", "pairs_per_step": args.batch, "width": W, "height": H,
                   "num_disparities": D, "pyramid_levels": LEVELS, "l2": "flushed (256 MB write) between steps",
                   "parallelism": f"replicas x{world}",
                   "execution": "plain per-pair compute()" if (args.mode == "plain" or args.impl == "reference")
                   else "batched: one BatchEngine run per step (CUDA graph), kernel shapes autotuned"},
        "e2e": {"value": round(e2e_value, 3), "unit": "pairs/s",
                "h2d_bytes_per_step": args.batch * 2 * W * H,
                "d2h_bytes_per_step": args.batch * W * H * (2 + 4 + 4),
                **({"trials_ms_per_step": headline["e2e_trials"]} if headline.get("e2e_trials") else {})},
        "gpu_launches": headline["launches"],
        "clocks": headline["clocks"],
        # the same rates per full-resolution pixel and per pixel-disparity
        "throughput": {"mpix_per_s": round(value * W * H / 1e6, 1),
                       "mpix_d_per_s": round(value * W * H * D / 1e6, 1),
                       "e2e_mpix_per_s": round(e2e_value * W * H / 1e6, 1)},
    }
    if plain["pair_ms"]:
        out["plain_compute"] = {"value": round(world * npairs / (plain["total_ms"] / 1e3), 3), "unit": "pairs/s",
                                "latency_ms_p50": round(_pct(plain["pair_ms"], 0.5), 4),
                                "latency_ms_p99": round(_pct(plain["pair_ms"], 0.99), 4)}
    if args.impl == "mine":
        prof = headline["prof"]
        ps = headline["prof_steps"]
        per_pair = {c: alg_bytes(W, H, params_for(c)) for c in (CENSUS, BT)}
        step_pairs = [CENSUS if i % 2 == 0 else BT for i in range(args.batch)]
        agg_alg = sum(per_pair[c]["aggregation"] for c in step_pairs)     # bytes per step
        tot_alg = sum(per_pair[c]["total"] for c in step_pairs)
        agg_keys = [k for k in AGG_STAGES if prof.get(k, {}).get("launches")]
        agg_ms = sum(prof[k]["ms"] for k in agg_keys) / ps
        agg_launches = sum(prof[k]["launches"] for k in agg_keys) / ps
        own = sum(prof[k]["bytes"] for k in agg_keys) / ps
        achieved = agg_alg / (agg_ms / 1e3) / 1e9 if agg_ms > 0 else None
        out["roofline"] = {
            "kernel": "aggregation (" + " + ".join(AGG_KERNELS[k] for k in agg_keys) + "), one step",
            "bound": "hbm",
            "achieved": round(achieved, 2) if achieved else None, "peak": pk["hbm_gbs"], "unit": "GB/s",
            "frac": round(achieved / pk["hbm_gbs"], 4) if achieved else None, "peak_source": pk["source"],
            "algorithmic": "4 B per voxel (partial aggregated volume written and read once as int16)",
            "alg_bytes_per_step": round(agg_alg / 1e9, 4),
            "implementation_bytes_per_step": round(own / 1e9, 4),
            "traffic": round(sum(AGG_TRAFFIC_PER_OWN_BYTE[k] * prof[k]["bytes"] for k in agg_keys) / ps / 1e9, 4)
            if all(k in AGG_TRAFFIC_PER_OWN_BYTE for k in agg_keys) else None,
            "traffic_unit": "GB per step (per kernel kind: ncu DRAM bytes per implementation byte x its "
                            "implementation bytes)",
            "ms_per_step": round(agg_ms, 4), "launches_per_step": agg_launches,
            "avg_launch_ms": round(agg_ms / agg_launches, 5) if agg_launches else None}
        step_ms = headline["total_ms"] / args.steps
        gbs = tot_alg / (step_ms / 1e3) / 1e9
        out["pipeline_roofline"] = {"alg_bytes_per_pair_mb": {("census" if c == CENSUS else "bt"):
                                                              round(per_pair[c]["total"] / 1e6, 1) for c in per_pair},
                                    "achieved": round(gbs, 1), "unit": "GB/s", "frac": round(gbs / pk["hbm_gbs"], 4)}
        out["kernels_ms_per_step"] = {k: round(v["ms"] / ps, 4) for k, v in prof.items() if v["launches"]}
        out["kernels_hbm"] = stage_bandwidth(prof, pk["hbm_gbs"])
    else:
        out["impl"] = "reference"
        out["reference_build"] = "reference src/sgm_kernels.cu + src/pyrdown.cu compiled unmodified for sm_103a"
    return out


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
    if args.impl == "reference":
        from tests import _oracle
        if not _oracle.ref_available():
            print(json.dumps({"impl": "reference", "unavailable": "reference kernels (oracle/_ref) not built"}))
            return None

    pairs = make_inputs(args.batch)
    stream = torch.cuda.Stream(device=dev)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)  # > 129 MB L2
    pk = peaks()
    npairs = args.batch * args.steps

    if args.impl == "reference":
        m = measure(ReferenceRunner(pairs, dev), args, stream, flush, dev, 1, dist, False, True)
        headline, plain = m, m
    else:
        plain = measure(MineRunner(pairs, dev), args, stream, flush, dev, world, dist, False, True)
        headline = plain if args.mode == "plain" else \
            measure(BatchRunner(pairs, dev), args, stream, flush, dev, world, dist, True, False)
        if args.mode == "plain":
            headline = measure(MineRunner(pairs, dev), args, stream, flush, dev, world, dist, True, True)
    if rank != 0:
        return None
    # the reference arm runs on rank 0 alone
    out = result_line(args, 1 if args.impl == "reference" else world, headline, plain, pk, npairs)
    value = out["value"]
    if args.impl == "mine" and args.mode == "batched":
        import pyrsgm_gb300 as pg
        out["autotune"] = pg.autotune_table()
        pg.set_autotune(False)
    if args.impl == "mine" and world == 1:
        out["latency_1080p_d256_l2_census"] = single_pair_latency(dev, stream)
    if args.impl == "mine" and world == 1:
        out["batched_mixed"] = batched_mixed(dev, stream, flush)
    if args.impl == "mine" and world == 1 and args.serve_requests > 0:
        import pyrsgm_gb300 as pg
        # below and above the server's capacity (its outputs' copies to host
        # memory bound it); plain compute is overloaded at both
        out["serving"] = [serve_compare(pairs, lambda c: pg.Params(**params_for(c)), round(f * value, 1),
                                        args.serve_requests) for f in (0.35, 0.7)]
        pool, cfg = mixed_pool(args.pool)
        out["serving_mixed"] = [serve_compare(pool, lambda k: cfg[k], r, args.mixed_requests, seed=int(r))
                                for r in args.mixed_rates]
    if not args.no_cpu and world == 1:
        out["cpu_baseline"] = cpu_baseline(pairs)
    return out


def single_pair_latency(dev, stream, runs: int = 20) -> dict:
    """One 1920x1080 D=256 pyramid_levels=2 Census pair through plain
    compute() (disp16 + disp32 + conf), device-resident, per-call CUDA
    events; p50/p99 over `runs` calls after 3 warm-ups."""
    import torch
    import pyrsgm_gb300 as pg
    from pyrsgm_gb300 import synth
    p = pg.Params(**{**params_for(CENSUS), "pyramid_levels": 2})
    left, right, _ = synth.make_pair(W, H, D - 1, 16, 7000)
    m = pg.StereoMatcher(W, H, p)
    L, R = torch.from_numpy(left).to(dev), torch.from_numpy(right).to(dev)
    d16 = torch.empty((H, W), dtype=torch.int16, device=dev)
    d32 = torch.empty((H, W), dtype=torch.float32, device=dev)
    cf = torch.empty((H, W), dtype=torch.float32, device=dev)
    ms = []
    for k in range(3 + runs):
        with torch.cuda.stream(stream):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            m.compute_into(L, R, d16, d32, cf, stream)
            b.record(stream)
        torch.cuda.synchronize()
        if k >= 3:
            ms.append(a.elapsed_time(b))
    m.close()
    # the opt-in speckle filter on that disparity map (regions <= 100 px, 1 px steps)
    src = d16.clone()
    sp = []
    for k in range(3 + runs):
        with torch.cuda.stream(stream):
            d16.copy_(src)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            pg.filter_speckles(d16, pg.invalid_disparity16(p), 100, 16, stream)
            b.record(stream)
        torch.cuda.synchronize()
        if k >= 3:
            sp.append(a.elapsed_time(b))
    return {"p50_ms": round(_pct(ms, 0.5), 4), "p99_ms": round(_pct(ms, 0.99), 4), "runs": runs,
            "levels": [(li.width, li.height, li.num_labels) for li in pg.level_geometry(W, H, p)],
            "speckle_filter_p50_ms": round(_pct(sp, 0.5), 4)}


MIX_SIZES = [(640, 480), (960, 540), (1280, 720), (1920, 1080)]


def mixed_params(rng) -> dict:
    """Parameters of one pair of the mixed workload: D from {64, 128, 256},
    pyramid_levels 1-4, Census / BT 50/50 (each with the penalties the
    1080p workload uses), adaptive P2 and median on."""
    D = int(rng.choice([64, 128, 256]))
    L = int(rng.integers(1, 5))
    c = int(rng.integers(2))
    return dict(num_disparities=D, pyramid_levels=L, cost_mode=c, p1=8 if c == CENSUS else 300,
                p2=32 if c == CENSUS else 2400, adaptive_p2=True, median_filter=True, lr_check=True,
                uniqueness_ratio=10, pyramid_coarse_disparities=128)


def mixed_images():
    """One seeded synthetic pair per size of the mixed workload (disparities
    up to 255, 10 slanted patches); the pairs of the workload reuse them."""
    from pyrsgm_gb300 import synth
    return {s: synth.make_pair(s[0], s[1], 255, 10, 4000 + k)[:2] for k, s in enumerate(MIX_SIZES)}


def mixed_pool(n: int, seed: int = 4000):
    """n pairs drawn like the mixed workload: sizes 25 % each of
    640x480 / 960x540 / 1280x720 / 1920x1080, parameters from mixed_params."""
    import pyrsgm_gb300 as pg
    import numpy as np
    rng = np.random.default_rng(seed)
    imgs = mixed_images()
    pool, cfg = [], []
    for i in range(n):
        s = MIX_SIZES[int(rng.integers(len(MIX_SIZES)))]
        left, right = imgs[s]
        pool.append((left, right, i))
        cfg.append(pg.Params(**mixed_params(rng)))
    return pool, cfg


def batched_mixed(dev, stream, flush, npairs: int = 64, steps: int = 10) -> dict:
    """The mixed batched workload: `npairs` pairs drawn like mixed_pool
    (seeded; sizes, D, depth, cost per pair) in one BatchEngine run per step
    (a CUDA graph after the first run; kernel shapes autotuned), against the
    same pairs through per-pair StereoMatcher::compute(), both device-resident
    with CUDA events on the compute stream and the L2 flushed between steps."""
    import numpy as np
    import torch
    import pyrsgm_gb300 as pg
    rng = np.random.default_rng(4000)
    imgs = {s: (torch.from_numpy(l).to(dev), torch.from_numpy(r).to(dev)) for s, (l, r) in mixed_images().items()}
    items, shapes = [], []
    for i in range(npairs):
        w, h = MIX_SIZES[i % 4] if i < 4 else MIX_SIZES[int(rng.integers(len(MIX_SIZES)))]
        p = mixed_params(rng)
        L, R = imgs[(w, h)]
        items.append(dict(left=L, right=R, params=pg.Params(**p),
                          disp16=torch.empty((h, w), dtype=torch.int16, device=dev),
                          disp32=torch.empty((h, w), dtype=torch.float32, device=dev),
                          conf=torch.empty((h, w), dtype=torch.float32, device=dev)))
        shapes.append((w, h))
    prev = pg.set_autotune(True)
    eng = pg.BatchEngine(60 << 30)
    arr = pg.BatchEngine.make_pairs(items)

    def timed(fn, n):
        ms = []
        for _ in range(n):
            with torch.cuda.stream(stream):
                flush.fill_(5)
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                fn()
                b.record(stream)
            torch.cuda.synchronize()
            ms.append(a.elapsed_time(b))
        return ms

    for _ in range(3):
        eng.run_pairs(arr, True, stream)
    torch.cuda.synchronize()
    bms = timed(lambda: eng.run_pairs(arr, True, stream), steps)
    pg.set_autotune(prev)
    eng.close()
    matchers = {}
    for it in items:
        key = (it["left"].shape[1], it["left"].shape[0], tuple(sorted(vars(it["params"]).items())))
        if key not in matchers:
            matchers[key] = pg.StereoMatcher(key[0], key[1], it["params"])
        it["m"] = matchers[key]

    def plain():
        for it in items:
            it["m"].compute_into(it["left"], it["right"], it["disp16"], it["disp32"], it["conf"], stream)

    plain()
    torch.cuda.synchronize()
    pms = timed(plain, 3)
    for m in matchers.values():
        m.close()
    mpix = sum(w * h for w, h in shapes) / 1e6
    bstep, pstep = statistics.median(bms), statistics.median(pms)
    return {"pairs_per_step": npairs, "value": round(npairs / (bstep / 1e3), 2), "unit": "pairs/s",
            "ms_per_step": round(bstep, 4), "mpix_per_s": round(mpix / (bstep / 1e3), 1),
            "plain_compute": {"value": round(npairs / (pstep / 1e3), 2), "ms_per_step": round(pstep, 4)},
            "workload": "sizes 25 % each of 640x480 / 960x540 / 1280x720 / 1920x1080, D in {64,128,256}, "
                        "pyramid_levels 1-4, Census/BT 50/50, seeded; one synthetic image pair per size",
            "l2": "flushed (256 MB write) between steps"}


def stage_times(args) -> None:
    """One batch-engine run of --batch 1080p D=256 L3 pairs (Census and BT
    alternating, the headline workload), without a graph, after --warmup
    runs: prints the per-stage CUDA-event times of the library profiler as
    one JSON line.  --packed-words forces a shape of the 16/32/64-label
    aggregation (0 = chosen per launch), --fused the fused two-pass form.
    This is the run the per-kernel ncu summaries capture."""
    import torch
    import pyrsgm_gb300 as pg
    from pyrsgm_gb300._native import lib
    torch.cuda.set_device(0)
    pg.set_packed_words(args.packed_words)
    pg.set_fused(args.fused)
    pg.set_autotune(False)
    items = []
    for left, right, c in make_inputs(args.batch):
        items.append(dict(left=torch.from_numpy(left).cuda(), right=torch.from_numpy(right).cuda(),
                          params=pg.Params(**params_for(c)),
                          disp16=torch.empty((H, W), dtype=torch.int16, device="cuda"),
                          disp32=torch.empty((H, W), dtype=torch.float32, device="cuda"),
                          conf=torch.empty((H, W), dtype=torch.float32, device="cuda")))
    eng = pg.BatchEngine(40 << 30)
    st = torch.cuda.Stream()
    for _ in range(args.warmup):
        eng.run(items, use_graph=False, stream=st)
    torch.cuda.synchronize()
    lib().pyrsgm_gb300_profile(1)
    eng.run(items, use_graph=False, stream=st)
    torch.cuda.synchronize()
    out = {}
    for k, nm in enumerate(PROF_NAMES):
        ms, cnt, by = C.c_double(), C.c_longlong(), C.c_double()
        lib().pyrsgm_gb300_profile_read(k, C.byref(ms), C.byref(cnt), C.byref(by))
        if cnt.value:
            out[nm] = {"ms": round(ms.value, 4), "launches": cnt.value,
                       "gbs": round(by.value / ms.value / 1e6, 1) if ms.value else 0.0}
    lib().pyrsgm_gb300_profile(0)
    eng.close()
    print(json.dumps({"mode": "stages", "pairs": args.batch, "packed_words": args.packed_words,
                      "fused": bool(args.fused), "stages": out,
                      "total_ms": round(sum(v["ms"] for v in out.values()), 4)}), flush=True)


def serve_sweep(args) -> None:
    """Serving on the mixed stream (sizes 640x480..1920x1080, D in {64,128,256},
    pyramid levels 1-4, Census/BT): one JSON line per arrival rate."""
    import torch
    torch.cuda.set_device(0)
    pool, cfg = mixed_pool(args.pool)
    for rate in args.rates:
        res = serve_compare(pool, lambda k: cfg[k], rate, args.serve_requests, seed=int(rate),
                            max_batch=args.serve_batch, streams=args.serve_streams)
        print(json.dumps({"metric": "mixed-stream serving", **res}), flush=True)


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--batch", type=int, default=32, help="pairs per step")
    ap.add_argument("--impl", choices=["mine", "reference"], default="mine")
    ap.add_argument("--mode", choices=["batched", "plain", "serve", "stages"], default="batched",
                    help="headline execution: one batched run per step, or per-pair compute(); "
                         "'serve' sweeps arrival rates on the mixed-size stream; "
                         "'stages' prints the per-stage times of one batched run")
    ap.add_argument("--packed-words", type=int, default=0,
                    help="stages: 16/32/64-label aggregation shape (0 = per launch, 8, 4 or 2)")
    ap.add_argument("--fused", action="store_true", help="stages: fused two-pass 16-label aggregation")
    ap.add_argument("--serve-requests", type=int, default=400,
                    help="requests of the serving comparison (0 skips it)")
    ap.add_argument("--mixed-requests", type=int, default=1000,
                    help="requests per rate of the mixed-stream serving comparison in the default line")
    ap.add_argument("--mixed-rates", type=float, nargs="*", default=[1000, 4000, 16000])
    ap.add_argument("--rates", type=float, nargs="*", default=[500, 1000, 2000, 5000, 10000, 20000])
    ap.add_argument("--pool", type=int, default=24, help="distinct pairs (shapes, parameters) of the mixed stream")
    ap.add_argument("--serve-batch", type=int, default=16, help="server: largest batch")
    ap.add_argument("--serve-streams", type=int, default=2, help="server: stream lanes")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.mode == "serve":
        serve_sweep(args)
        return
    if args.mode == "stages":
        stage_times(args)
        return
    out = run(args)
    if out is not None:
        print(json.dumps(out))


if __name__ == "__main__":
    main()
