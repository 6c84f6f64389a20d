"""Continuous-batching server: requests of mixed sizes, label counts, depths
and costs submitted from several threads while earlier batches are still on
the GPU; every result must equal StereoMatcher::compute of that pair alone
(disparity x16 bit-exact, float outputs within 1e-6).  Failures stay per
request: an invalid request is refused at submission without disturbing the
others, a batch failing on the host (injected) fails only its own requests,
and a full queue refuses new work."""
from __future__ import annotations

import threading

import numpy as np
import pytest
import torch

import pyrsgm_gb300 as pg
from pyrsgm_gb300 import synth

pytestmark = pytest.mark.gpu

SIZES = [(160, 96), (200, 120), (128, 72)]


def _requests(n, seed=6000):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        w, h = SIZES[rng.integers(len(SIZES))]
        D = int(rng.choice([32, 64, 96]))
        cost = int(rng.integers(2))
        p = pg.Params(num_disparities=D, pyramid_levels=int(rng.integers(0, 4)), cost_mode=cost,
                      p1=8 if cost else 300, p2=32 if cost else 2400, adaptive_p2=bool(rng.integers(2)))
        left, right, _ = synth.make_pair(w, h, max(4, min(D - 1, w // 3)), 5, seed + i)
        out.append((p, left, right))
    return out


def _alone(p, left, right):
    h, w = left.shape
    m = pg.StereoMatcher(w, h, p)
    r = m.compute(torch.from_numpy(left).cuda(), torch.from_numpy(right).cuda(), True, True, True)
    torch.cuda.synchronize()
    m.close()
    return {k: v.cpu().numpy() for k, v in r.items()}


def test_results_in_the_mix_equal_results_alone():
    reqs = _requests(24)
    srv = pg.Server(4 << 30, max_batch=6, streams=2)
    ids = [None] * len(reqs)

    def submitter(k):
        for i in range(k, len(reqs), 3):
            p, left, right = reqs[i]
            ids[i] = srv.submit(left, right, p, True, True, True)

    ts = [threading.Thread(target=submitter, args=(k,)) for k in range(3)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    for i, (p, left, right) in enumerate(reqs):
        rid, out = ids[i]
        assert srv.wait(rid, 60.0) == 1
        want = _alone(p, left, right)
        np.testing.assert_array_equal(out["disp16"], want["disp16"], err_msg=f"request {i}")
        np.testing.assert_allclose(out["disp32"], want["disp32"], rtol=0, atol=1e-6)
        np.testing.assert_allclose(out["conf"], want["conf"], rtol=0, atol=1e-6)
    st = srv.stats()
    assert st["completed"] == len(reqs) and st["failed"] == 0
    assert st["p50_ms"] > 0 and st["p99_ms"] >= st["p50_ms"]
    srv.close()


def test_invalid_request_is_refused_and_others_still_served():
    reqs = _requests(4, seed=6100)
    srv = pg.Server(2 << 30, max_batch=4, streams=2)
    p, left, right = reqs[0]
    with pytest.raises(ValueError, match="invalid request"):
        srv.submit(left, right, pg.Params(pyramid_levels=9))
    with pytest.raises(ValueError, match="budget"):
        big = np.zeros((4000, 6000), np.uint8)
        srv.submit(big, big, pg.Params(num_disparities=1024))
    got = [srv.submit(l, r, q) for q, l, r in reqs]
    for (rid, out), (q, l, r) in zip(got, reqs):
        assert srv.wait(rid, 60.0) == 1
        np.testing.assert_array_equal(out["disp16"], _alone(q, l, r)["disp16"])
    srv.close()


def test_injected_batch_failure_fails_only_that_batch():
    reqs = _requests(6, seed=6200)
    srv = pg.Server(2 << 30, max_batch=1, streams=1)
    srv.inject_failure(1)
    got = [srv.submit(l, r, q) for q, l, r in reqs]
    status = [srv.wait(rid, 60.0) for rid, _ in got]
    assert status.count(-1) == 1 and status.count(1) == len(reqs) - 1
    assert "injected" in srv.last_error
    for s, (rid, out), (q, l, r) in zip(status, got, reqs):
        if s == 1:
            np.testing.assert_array_equal(out["disp16"], _alone(q, l, r)["disp16"])
    st = srv.stats()
    assert st["failed"] == 1
    srv.close()


def test_full_queue_refuses():
    reqs = _requests(1, seed=6300)
    q, l, r = reqs[0]
    srv = pg.Server(2 << 30, max_batch=1, streams=1, max_queue=1)
    refused = 0
    ids = []
    for _ in range(64):
        try:
            ids.append(srv.submit(l, r, q)[0])
        except ValueError as e:
            assert "queue full" in str(e)
            refused += 1
    assert refused > 0
    for rid in ids:
        assert srv.wait(rid, 60.0) == 1
    srv.close()


def test_registered_buffers_are_copied_in_place():
    """Images and outputs the caller registered (page-locked) skip the staging
    copies; results equal those of the pair alone, also when only some of a
    request's buffers are registered."""
    reqs = _requests(8, seed=6100)
    srv = pg.Server(2 << 30, max_batch=4, streams=2)
    subs = []
    for i, (p, left, right) in enumerate(reqs):
        h, w = left.shape
        left = np.ascontiguousarray(left)
        right = np.ascontiguousarray(right)
        out = {"disp16": np.empty((h, w), np.int16), "disp32": np.empty((h, w), np.float32),
               "conf": np.empty((h, w), np.float32)}
        regs = [left, right] + list(out.values())
        for j, a in enumerate(regs):
            if (i + j) % 3 != 0:  # leave some buffers to the staging path
                srv.register(a)
        rid, _ = srv.submit(left, right, p, outputs=out)
        subs.append((rid, p, left, right, out))
    for rid, p, left, right, out in subs:
        assert srv.wait(rid) == 1, getattr(srv, "last_error", "")
        ref = _alone(p, left, right)
        np.testing.assert_array_equal(out["disp16"], ref["disp16"])
        np.testing.assert_allclose(out["disp32"], ref["disp32"], atol=1e-6, rtol=0)
        np.testing.assert_allclose(out["conf"], ref["conf"], atol=1e-6, rtol=0)
    srv.close()


def test_reserved_plans_serve_bursts_without_allocation():
    """Plans reserved up front in the server's pool (shared by its lanes): a
    burst of that shape runs on them and gives the results of each pair
    alone; a reservation beyond the server's budget is refused."""
    p = pg.Params(num_disparities=64, pyramid_levels=1, cost_mode=pg.COST_CENSUS, p1=8, p2=32)
    w, h = 160, 96
    one = pg.pair_bytes(w, h, p)
    srv = pg.Server(64 * one, max_batch=4, streams=2)
    srv.reserve(w, h, p, 4)
    reqs = [synth.make_pair(w, h, 40, 5, 6500 + i)[:2] for i in range(8)]
    ids = [srv.submit(l, r, p, True, True, True) for l, r in reqs]
    for (l, r), (rid, out) in zip(reqs, ids):
        assert srv.wait(rid, 60.0) == 1
        want = _alone(p, l, r)
        np.testing.assert_array_equal(out["disp16"], want["disp16"])
        np.testing.assert_allclose(out["conf"], want["conf"], rtol=0, atol=1e-6)
    with pytest.raises(RuntimeError, match="budget"):
        srv.reserve(w, h, p, 65)   # 65 plans > the 64-plan budget
    srv.close()


def test_batch_reserve_allocates_plans_up_front():
    p = pg.Params(num_disparities=64, pyramid_levels=1)
    one = pg.pair_bytes(160, 96, p)
    eng = pg.BatchEngine(8 * one)
    eng.reserve(160, 96, p, 3)
    assert eng.bytes_in_use() == 3 * one
    eng.reserve(160, 96, p, 2)   # already there
    assert eng.bytes_in_use() == 3 * one
    with pytest.raises(RuntimeError, match="budget"):
        eng.reserve(160, 96, p, 9)
    assert eng.bytes_in_use() == 8 * one   # filled up to the budget before refusing
    eng.close()
