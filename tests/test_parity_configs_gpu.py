"""Parity at the sizes the benchmarks run, against the reference's own kernels.

Each configuration is the workload a benchmark line is quoted on, at full
size, on the seeded synthetic pairs (pair i of configuration k uses seed
1000 k + i):

  * 640x480, D=64, single-scale Birchfield-Tomasi (block 5, P1=200, P2=800,
    uniqueness 10, pseudo-LR check, no median) through
    pyrsgm_compute_single_scale, and the same pair with pyramid_levels=1
    level by level through pyrsgm_compute_level;
  * 1280x720 Census, D=128, pyramid_levels=2, level by level;
  * 1920x1080, D=256: pyramid_levels=3 Birchfield-Tomasi and
    pyramid_levels=2 Census (the single-pair latency configuration), level
    by level, adaptive P2 and median on;
  * a mix of pairs drawn like the batched workload (640x480 ... 1920x1080,
    D 64/128/256, 1-4 levels, Census / Birchfield-Tomasi) run together
    through the batch engine and through the server, each pair against the
    reference kernels on the reference's StereoMatcher schedule.

Level by level means: every level's cost volume and aggregated volume
(bit-exact), disparity x16 (bit-exact), confidence and float disparity
(within 1e-6 absolute), each side fed its own coarser result.  Both kernel
shapes of the 16/32/64-label aggregation run (one thread per 16 labels, and
a chain spread over several threads).
"""
from __future__ import annotations

import numpy as np
import pytest

from tests import _oracle, _runners, cases

pytestmark = pytest.mark.gpu

TOL = 1e-6   # absolute, float disparity and confidence


def _need_ref():
    if not _oracle.ref_available():
        pytest.fail("reference kernels (oracle/_ref/*.fatbin + harness) are not available")


def _pair(w, h, dmax, patches, seed):
    from pyrsgm_gb300 import synth
    left, right, _ = synth.make_pair(w, h, dmax, patches, seed)
    return left, right


def _check_levels(records):
    for rec in records:
        tag = f"level {rec['level']} ({rec['w']}x{rec['h']}, {rec['D']} labels)"
        np.testing.assert_array_equal(rec["mine"]["left"], rec["ref"]["left"], err_msg=f"{tag} pyramid left")
        np.testing.assert_array_equal(rec["mine"]["right"], rec["ref"]["right"], err_msg=f"{tag} pyramid right")
        bad = _runners.compare(rec["mine"], rec["ref"])
        assert not bad, (tag, bad)
        assert int((rec["mine"]["disp16"] > 0).sum()) > 0, tag


def _with_words(words, fn):
    import pyrsgm_gb300 as pg
    prev = pg.set_packed_words(words)
    try:
        return fn()
    finally:
        pg.set_packed_words(prev)


C1_PAIR = None


def _c1_pair():
    global C1_PAIR
    if C1_PAIR is None:
        C1_PAIR = _pair(640, 480, 63, 6, 1000)
    return C1_PAIR


@pytest.mark.parametrize("words", [0, 8, 2])
def test_c1_640x480_d64_single_scale_bt(words):
    _need_ref()
    case = cases._ss("c1_640x480_d64_bt", 640, 480, 64, cases.BT, bs=5, P1=200, P2=800, uniq=10,
                     post=cases.LRC)
    case["pair"] = _c1_pair()
    mine = _with_words(words, lambda: _runners.run_mine(case))
    ref = _runners.run_ref(case)
    bad = _runners.compare(mine, ref)
    assert not bad, bad
    assert int((mine["disp16"] > 0).sum()) > 640 * 480 // 2


@pytest.mark.parametrize("D,cost", [(96, cases.CENSUS), (48, cases.BT)], ids=["census_d96", "bt_d48"])
def test_640x480_single_scale_label_counts_outside_the_packed_kernels(D, cost):
    """Label counts other than 16/32/64 take the lane-parallel path kernels
    (k_path_tb, k_path_row with its fused WTA and LR check): the C1 pair at
    full size, cost and aggregated volumes included."""
    _need_ref()
    case = cases._ss(f"c1_640x480_d{D}", 640, 480, D, cost, bs=5, uniq=10, post=cases.LRC, adaptive=True)
    case["pair"] = _c1_pair()
    mine = _runners.run_mine(case)
    bad = _runners.compare(mine, _runners.run_ref(case))
    assert not bad, bad
    assert int((mine["disp16"] > 0).sum()) > 640 * 480 // 4


@pytest.mark.parametrize("words", [0, 8])
def test_c1_640x480_d64_one_pyramid_level_bt(words):
    _need_ref()
    left, right = _c1_pair()
    params = dict(num_disparities=64, pyramid_levels=1, cost_mode=cases.BT, block_size=5, p1=200, p2=800,
                  uniqueness_ratio=10, lr_check=True, median_filter=False)
    _check_levels(_with_words(words, lambda: _runners.matcher_levels(640, 480, params, left, right)))


@pytest.mark.parametrize("words", [0, 8, 2])
def test_c2_1280x720_census_d128_two_levels(words):
    _need_ref()
    left, right = _pair(1280, 720, 127, 10, 2000)
    params = dict(num_disparities=128, pyramid_levels=2, cost_mode=cases.CENSUS, p1=8, p2=32)
    _check_levels(_with_words(words, lambda: _runners.matcher_levels(1280, 720, params, left, right)))


def _c3_params(cost, levels):
    return dict(num_disparities=256, pyramid_levels=levels, cost_mode=cost,
                p1=8 if cost == cases.CENSUS else 300, p2=32 if cost == cases.CENSUS else 2400,
                adaptive_p2=True, median_filter=True, lr_check=True, uniqueness_ratio=10,
                pyramid_coarse_disparities=128)


@pytest.mark.parametrize("words,tbw", [(0, 1), (8, 2), (8, 0)], ids=["auto", "wide", "wide_three_pass"])
def test_c3_1920x1080_d256_bt_three_levels(words, tbw):
    """The 16-label levels with the winner-take-all in the T->B pass (the
    default) and in a pass of its own."""
    import pyrsgm_gb300 as pg
    _need_ref()
    left, right = _pair(1920, 1080, 255, 16, 3001)
    prev = pg.set_tbw(tbw)
    try:
        records = _with_words(words, lambda: _runners.matcher_levels(1920, 1080, _c3_params(cases.BT, 3), left, right))
    finally:
        pg.set_tbw(prev)
    _check_levels(records)


@pytest.mark.parametrize("words", [0, 8])
def test_c3_1920x1080_d256_census_two_levels_latency_config(words):
    """The single-pair latency configuration: coarse level 480x270 with 64 labels."""
    _need_ref()
    left, right = _pair(1920, 1080, 255, 16, 3000)
    records = _with_words(words, lambda: _runners.matcher_levels(
        1920, 1080, _c3_params(cases.CENSUS, 2), left, right))
    assert (records[0]["w"], records[0]["h"], records[0]["D"]) == (480, 270, 64)
    _check_levels(records)


# ---------------------------------------------------------------------------
# the batched / served mix at real sizes
# ---------------------------------------------------------------------------
MIX_SIZES = [(640, 480), (960, 540), (1280, 720), (1920, 1080)]


def mix(n: int, seed: int = 4000):
    """Pairs drawn like the batched workload: sizes 25% each, D from
    {64, 128, 256}, pyramid_levels 1-4, Census / BT 50/50, adaptive P2 and
    median on; each with the parameters the benchmark uses for its cost."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        w, h = MIX_SIZES[i % 4] if i < 4 else MIX_SIZES[int(rng.integers(4))]
        D = int(rng.choice([64, 128, 256]))
        L = int(rng.integers(1, 5))
        cost = int(i % 2) if i < 4 else int(rng.integers(2))
        params = dict(num_disparities=D, pyramid_levels=L, cost_mode=cost,
                      p1=8 if cost == cases.CENSUS else 300, p2=32 if cost == cases.CENSUS else 2400,
                      adaptive_p2=True, median_filter=True, lr_check=True, uniqueness_ratio=10,
                      pyramid_coarse_disparities=128)
        left, right = _pair(w, h, D - 1, 16, seed + i)
        out.append((w, h, params, left, right))
    return out


def _ref_outputs(w, h, params, left, right):
    import torch
    L, R = torch.from_numpy(left).cuda(), torch.from_numpy(right).cuda()
    r16 = torch.zeros((h, w), dtype=torch.int16, device="cuda")
    r32 = torch.zeros((h, w), dtype=torch.float32, device="cuda")
    rcf = torch.zeros((h, w), dtype=torch.float32, device="cuda")
    _runners._ref_matcher(dict(w=w, h=h, params=params), L, R, r16, r32, rcf)
    return dict(disp16=r16.cpu().numpy(), disp32=r32.cpu().numpy(), conf=rcf.cpu().numpy())


def _assert_same(got, want, tag):
    np.testing.assert_array_equal(got["disp16"], want["disp16"], err_msg=f"{tag} disp16")
    np.testing.assert_allclose(got["disp32"], want["disp32"], rtol=0, atol=TOL, err_msg=f"{tag} disp32")
    np.testing.assert_allclose(got["conf"], want["conf"], rtol=0, atol=TOL, err_msg=f"{tag} conf")
    assert int((got["disp16"] > 0).sum()) > 0, tag


@pytest.mark.parametrize("use_graph", [True, False])
def test_c4_mixed_real_size_batch_matches_reference_kernels(use_graph):
    import torch
    import pyrsgm_gb300 as pg
    _need_ref()
    pairs = mix(12)
    items, outs = [], []
    for w, h, params, left, right in pairs:
        o = dict(disp16=torch.full((h, w), 77, dtype=torch.int16, device="cuda"),
                 disp32=torch.full((h, w), -1.0, dtype=torch.float32, device="cuda"),
                 conf=torch.full((h, w), -1.0, dtype=torch.float32, device="cuda"))
        items.append(dict(left=torch.from_numpy(left).cuda(), right=torch.from_numpy(right).cuda(),
                          params=pg.Params(**params), **o))
        outs.append(o)
    eng = pg.BatchEngine(40 << 30)
    st = torch.cuda.Stream()
    torch.cuda.synchronize()
    eng.run(items, use_graph=use_graph, stream=st)
    if use_graph:   # the replay of the captured graph gives the same
        torch.cuda.synchronize()
        for o in outs:
            o["disp16"].fill_(77)
        eng.run(items, use_graph=True, stream=st)
    torch.cuda.synchronize()
    for i, (w, h, params, left, right) in enumerate(pairs):
        got = {k: v.cpu().numpy() for k, v in outs[i].items()}
        _assert_same(got, _ref_outputs(w, h, params, left, right),
                     f"pair {i} {w}x{h} D={params['num_disparities']} L={params['pyramid_levels']}")
    eng.close()


def test_c4_mixed_real_size_served_matches_reference_kernels():
    import pyrsgm_gb300 as pg
    _need_ref()
    pairs = mix(8, seed=5000)
    srv = pg.Server(40 << 30, max_batch=4, streams=2)
    subs = [srv.submit(left, right, pg.Params(**params), True, True, True) for w, h, params, left, right in pairs]
    for rid, _ in subs:
        assert srv.wait(rid, 120.0) == 1, getattr(srv, "last_error", rid)
    for i, (w, h, params, left, right) in enumerate(pairs):
        got = subs[i][1]
        _assert_same(got, _ref_outputs(w, h, params, left, right),
                     f"request {i} {w}x{h} D={params['num_disparities']} L={params['pyramid_levels']}")
    srv.close()
