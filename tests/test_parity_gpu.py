"""Parity on the GPU: the CUDA library against the CPU oracle and against the
reference's own kernels (run from oracle/_ref through the harness), on the
same seeded inputs.  Integer outputs (disparity x16, cost volume, aggregated
volume) must match bit for bit; disp32 and confidence within 1e-6 absolute.
"""
from __future__ import annotations

import numpy as np
import pytest

from tests import _oracle, _runners, cases

pytestmark = pytest.mark.gpu

ALL_CASES = cases.SINGLE_SCALE + cases.LEVELS + cases.MATCHER
IDS = [c["name"] for c in ALL_CASES]


@pytest.mark.parametrize("case", ALL_CASES, ids=IDS)
def test_cuda_matches_oracle(case):
    lut = _runners.device_lut(case)
    mine = _runners.run_mine(case)
    orc = _runners.run_oracle(case, lut)
    bad = _runners.compare(mine, orc)
    assert not bad, bad


def _need_ref():
    if not _oracle.ref_available():
        pytest.fail("reference kernels (oracle/_ref/*.fatbin + harness) are not available")


@pytest.mark.parametrize("case", ALL_CASES, ids=IDS)
def test_cuda_matches_reference_kernels(case):
    _need_ref()
    mine = _runners.run_mine(case)
    ref = _runners.run_ref(case)
    bad = _runners.compare(mine, ref)
    assert not bad, bad


@pytest.mark.parametrize("case", ALL_CASES, ids=IDS)
def test_oracle_matches_reference_kernels(case):
    _need_ref()
    lut = _runners.device_lut(case)
    orc = _runners.run_oracle(case, lut)
    ref = _runners.run_ref(case)
    bad = _runners.compare(orc, ref)
    assert not bad, bad


@pytest.mark.parametrize("w,h", cases.PYRDOWN)
def test_pyrdown_matches_reference(w, h):
    import torch
    import pyrsgm_gb300 as pg
    src = cases.pyrdown_input(w, h)
    mine = pg.pyrdown(torch.from_numpy(src).cuda()).cpu().numpy()
    np.testing.assert_array_equal(mine, _oracle.orc_pyrdown(src))
    if _oracle.ref_available():
        np.testing.assert_array_equal(mine, _runners.run_ref_pyrdown(src))


def test_pyrdown_pitched_views():
    """Pitched (strided) source and destination, as from cudaMallocPitch."""
    import torch
    import pyrsgm_gb300 as pg
    src = cases.pyrdown_input(97, 48)
    big = torch.zeros((48, 128), dtype=torch.uint8, device="cuda")
    big[:, :97] = torch.from_numpy(src).cuda()
    dst_big = torch.zeros((24, 64), dtype=torch.uint8, device="cuda")
    pg.pyrdown(big[:, :97], dst_big[:, :49])
    np.testing.assert_array_equal(dst_big[:, :49].cpu().numpy(), _oracle.orc_pyrdown(src))
    assert int(dst_big[:, 49:].abs().sum()) == 0


def test_p2_table_matches_libm_closely():
    """The device table uses __expf; libm expf may round differently near .5,
    but never by more than one P2 step."""
    for P2, a in ((2400, cases.P2_DEFAULT), (32, cases.P2_SMOKE), (800, (0.0, 5.0, 0.2, 1.0))):
        case = dict(kind="ss", adaptive=True, P2=P2, p2p=a)
        dev = _runners.device_lut(case)
        host = _oracle.p2_table_libm(P2, *a)
        assert np.max(np.abs(dev.astype(np.int64) - host)) <= 1


PACKED = [c for c in cases.SINGLE_SCALE + cases.LEVELS if c["D"] in (16, 32, 64)]


# kernel shapes of the 16/32/64-label aggregation: (words per thread, fused
# passes for 16-label pyramid levels, mode of the T->B pass with the
# winner-take-all for 16-label pyramid levels: 2 always, 0 never)
SHAPES = [(8, True, 1), (8, False, 2), (8, False, 0), (2, True, 1)]
SHAPE_IDS = ["wide_fused", "wide", "wide_three_pass", "spread"]


def _run_shape(case, words, fused, tbw):
    import pyrsgm_gb300 as pg
    prev = pg.set_packed_words(words)
    prev_f = pg.set_fused(fused)
    prev_t = pg.set_tbw(tbw)
    try:
        return _runners.run_mine(case)
    finally:
        pg.set_packed_words(prev)
        pg.set_fused(prev_f)
        pg.set_tbw(prev_t)


@pytest.mark.parametrize("words,fused,tbw", SHAPES, ids=SHAPE_IDS)
@pytest.mark.parametrize("case", PACKED, ids=[c["name"] for c in PACKED])
def test_packed_shapes_match_reference(case, words, fused, tbw):
    """Every shape of the 16/32/64-label kernels (one thread per 16 labels
    with the winner-take-all in the T->B pass or in a pass of its own, the
    fused two-pass form of the 16-label pyramid levels, or a chain spread
    over several threads) gives the reference's results."""
    import pyrsgm_gb300 as pg
    mine = _run_shape(case, words, fused, tbw)
    assert pg.fused_stalls() == 0
    if _oracle.ref_available():
        other = _runners.run_ref(case)
    else:
        other = _runners.run_oracle(case, _runners.device_lut(case))
    bad = _runners.compare(mine, other)
    assert not bad, bad


# Widths that are not a multiple of 4 and single-scale ranges that start
# off a 4-pixel boundary: the horizontal pass then mixes whole-run and
# per-step copies of the label bases and image bytes.
ODD_PACKED = [
    cases._lvl("lvl_bt_refine_w157_adaptive", 157, 61, 16, cases.BT, True, bs=5, adaptive=True, seed=11),
    cases._lvl("lvl_census_refine_w93_adaptive", 93, 47, 16, cases.CENSUS, True, adaptive=True,
               p2p=cases.P2_SMOKE, seed=12),
    cases._lvl("lvl_census_refine_d32_w131", 131, 40, 32, cases.CENSUS, True, seed=13),
    cases._ss("ss_bt_d16_w101_minD3_adaptive", 101, 40, 16, cases.BT, minD=3, adaptive=True, seed=14),
    cases._ss("ss_census_d64_w199_minDneg", 199, 36, 64, cases.CENSUS, minD=-5, adaptive=True,
              p2p=cases.P2_SMOKE, seed=15),
]


@pytest.mark.parametrize("words,fused,tbw", SHAPES, ids=SHAPE_IDS)
@pytest.mark.parametrize("case", ODD_PACKED, ids=[c["name"] for c in ODD_PACKED])
def test_packed_shapes_odd_widths_match_reference(case, words, fused, tbw):
    mine = _run_shape(case, words, fused, tbw)
    if _oracle.ref_available():
        other = _runners.run_ref(case)
    else:
        other = _runners.run_oracle(case, _runners.device_lut(case))
    bad = _runners.compare(mine, other)
    assert not bad, bad


def test_full_size_batched_pairs_match_reference_kernels():
    """The benchmark workload at full size -- 1920x1080, D=256,
    pyramid_levels=3, adaptive P2, 3x3 median, all three outputs -- for two
    Census and two BT pairs run together through the batch engine (so the
    level launches take the many-row kernel shapes), against the
    reference's kernels on its StereoMatcher schedule, pair by pair."""
    import torch
    import pyrsgm_gb300 as pg
    from pyrsgm_gb300 import synth
    if not _oracle.ref_available():
        pytest.skip("reference kernels not built (oracle/_ref)")
    w, h = 1920, 1080

    def params(cost):
        return dict(num_disparities=256, pyramid_levels=3, cost_mode=cost,
                    p1=8 if cost == cases.CENSUS else 300, p2=32 if cost == cases.CENSUS else 2400,
                    adaptive_p2=True, median_filter=True, lr_check=True, uniqueness_ratio=10,
                    pyramid_coarse_disparities=128)

    costs = [cases.CENSUS, cases.BT, cases.CENSUS, cases.BT]
    pairs = [synth.make_pair(w, h, 255, 16, 3000 + i)[:2] for i in range(len(costs))]
    items, outs = [], []
    for (left, right), c in zip(pairs, costs):
        o = dict(disp16=torch.zeros((h, w), dtype=torch.int16, device="cuda"),
                 disp32=torch.zeros((h, w), dtype=torch.float32, device="cuda"),
                 conf=torch.zeros((h, w), dtype=torch.float32, device="cuda"))
        items.append(dict(left=torch.from_numpy(left).cuda(), right=torch.from_numpy(right).cuda(),
                          params=pg.Params(**params(c)), **o))
        outs.append(o)
    eng = pg.BatchEngine(16 << 30)
    st = torch.cuda.Stream()
    torch.cuda.synchronize()
    eng.run(items, use_graph=True, stream=st)
    torch.cuda.synchronize()
    for i, ((left, right), c) in enumerate(zip(pairs, costs)):
        r16 = torch.zeros((h, w), dtype=torch.int16, device="cuda")
        r32 = torch.zeros((h, w), dtype=torch.float32, device="cuda")
        rcf = torch.zeros((h, w), dtype=torch.float32, device="cuda")
        _runners._ref_matcher(dict(w=w, h=h, params=params(c)), items[i]["left"], items[i]["right"], r16, r32, rcf)
        np.testing.assert_array_equal(outs[i]["disp16"].cpu().numpy(), r16.cpu().numpy(), err_msg=f"pair {i}")
        np.testing.assert_allclose(outs[i]["disp32"].cpu().numpy(), r32.cpu().numpy(), rtol=0, atol=1e-6)
        np.testing.assert_allclose(outs[i]["conf"].cpu().numpy(), rcf.cpu().numpy(), rtol=0, atol=1e-6)
        assert int((outs[i]["disp16"] > 0).sum()) > w * h // 2
    eng.close()
