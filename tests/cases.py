"""Parity cases shared by the golden-fixture generator and the parity tests.

Every case is a small, seeded invocation of one reference entry point
(pyrsgm_compute_single_scale, pyrsgm_compute_level, pyrsgm_pyrdown_u8 or
StereoMatcher::compute).  Inputs come from pyrsgm_gb300.synth; refine levels
get a synthetic parent (disparity from the ground truth at half resolution
with noise, ~10% invalid pixels, random confidence, and a band of
alternating far-apart parents that exercises both bounds of same +- 1).
"""
from __future__ import annotations

import numpy as np

from pyrsgm_gb300 import synth

BT, CENSUS = 0, 1
LRC, MED = 1, 2

# adaptive P2 parameters used by the reference's own smoke test
# (tests/pyramid_smoke.cpp:186) and its defaults (include/pyrsgm/pyrsgm.h:78-81)
P2_SMOKE = (2.0, 14.0, 0.75, 2.0)
P2_DEFAULT = (3.041, 16.137, 0.601, 1.77)


def _ss(name, w, h, D, cost, *, minD=0, bs=5, P1=None, P2=None, uniq=10, maxdiff=1, pfc=63,
        post=LRC, paths=3, adaptive=False, p2p=P2_DEFAULT, seed=1):
    P1 = P1 if P1 is not None else (200 if cost == BT else 8)
    P2 = P2 if P2 is not None else (800 if cost == BT else 32)
    return dict(kind="ss", name=name, w=w, h=h, D=D, minD=minD, bs=bs, P1=P1, P2=P2, uniq=uniq,
                maxdiff=maxdiff, pfc=pfc, cost=cost, post=post, paths=paths, adaptive=adaptive,
                p2p=p2p, seed=seed)


def _lvl(name, w, h, D, cost, refine, *, maxD=None, bs=3, P1=None, P2=None, uniq=10, maxdiff=1, pfc=63,
         post=LRC, paths=3, minConf=0.05, adaptive=False, p2p=P2_DEFAULT, seed=2):
    P1 = P1 if P1 is not None else (300 if cost == BT else 8)
    P2 = P2 if P2 is not None else (2400 if cost == BT else 32)
    if maxD is None:
        maxD = (D - 1) if not refine else min(4 * D, w - 1)
    return dict(kind="level", name=name, w=w, h=h, D=D, cost=cost, refine=refine, maxD=maxD, bs=bs, P1=P1,
                P2=P2, uniq=uniq, maxdiff=maxdiff, pfc=pfc, post=post, paths=paths, minConf=minConf,
                adaptive=adaptive, p2p=p2p, seed=seed)


def _mat(name, w, h, *, seed=3, **params):
    return dict(kind="matcher", name=name, w=w, h=h, params=params, seed=seed)


SINGLE_SCALE = [
    _ss("ss_bt_d64_p3", 160, 96, 64, BT, post=LRC),
    _ss("ss_census_d64_p3_med", 160, 96, 64, CENSUS, post=LRC | MED),
    _ss("ss_bt_d32_p2", 128, 64, 32, BT, paths=2),
    _ss("ss_census_d32_p1", 128, 64, 32, CENSUS, paths=1),
    _ss("ss_bt_d48_adaptive", 144, 80, 48, BT, adaptive=True, post=LRC | MED, seed=5),
    _ss("ss_census_d16_minD4", 96, 64, 16, CENSUS, minD=4, maxdiff=0),
    _ss("ss_bt_d32_minDneg", 112, 64, 32, BT, minD=-6, uniq=0),
    _ss("ss_census_d96_adaptive", 192, 80, 96, CENSUS, adaptive=True, p2p=P2_SMOKE),
    _ss("ss_bt_d16_bs7_noLR", 80, 48, 16, BT, bs=7, post=MED, uniq=25),
    _ss("ss_bt_d128_p3", 256, 64, 128, BT, post=LRC | MED, seed=9),
]

LEVELS = [
    _lvl("lvl_census_coarse_d32", 120, 68, 32, CENSUS, False),
    _lvl("lvl_bt_coarse_d64", 160, 90, 64, BT, False, bs=5),
    _lvl("lvl_census_coarse_d64_p2", 160, 90, 64, CENSUS, False, paths=2),
    _lvl("lvl_bt_coarse_d32_p1_adaptive", 120, 68, 32, BT, False, paths=1, adaptive=True, p2p=P2_SMOKE),
    _lvl("lvl_census_refine", 160, 96, 16, CENSUS, True),
    _lvl("lvl_bt_refine_bs3", 160, 96, 16, BT, True),
    _lvl("lvl_bt_refine_bs5_adaptive", 160, 96, 16, BT, True, bs=5, adaptive=True),
    _lvl("lvl_census_refine_p1", 160, 96, 16, CENSUS, True, paths=1, post=LRC | MED),
    _lvl("lvl_census_refine_p2_minconf", 160, 96, 16, CENSUS, True, paths=2, minConf=0.3),
    _lvl("lvl_census_refine_d32", 128, 80, 32, CENSUS, True),
    _lvl("lvl_bt_coarse_d48_med", 144, 80, 48, BT, False, post=LRC | MED, uniq=0),
    _lvl("lvl_census_refine_d64", 160, 64, 64, CENSUS, True, maxD=120),
]

MATCHER = [
    _mat("m_bt_L0", 160, 96, num_disparities=48, pyramid_levels=0, cost_mode=BT, p1=300, p2=2400),
    _mat("m_census_L1", 160, 96, num_disparities=64, pyramid_levels=1, cost_mode=CENSUS, p1=8, p2=32),
    _mat("m_census_L2_adaptive", 200, 120, num_disparities=96, pyramid_levels=2, cost_mode=CENSUS, p1=8, p2=32,
         adaptive_p2=True),
    _mat("m_bt_L3", 240, 136, num_disparities=128, pyramid_levels=3, cost_mode=BT, p1=300, p2=2400,
         adaptive_p2=True),
    _mat("m_census_L4_p2", 256, 160, num_disparities=128, pyramid_levels=4, cost_mode=CENSUS, p1=8, p2=32,
         num_paths=2),
    _mat("m_bt_L2_nomed", 180, 100, num_disparities=64, pyramid_levels=2, cost_mode=BT, median_filter=False,
         lr_check=False),
]

PYRDOWN = [(64, 48), (97, 33), (64, 33), (97, 48), (2, 2), (3, 5), (161, 97)]


def pair_for(case: dict) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    dmax = max(4, min(case.get("D", 64) - 1 + max(case.get("minD", 0), 0), case["w"] // 3))
    if case["kind"] == "matcher":
        dmax = max(4, min(case["params"].get("num_disparities", 128) - 1, case["w"] // 3))
    return synth.make_pair(case["w"], case["h"], dmax, 5, 7000 + case["seed"] * 31 + case["w"])


def parent_for(case: dict, truth: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """Synthetic parent level (half resolution) for a refine case."""
    rng = np.random.default_rng(case["seed"] * 977 + 13)
    w, h = case["w"], case["h"]
    pw, ph = (w + 1) // 2, (h + 1) // 2
    t = truth[::2, ::2][:ph, :pw] / 2.0
    raw = np.rint((t + rng.normal(0, 0.6, t.shape)) * 16).astype(np.int32)
    raw = np.clip(raw, 0, 16 * (pw - 1))
    inv = rng.random(t.shape) < 0.1
    raw[inv] = -16
    # alternating bases far apart in a band of rows
    band = slice(ph // 3, ph // 3 + 3)
    alt = np.where(np.arange(pw) % 2 == 1, 30, 2) * 16
    raw[band, :] = np.minimum(alt[None, :], 16 * (pw - 1))
    conf = rng.random(t.shape).astype(np.float32)
    conf[band, :] = 1.0
    return raw.astype(np.int16), conf


def pyrdown_input(w: int, h: int) -> np.ndarray:
    """The reference test's pyrDown pattern (tests/matcher_test.cpp:107-110)."""
    y, x = np.mgrid[0:h, 0:w]
    return ((x * 13 + y * 29 + (x * y) // 7) & 0xFF).astype(np.uint8)
