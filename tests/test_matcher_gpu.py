"""Behavioural known-answer tests ported from the reference's own test suite
(tests/matcher_test.cpp:128-281 and tests/pyramid_smoke.cpp:21-164): accuracy
on synthetic scenes at pyramid levels 0..4 with both costs, output subsets,
the invalid marker, and the five-level C-API refinement chain."""
from __future__ import annotations

import numpy as np
import pytest
import torch

import pyrsgm_gb300 as pg

pytestmark = pytest.mark.gpu


def make_pattern(w, h, disparity, right):
    """testutil::makePattern (tests/test_utils.h:72-83)."""
    y, x = np.mgrid[0:h, 0:w]
    sx = x + disparity if right else x
    return ((sx * 37 + y * 17 + ((sx // 7) ^ (y // 5)) * 29) & 0xFF).astype(np.uint8)


def _tex(sx, sy):
    return ((sx * 37 + sy * 17 + ((sx // 7) ^ (sy // 5)) * 29) & 0xFF).astype(np.float32)


def sample_texture(xf, y):
    """testutil::sampleTexture (tests/test_utils.h:89-98), float32 arithmetic."""
    x0 = np.floor(xf).astype(np.int64)
    f = (xf - x0.astype(np.float32)).astype(np.float32)
    v = (np.float32(1.0) - f) * _tex(x0, y) + f * _tex(x0 + 1, y)
    return (v + np.float32(0.5)).astype(np.uint8)


def constant_scene(w, h, d):
    return make_pattern(w, h, d, False), make_pattern(w, h, d, True), np.full((h, w), float(d), np.float32)


def slanted_scene(w, h, d0, slope):
    y, x = np.mgrid[0:h, 0:w]
    xf = x.astype(np.float32)
    left = sample_texture(xf, y)
    right = sample_texture(((xf + np.float32(d0)) / np.float32(1.0 - slope)).astype(np.float32), y)
    return left, right, (d0 + slope * xf).astype(np.float32)


def stats(disp32, gt, tol, margin):
    h, w = disp32.shape
    d = disp32[margin:h - margin, margin:w - margin]
    g = gt[margin:h - margin, margin:w - margin]
    valid = d > 0
    err = np.abs(d - g)[valid]
    return dict(total=d.size, valid=int(valid.sum()), good=int((err <= tol).sum()),
                mae=float(err.mean()) if err.size else 0.0)


def run(scene, params, want16=True, want32=True, want_conf=True):
    left, right, _ = scene
    h, w = left.shape
    m = pg.StereoMatcher(w, h, params)
    out = m.compute(torch.from_numpy(left).cuda(), torch.from_numpy(right).cuda(), want16, want32, want_conf)
    torch.cuda.synchronize()
    return {k: (v.cpu().numpy() if v is not None else None) for k, v in out.items()}


CONST = constant_scene(640, 480, 40)
SLANT = slanted_scene(640, 480, 12.0, 0.06)


@pytest.mark.parametrize("levels", [0, 1, 2, 3, 4])
@pytest.mark.parametrize("cost", [pg.COST_BT, pg.COST_CENSUS])
def test_matcher_accuracy(levels, cost):
    p = pg.Params(num_disparities=64, pyramid_levels=levels, cost_mode=cost,
                  p1=8 if cost == pg.COST_CENSUS else 300, p2=32 if cost == pg.COST_CENSUS else 2400)
    margin = p.num_disparities + 8
    c = run(CONST, p)
    s = stats(c["disp32"], CONST[2], 1.0, margin)
    assert s["valid"] / s["total"] > 0.5, s
    assert s["good"] / s["valid"] > 0.95, s
    inv = pg.invalid_disparity16(p)
    is_inv = c["disp16"] == inv
    assert np.all(c["disp32"][is_inv] == 0.0)
    ok = ~is_inv & (c["disp32"] != 0.0)
    assert np.all(np.abs(c["disp16"][ok] / 16.0 - c["disp32"][ok]) <= 1e-6)
    assert is_inv.sum() > 0, "border pixels are invalid"
    t = run(SLANT, p)
    st = stats(t["disp32"], SLANT[2], 1.0, margin)
    assert st["good"] / st["valid"] > 0.9, st
    assert st["mae"] < 0.5, st


def test_output_subsets():
    p = pg.Params(num_disparities=64, pyramid_levels=2)
    only16 = run(CONST, p, True, False, False)
    assert (only16["disp16"] != pg.invalid_disparity16(p)).sum() > 0
    only32 = run(CONST, p, False, True, False)
    assert (only32["disp32"] > 0).sum() > 0
    only_conf = run(CONST, p, False, False, True)
    assert (only_conf["conf"] > 0).sum() > 0


def test_level_info_and_memory():
    p = pg.Params(num_disparities=128, pyramid_levels=3)
    m = pg.StereoMatcher(961, 541, p)
    assert m.num_levels() == 4
    l3 = m.level_info(3)
    assert (l3.width, l3.height, l3.refine, l3.num_labels, l3.max_disparity) == (121, 68, False, 16, 15)
    assert m.level_info(0).refine and m.level_info(0).num_labels == 16
    assert m.level_info(2).block_size == 3 and m.level_info(1).block_size == 5
    assert m.device_memory_bytes() > 0
    with pytest.raises(IndexError):
        m.level_info(4)


def test_null_input_raises():
    m = pg.StereoMatcher(64, 48, pg.Params(num_disparities=16))
    with pytest.raises(ValueError):
        m.compute_into(torch.empty(0), torch.empty(0), torch.empty((48, 64), dtype=torch.int16, device="cuda"))


# --- C-API chain, tests/pyramid_smoke.cpp:21-164 ----------------------------
def _level(ws, left, right, parent, labels, max_disp, refine, cost=pg.COST_BT, paths=3):
    h, w = left.shape
    d16 = torch.zeros((h, w), dtype=torch.int16, device="cuda")
    d32 = torch.zeros((h, w), dtype=torch.float32, device="cuda")
    cf = torch.zeros((h, w), dtype=torch.float32, device="cuda")
    r = pg.compute_level(ws, left, right, parent[0] if parent else None, parent[1] if parent else None, d16, d32, cf,
                         num_disparities=labels, min_disparity=0, max_disparity=max_disp, block_size=3, p1=24, p2=96,
                         uniqueness=0, disp12_max_diff=1, pre_filter_cap=63, cost_mode=cost,
                         post_flags=pg.POST_LRCHECK, num_paths=paths, refine=refine, min_confidence=0.0,
                         adaptive_p2=True, p2_alpha=2.0, p2_beta=14.0, p2_lower=0.75, p2_upper=2.0)
    assert r == 0
    torch.cuda.synchronize()
    return d16, d32, cf


def _has_expected(d32, expected, tol):
    d = d32.cpu().numpy()
    v = d > 0
    return v.sum() > 0 and (np.abs(d[v] - expected) <= tol).sum() >= v.sum() // 2


def test_pyramid_smoke_chain():
    sizes = [(40, 16, 2), (80, 32, 4), (160, 64, 8), (320, 128, 16), (640, 256, 32)]
    imgs = [(torch.from_numpy(make_pattern(w, h, d, False)).cuda(), torch.from_numpy(make_pattern(w, h, d, True)).cuda())
            for w, h, d in sizes]
    wss = [pg.Workspace() for _ in sizes]
    d16, d32, cf = _level(wss[0], *imgs[0], None, 32, 31, False)
    assert _has_expected(d32, 2.0, 1.5)
    for i, (max_disp, tol) in enumerate(((63, 1.5), (127, 1.5), (255, 1.5), (511, 2.0)), start=1):
        d16, d32, cf = _level(wss[i], *imgs[i], (d16, cf), 16, max_disp, True)
        assert _has_expected(d32, float(sizes[i][2]), tol), f"level {i}"
    # large base jumps between adjacent parents (both bounds of same +- 1), 3 and 1 paths
    pd = torch.from_numpy(np.where(np.arange(160) % 2 == 1, 30, 2).astype(np.int16)[None, :].repeat(64, 0) * 16).cuda()
    pc = torch.ones((64, 160), dtype=torch.float32, device="cuda")
    _level(wss[3], *imgs[3], (pd, pc), 16, 255, True)
    _level(wss[3], *imgs[3], (pd, pc), 16, 255, True, pg.COST_BT, 1)
    # Census coarse search, two paths
    d16, d32, cf = _level(wss[2], *imgs[2], None, 128, 127, False, pg.COST_CENSUS, 2)
    assert _has_expected(d32, 8.0, 2.0)


@pytest.mark.parametrize("cost", [pg.COST_BT, pg.COST_CENSUS])
def test_single_scale_entry(cost):
    L = torch.from_numpy(make_pattern(640, 256, 32, False)).cuda()
    R = torch.from_numpy(make_pattern(640, 256, 32, True)).cuda()
    ws = pg.Workspace()
    d16 = torch.zeros((256, 640), dtype=torch.int16, device="cuda")
    d32 = torch.zeros((256, 640), dtype=torch.float32, device="cuda")
    cf = torch.zeros((256, 640), dtype=torch.float32, device="cuda")
    r = pg.compute_single_scale(ws, L, R, d16, d32, cf, num_disparities=64, min_disparity=0, block_size=5,
                                p1=300 if cost == pg.COST_BT else 8, p2=2400 if cost == pg.COST_BT else 32,
                                uniqueness=10, disp12_max_diff=1, pre_filter_cap=63, cost_mode=cost,
                                post_flags=pg.POST_LRCHECK | pg.POST_MEDIAN, num_paths=3, adaptive_p2=False,
                                p2_alpha=0.0, p2_beta=1.0, p2_lower=1.0, p2_upper=1.0)
    assert r == 0
    torch.cuda.synchronize()
    assert _has_expected(d32, 32.0, 1.0)


class _Tri3sgmNames:
    """The library with the pyrsgm_c.h entry points replaced by their
    Tri3SGM-engine names (pyrsgm_tri3sgm.h)."""

    def __init__(self, lib):
        self._lib = lib
        self.pyrsgm_compute_single_scale = lib.cuda_3sgm_compute_with_workspace
        self.pyrsgm_compute_level = lib.cuda_3sgm_compute_pyramid_level_with_workspace

    def __getattr__(self, name):
        return getattr(self._lib, name)


def test_tri3sgm_entry_points_equal_the_c_api(monkeypatch):
    from pyrsgm_gb300 import _native, api
    L = torch.from_numpy(make_pattern(320, 128, 16, False)).cuda()
    R = torch.from_numpy(make_pattern(320, 128, 16, True)).cuda()

    def run():
        ws = [pg.Workspace(), pg.Workspace()]
        out = []
        d16, d32, cf = (torch.zeros((128, 320), dtype=t, device="cuda") for t in (torch.int16, torch.float32,
                                                                                   torch.float32))
        assert pg.compute_single_scale(ws[0], L, R, d16, d32, cf, num_disparities=32) == 0
        out += [d16.clone(), d32.clone(), cf.clone()]
        pl, pr = L[::2, ::2].contiguous(), R[::2, ::2].contiguous()
        p16, p32, pcf = (torch.zeros((64, 160), dtype=t, device="cuda") for t in (torch.int16, torch.float32,
                                                                                  torch.float32))
        assert pg.compute_level(ws[1], pl, pr, None, None, p16, p32, pcf, num_disparities=16, max_disparity=15) == 0
        assert pg.compute_level(ws[0], L, R, p16, pcf, d16, d32, cf, num_disparities=16, max_disparity=31,
                                refine=True) == 0
        out += [p16, d16, d32, cf]
        torch.cuda.synchronize()
        for w in ws:
            w.close()
        return [t.cpu().numpy() for t in out]

    want = run()
    monkeypatch.setattr(api, "lib", lambda: _Tri3sgmNames(_native.lib()))
    got = run()
    for a, b in zip(got, want):
        np.testing.assert_array_equal(a, b)
