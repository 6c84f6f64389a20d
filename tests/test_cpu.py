"""CPU tests (no GPU): the oracle against the reference's known answers and
the golden fixtures made by the reference kernels, the host-side logic of
the library (parameter validation, level geometry, argument checks) and its
exported C ABI.  Reference tests mirrored: tests/matcher_test.cpp:42-126,
266-281."""
from __future__ import annotations

import ctypes as C
import os
import re

import numpy as np
import pytest

import pyrsgm_gb300 as pg
from pyrsgm_gb300 import _native
from tests import _oracle, _runners, cases

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden", "ref_golden.npz")


# --- pyrDown known answer (tests/matcher_test.cpp:74-126) -------------------
def _reflect101(i, n):
    i = np.abs(i)
    return np.where(i >= n, 2 * n - 2 - i, i)


def pyrdown_numpy(src: np.ndarray) -> np.ndarray:
    """The reference test's pyrDownRef (tests/matcher_test.cpp:81-101)."""
    h, w = src.shape
    dh, dw = (h + 1) // 2, (w + 1) // 2
    k = np.array([1, 4, 6, 4, 1], np.int64)
    ys = _reflect101(2 * np.arange(dh)[:, None] + np.arange(5)[None, :] - 2, h)
    xs = _reflect101(2 * np.arange(dw)[:, None] + np.arange(5)[None, :] - 2, w)
    s = src.astype(np.int64)
    acc = np.zeros((dh, dw), np.int64)
    for ky in range(5):
        for kx in range(5):
            acc += k[ky] * k[kx] * s[ys[:, ky]][:, xs[:, kx]]
    return ((acc + 128) >> 8).astype(np.uint8)


@pytest.mark.parametrize("w,h", cases.PYRDOWN)
def test_oracle_pyrdown_known_answer(w, h):
    src = cases.pyrdown_input(w, h)
    np.testing.assert_array_equal(_oracle.orc_pyrdown(src), pyrdown_numpy(src))


# --- validateParams (tests/matcher_test.cpp:42-72) --------------------------
INVALID = [
    dict(pyramid_levels=5), dict(pyramid_levels=1, min_disparity=8), dict(pyramid_levels=1, disp12_max_diff=-1),
    dict(num_disparities=2048), dict(p1=100, p2=50), dict(adaptive_p2=True, p2_beta=0.0),
    dict(num_disparities=0), dict(uniqueness_ratio=100), dict(pre_filter_cap=0), dict(block_size=0),
    dict(pyramid_levels=2, pyramid_coarse_disparities=0), dict(pyramid_levels=-1),
]


@pytest.mark.parametrize("kw", INVALID)
def test_validate_rejects(kw):
    with pytest.raises(ValueError):
        pg.validate_params(pg.Params(**kw))
    assert _oracle.orc_validate(**kw) is None


VALID = [dict(), dict(num_disparities=100), dict(num_disparities=100, block_size=4), dict(pyramid_levels=2),
         dict(num_paths=7), dict(num_paths=0), dict(pyramid_levels=3, pyramid_coarse_disparities=1500),
         dict(pyramid_levels=1, pyramid_min_confidence=2.0), dict(block_size=1), dict(num_disparities=1017)]


@pytest.mark.parametrize("kw", VALID)
def test_validate_matches_oracle(kw):
    mine = pg.validate_params(pg.Params(**kw))
    ref = _oracle.orc_validate(**kw)
    for k, v in ref.items():
        assert getattr(mine, k) == pytest.approx(v), k


def test_validate_known_answers():
    v = pg.validate_params(pg.Params())
    assert v.num_disparities == 128 and v.block_size == 5 and v.pyramid_max_disparity == 0
    assert pg.validate_params(pg.Params(num_disparities=100)).num_disparities == 112
    assert pg.validate_params(pg.Params(num_disparities=100, block_size=4)).block_size == 5
    assert pg.validate_params(pg.Params(pyramid_levels=2)).pyramid_max_disparity == 127


# --- level geometry (tests/matcher_test.cpp:266-281) ------------------------
def test_level_geometry_known_answer():
    info = pg.level_geometry(961, 541, pg.Params(num_disparities=128, pyramid_levels=3))
    assert len(info) == 4
    l3 = info[3]
    assert (l3.width, l3.height) == (121, 68)
    assert not l3.refine and l3.num_labels == 16 and l3.max_disparity == 15
    assert info[0].refine and info[0].num_labels == 16
    assert info[2].block_size == 3 and info[1].block_size == 5


@pytest.mark.parametrize("w,h,kw", [
    (1920, 1080, dict(num_disparities=256, pyramid_levels=3)),
    (1920, 1080, dict(num_disparities=256, pyramid_levels=2)),
    (1280, 720, dict(num_disparities=128, pyramid_levels=2)),
    (640, 480, dict(num_disparities=64, pyramid_levels=0)),
    (33, 17, dict(num_disparities=64, pyramid_levels=4, pyramid_coarse_disparities=48)),
    (700, 500, dict(num_disparities=1000, pyramid_levels=1, pyramid_max_disparity=300)),
])
def test_level_geometry_matches_oracle(w, h, kw):
    mine = pg.level_geometry(w, h, pg.Params(**kw))
    ref = _oracle.orc_geometry(w, h, **kw)
    assert len(mine) == len(ref)
    for a, b in zip(mine, ref):
        assert (a.level, a.width, a.height, a.num_labels, a.max_disparity, a.block_size, int(a.refine)) == \
            (b["level"], b["width"], b["height"], b["num_labels"], b["max_disparity"], b["block_size"], b["refine"])


# --- C ABI: exports and argument checks (no device work) --------------------
def _declared_functions() -> set[str]:
    names = set()
    for hdr in sorted(os.listdir(os.path.join(ROOT, "include", "pyrsgm"))):
        text = open(os.path.join(ROOT, "include", "pyrsgm", hdr)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        names.update(re.findall(r"\b((?:pyrsgm|cuda_3sgm)_\w+)\s*\(", text))
    return names


def test_library_exports_every_declared_symbol():
    lib = C.CDLL(_native.LIB_PATH)
    declared = _declared_functions()
    assert {"pyrsgm_create_workspace", "pyrsgm_compute_level", "pyrsgm_compute_single_scale",
            "pyrsgm_pyrdown_u8", "pyrsgm_workspace_reserve", "pyrsgm_destroy_workspace"} <= declared
    missing = [n for n in sorted(declared) if not hasattr(lib, n)]
    assert not missing, missing
    assert set(_native.EXPORTS) <= declared


def test_capi_rejects_bad_arguments_without_device_work():
    lib = _native.lib()
    # pyrsgm_pyrdown_u8: wrong destination size / tiny source (src/pyrdown.cu:63-67)
    assert lib.pyrsgm_pyrdown_u8(1, 64, 64, 48, 2, 32, 31, 24, None) == -1
    assert lib.pyrsgm_pyrdown_u8(1, 64, 1, 48, 2, 32, 1, 24, None) == -1
    assert lib.pyrsgm_pyrdown_u8(None, 64, 64, 48, 2, 32, 32, 24, None) == -1
    ws = lib.pyrsgm_create_workspace()
    try:
        assert lib.pyrsgm_workspace_reserve(ws, 64, 48, 24) == -1
        assert lib.pyrsgm_workspace_reserve(ws, 64, 48, 2048) == -1
        assert lib.pyrsgm_workspace_reserve(None, 64, 48, 32) == -1

        def level(D=32, refine=0, parent=1, w=64, h=48, maxD=31, minD=0):
            return lib.pyrsgm_compute_level(ws, 1, 2, parent if refine else None, parent if refine else None,
                                            None, None, None, 64, 64, 64, 128, 128, 256, 256, w, h, 32 if refine else 0,
                                            24 if refine else 0, D, minD, maxD, 3, 8, 32, 10, 1, 63, 1, 1, 3, refine,
                                            0.05, 0, 1.0, 1.0, 1.0, 1.0, None)
        assert level(D=24) == -1            # not a multiple of 16
        assert level(D=2048) == -1          # too many labels
        assert level(D=272, refine=1) == -1  # refine > 256 labels
        assert level(refine=1, parent=None) == -1
        assert level(w=0) == -1
        assert level(maxD=-5) == -1         # maxDisparity < minDisparity after clamps
        ss = lib.pyrsgm_compute_single_scale
        assert ss(ws, None, 2, None, None, None, 64, 64, 128, 256, 256, 64, 48, 32, 0, 5, 8, 32, 10, 1, 63, 1, 1, 3,
                  0, 1.0, 1.0, 1.0, 1.0, None) == -1
        assert ss(ws, 1, 2, None, None, None, 64, 64, 128, 256, 256, 64, 48, 40, 0, 5, 8, 32, 10, 1, 63, 1, 1, 3,
                  0, 1.0, 1.0, 1.0, 1.0, None) == -1
    finally:
        lib.pyrsgm_destroy_workspace(ws)


def test_workspace_bytes_formula():
    lib = _native.lib()
    n = lib.pyrsgm_gb300_workspace_bytes(1920, 1080, 16)
    assert n >= 1920 * 1080 * (16 + 2 * 16 * 2 + 8)
    assert lib.pyrsgm_gb300_workspace_bytes(0, 10, 16) == 0


# --- the oracle pinned by the reference kernels' golden outputs -------------
def _golden():
    if not os.path.exists(GOLDEN):
        pytest.skip("golden fixtures not generated yet (tests/golden/make_golden.py on a GPU)")
    return np.load(GOLDEN)


ALL_CASES = cases.SINGLE_SCALE + cases.LEVELS + cases.MATCHER


@pytest.mark.parametrize("case", ALL_CASES, ids=[c["name"] for c in ALL_CASES])
def test_oracle_matches_reference_golden(case):
    from tests.golden.make_golden import row_hashes
    g = _golden()
    n = case["name"]
    lut = g[f"{n}/p2lut"] if f"{n}/p2lut" in g.files else None
    out = _runners.run_oracle(case, lut)
    np.testing.assert_array_equal(out["disp16"], g[f"{n}/disp16"])
    np.testing.assert_allclose(out["conf"], g[f"{n}/conf"], rtol=0, atol=1e-6)
    np.testing.assert_array_equal(row_hashes(out["disp32"]), g[f"{n}/disp32_rows"])
    if f"{n}/cost_rows" in g.files:
        x0, x1 = out["acc_cols"]
        np.testing.assert_array_equal(row_hashes(out["cost"]), g[f"{n}/cost_rows"])
        np.testing.assert_array_equal(row_hashes(out["acc"][:, x0:x1]), g[f"{n}/acc_rows"])


@pytest.mark.parametrize("w,h", cases.PYRDOWN)
def test_oracle_pyrdown_matches_reference_golden(w, h):
    g = _golden()
    np.testing.assert_array_equal(_oracle.orc_pyrdown(cases.pyrdown_input(w, h)), g[f"pyrdown_{w}x{h}"])


def test_autotune_switch_and_empty_table_without_device_work():
    import pyrsgm_gb300 as pg
    prev = pg.set_autotune(True)
    try:
        assert pg.set_autotune(True) is True
        pg.autotune_clear()
        assert pg.autotune_table() == []
    finally:
        pg.set_autotune(prev)


def test_kernel_form_switches_without_device_work():
    """The three-way T->B winner switch and the fused switch set and return
    their previous values; out-of-range modes are refused."""
    import pytest
    import pyrsgm_gb300 as pg
    from pyrsgm_gb300._native import lib
    prev = pg.set_tbw(2)
    try:
        assert pg.set_tbw(0) == 2
        assert pg.set_tbw(1) == 0
        assert lib().pyrsgm_gb300_set_tbw(3) == -1
        assert lib().pyrsgm_gb300_set_tbw(-1) == -1
        assert pg.set_tbw(1) == 1
        with pytest.raises(ValueError):
            pg.set_tbw(7)
    finally:
        pg.set_tbw(prev)
    prev_f = pg.set_fused(True)
    try:
        assert pg.set_fused(False) is True
        assert pg.set_fused(False) is False
    finally:
        pg.set_fused(prev_f)


def test_default_library_is_not_the_checked_build():
    import pyrsgm_gb300 as pg
    assert pg.is_checked() is False
    assert pg.check_report() == (0, "")


def test_new_entry_points_reject_bad_arguments_without_device_work():
    """Speckle filter, plan reservation and the autotune table check their
    arguments before any device call."""
    lib = _native.lib()
    # filter_speckles: null map, empty size, odd or short pitch, negative max_diff
    assert lib.pyrsgm_gb300_filter_speckles(None, 64, 32, 8, -16, 10, 1, None) == -1
    assert lib.pyrsgm_gb300_filter_speckles(1, 64, 0, 8, -16, 10, 1, None) == -1
    assert lib.pyrsgm_gb300_filter_speckles(1, 63, 31, 8, -16, 10, 1, None) == -1
    assert lib.pyrsgm_gb300_filter_speckles(1, 32, 32, 8, -16, 10, 1, None) == -1
    assert lib.pyrsgm_gb300_filter_speckles(1, 64, 32, 8, -16, 10, -1, None) == -1
    assert lib.pyrsgm_gb300_filter_speckles(1, 64, 32, 8, -16, 0, 1, None) == 0   # max size 0: nothing to do
    # batch reservation: null engine / params, empty size, invalid parameters
    import pyrsgm_gb300 as pg
    p = pg.Params(num_disparities=64, pyramid_levels=1)
    err = C.create_string_buffer(256)
    eng = lib.pyrsgm_gb300_batch_create(1 << 20, err, 256)
    assert eng
    try:
        assert lib.pyrsgm_gb300_batch_reserve(None, 64, 48, C.byref(p.to_c()), 1, None, err, 256) == -1
        assert lib.pyrsgm_gb300_batch_reserve(eng, 64, 48, None, 1, None, err, 256) == -1
        assert lib.pyrsgm_gb300_batch_reserve(eng, 0, 48, C.byref(p.to_c()), 1, None, err, 256) == -1
        bad = pg.Params(num_disparities=64, pyramid_levels=9)   # validateParams rejects it
        assert lib.pyrsgm_gb300_batch_reserve(eng, 64, 48, C.byref(bad.to_c()), 1, None, err, 256) == -1
        assert b"pyramid_levels" in err.value
        assert lib.pyrsgm_gb300_batch_bytes_in_use(eng) == 0
    finally:
        lib.pyrsgm_gb300_batch_destroy(eng)
    assert lib.pyrsgm_gb300_server_reserve(None, 64, 48, C.byref(p.to_c()), 1, err, 256) == -1
    # the autotune table can be sized with a null buffer
    pg.autotune_clear()
    assert lib.pyrsgm_gb300_autotune_entries(None, 0) == 0
