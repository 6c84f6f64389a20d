"""Bindings of the test oracles (oracle/): the CPU restatement and the
reference-kernel harness.  Test infrastructure only.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_SO = os.path.join(ROOT, "oracle", "_build", "libsgm_oracle.so")
HARNESS_SO = os.path.join(ROOT, "oracle", "_build", "libref_harness.so")
SGM_FATBIN = os.path.join(ROOT, "oracle", "_ref", "sgm_kernels.fatbin")
PYR_FATBIN = os.path.join(ROOT, "oracle", "_ref", "pyrdown.fatbin")

_vp, _sz, _i, _f = C.c_void_p, C.c_size_t, C.c_int, C.c_float


class OrcParams(C.Structure):
    _fields_ = [(n, _i) for n in (
        "num_disparities", "min_disparity", "block_size", "cost_mode",
        "p1", "p2", "uniqueness_ratio", "disp12_max_diff",
        "lr_check", "median_filter", "num_paths", "pre_filter_cap",
        "pyramid_levels", "pyramid_coarse_disparities", "pyramid_max_disparity")] + [
        ("pyramid_min_confidence", _f), ("adaptive_p2", _i),
        ("p2_alpha", _f), ("p2_beta", _f), ("p2_lower_mult", _f), ("p2_upper_mult", _f)]


class OrcLevelInfo(C.Structure):
    _fields_ = [(n, _i) for n in ("level", "width", "height", "num_labels", "max_disparity", "block_size",
                                  "refine")]


_orc = None


def oracle() -> C.CDLL:
    global _orc
    if _orc is None:
        if not os.path.exists(ORACLE_SO):
            import importlib.util
            spec = importlib.util.spec_from_file_location("build_oracle", os.path.join(ROOT, "oracle", "build_oracle.py"))
            m = importlib.util.module_from_spec(spec)
            spec.loader.exec_module(m)
            m.build_oracle()
        h = C.CDLL(ORACLE_SO)
        h.orc_create_workspace.restype = _vp
        h.orc_destroy_workspace.argtypes = [_vp]
        h.orc_ws_cost.restype = _vp
        h.orc_ws_cost.argtypes = [_vp]
        h.orc_ws_acc.restype = _vp
        h.orc_ws_acc.argtypes = [_vp]
        h.orc_pyrdown_u8.argtypes = [_vp, _sz, _i, _i, _vp, _sz, _i, _i]
        h.orc_compute_single_scale.argtypes = [_vp, _vp, _vp, _vp, _vp, _vp, _sz, _sz, _sz, _sz, _sz] + \
            [_i] * 14 + [_f] * 4 + [_vp]
        h.orc_compute_level.argtypes = [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp] + [_sz] * 7 + [_i] * 17 + \
            [_f, _i, _f, _f, _f, _f, _vp]
        h.orc_default_params.argtypes = [C.POINTER(OrcParams)]
        h.orc_validate_params.argtypes = [C.POINTER(OrcParams), C.POINTER(OrcParams)]
        h.orc_level_geometry.argtypes = [_i, _i, C.POINTER(OrcParams), C.POINTER(OrcLevelInfo)]
        h.orc_matcher_compute.argtypes = [_i, _i, C.POINTER(OrcParams), _vp, _sz, _vp, _sz, _vp, _sz, _vp, _sz,
                                          _vp, _sz, _vp]
        h.orc_p2_table_libm.argtypes = [_i, _f, _f, _f, _f, _vp]
        h.orc_set_num_threads.argtypes = [_i]
        h.orc_filter_speckles.argtypes = [_vp, _sz, _i, _i, C.c_short, _i, _i]
        _orc = h
    return _orc


def _p(a: np.ndarray | None):
    return None if a is None else a.ctypes.data


def orc_pyrdown(src: np.ndarray) -> np.ndarray:
    h, w = src.shape
    dst = np.zeros(((h + 1) // 2, (w + 1) // 2), np.uint8)
    src = np.ascontiguousarray(src)
    r = oracle().orc_pyrdown_u8(_p(src), w, w, h, _p(dst), dst.shape[1], dst.shape[1], dst.shape[0])
    assert r == 0
    return dst


def orc_speckles(img: np.ndarray, new_val: int, max_size: int, max_diff: int) -> np.ndarray:
    out = np.ascontiguousarray(img, dtype=np.int16).copy()
    h, w = out.shape
    assert oracle().orc_filter_speckles(_p(out), w * 2, w, h, new_val, max_size, max_diff) == 0
    return out


def _lut_arg(lut):
    if lut is None:
        return None, None
    arr = np.ascontiguousarray(np.asarray(lut, np.int32))
    return arr, arr.ctypes.data


def orc_single_scale(left, right, c: dict, lut=None, want=("disp16", "disp32", "conf")) -> dict:
    h, w = left.shape
    D = c["D"]
    orc = oracle()
    ws = orc.orc_create_workspace()
    out = {k: None for k in ("disp16", "disp32", "conf")}
    out["disp16"] = np.zeros((h, w), np.int16) if "disp16" in want else None
    out["disp32"] = np.zeros((h, w), np.float32) if "disp32" in want else None
    out["conf"] = np.zeros((h, w), np.float32) if "conf" in want else None
    keep, lp = _lut_arg(lut)
    a = c["p2p"]
    r = orc.orc_compute_single_scale(ws, _p(left), _p(right), _p(out["disp16"]), _p(out["disp32"]), _p(out["conf"]),
                                     w, w, w * 2, w * 4, w * 4, w, h, D, c["minD"], c["bs"], c["P1"], c["P2"],
                                     c["uniq"], c["maxdiff"], c["pfc"], c["cost"], c["post"], c["paths"],
                                     int(c["adaptive"]), a[0], a[1], a[2], a[3], lp)
    assert r == 0
    n = w * h * D
    out["cost"] = np.ctypeslib.as_array(C.cast(orc.orc_ws_cost(ws), C.POINTER(C.c_int16)), (n,)).copy().reshape(h, w, D)
    out["acc"] = np.ctypeslib.as_array(C.cast(orc.orc_ws_acc(ws), C.POINTER(C.c_int16)), (n,)).copy().reshape(h, w, D)
    orc.orc_destroy_workspace(ws)
    return out


def orc_level(left, right, parent_disp, parent_conf, c: dict, lut=None, want=("disp16", "disp32", "conf")) -> dict:
    h, w = left.shape
    D = c["D"]
    orc = oracle()
    ws = orc.orc_create_workspace()
    out = {}
    out["disp16"] = np.zeros((h, w), np.int16) if "disp16" in want else None
    out["disp32"] = np.zeros((h, w), np.float32) if "disp32" in want else None
    out["conf"] = np.zeros((h, w), np.float32) if "conf" in want else None
    keep, lp = _lut_arg(lut)
    a = c["p2p"]
    ph, pw = parent_disp.shape if parent_disp is not None else (0, 0)
    r = orc.orc_compute_level(ws, _p(left), _p(right), _p(parent_disp), _p(parent_conf), _p(out["disp16"]),
                              _p(out["disp32"]), _p(out["conf"]), w, w, pw * 2, pw * 4, w * 2, w * 4, w * 4,
                              w, h, pw, ph, D, 0, c["maxD"], c["bs"], c["P1"], c["P2"], c["uniq"], c["maxdiff"],
                              c["pfc"], c["cost"], c["post"], c["paths"], int(c["refine"]), c["minConf"],
                              int(c["adaptive"]), a[0], a[1], a[2], a[3], lp)
    assert r == 0
    n = w * h * D
    out["cost"] = np.ctypeslib.as_array(C.cast(orc.orc_ws_cost(ws), C.POINTER(C.c_int16)), (n,)).copy().reshape(h, w, D)
    out["acc"] = np.ctypeslib.as_array(C.cast(orc.orc_ws_acc(ws), C.POINTER(C.c_int16)), (n,)).copy().reshape(h, w, D)
    orc.orc_destroy_workspace(ws)
    return out


def orc_params(**kw) -> OrcParams:
    p = OrcParams()
    oracle().orc_default_params(C.byref(p))
    for k, v in kw.items():
        setattr(p, k, int(v) if isinstance(v, bool) else v)
    return p


def orc_validate(**kw):
    p = orc_params(**kw)
    out = OrcParams()
    r = oracle().orc_validate_params(C.byref(p), C.byref(out))
    return None if r != 0 else {n: getattr(out, n) for n, _ in OrcParams._fields_}


def orc_geometry(w, h, **kw):
    p = orc_params(**kw)
    v = OrcParams()
    assert oracle().orc_validate_params(C.byref(p), C.byref(v)) == 0
    info = (OrcLevelInfo * 5)()
    n = oracle().orc_level_geometry(w, h, C.byref(v), info)
    return [{f: getattr(info[i], f) for f, _ in OrcLevelInfo._fields_} for i in range(n)]


def orc_matcher(left, right, lut=None, want=("disp16", "disp32", "conf"), **kw) -> dict:
    h, w = left.shape
    p = orc_params(**kw)
    out = {}
    out["disp16"] = np.zeros((h, w), np.int16) if "disp16" in want else None
    out["disp32"] = np.zeros((h, w), np.float32) if "disp32" in want else None
    out["conf"] = np.zeros((h, w), np.float32) if "conf" in want else None
    keep, lp = _lut_arg(lut)
    r = oracle().orc_matcher_compute(w, h, C.byref(p), _p(left), w, _p(right), w, _p(out["disp16"]), w * 2,
                                     _p(out["disp32"]), w * 4, _p(out["conf"]), w * 4, lp)
    assert r == 0
    return out


def p2_table_libm(P2, alpha, beta, lower, upper) -> np.ndarray:
    lut = np.zeros(256, np.int32)
    oracle().orc_p2_table_libm(P2, alpha, beta, lower, upper, lut.ctypes.data)
    return lut


# ---------------------------------------------------------------------------
# Reference kernels (GPU): oracle/_build/libref_harness.so + oracle/_ref/*.fatbin
# ---------------------------------------------------------------------------
_ref = None


def ref_available() -> bool:
    return os.path.exists(HARNESS_SO) and os.path.exists(SGM_FATBIN) and os.path.exists(PYR_FATBIN)


def ref() -> C.CDLL:
    global _ref
    if _ref is None:
        h = C.CDLL(HARNESS_SO)
        h.ref_init.argtypes = [C.c_char_p, C.c_char_p]
        h.ref_last_error.restype = C.c_char_p
        h.ref_create_workspace.restype = _vp
        h.ref_destroy_workspace.argtypes = [_vp]
        h.ref_workspace_reserve.argtypes = [_vp, _i, _i, _i]
        h.ref_copy_volumes.argtypes = [_vp, _vp, _vp, _vp]
        h.ref_pyrdown_u8.argtypes = [_vp, _sz, _i, _i, _vp, _sz, _i, _i, _vp]
        h.ref_compute_level.argtypes = [_vp] * 8 + [_sz] * 7 + [_i] * 17 + [_f, _i, _f, _f, _f, _f, _vp]
        h.ref_compute_single_scale.argtypes = [_vp] * 6 + [_sz] * 5 + [_i] * 14 + [_f] * 4 + [_vp]
        if h.ref_init(SGM_FATBIN.encode(), PYR_FATBIN.encode()) != 0:
            raise RuntimeError("reference harness init failed: " + h.ref_last_error().decode())
        _ref = h
    return _ref
