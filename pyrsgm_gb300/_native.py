"""ctypes bindings of libpyrsgm_gb300.so (the C ABI in include/pyrsgm/).

The library is built in-tree by pyrsgm_gb300.build; importing this module
never falls back to anything else: a missing library raises.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
# PYRSGM_GB300_CHECKED=1 loads the checked build (pyrsgm_gb300.build.build(checked=True))
CHECKED = os.environ.get("PYRSGM_GB300_CHECKED", "0") not in ("", "0")
LIB_PATH = os.path.join(_HERE, "libpyrsgm_gb300_checked.so" if CHECKED else "libpyrsgm_gb300.so")

_vp, _u8p, _i16p, _f32p = C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p
_sz, _i, _f = C.c_size_t, C.c_int, C.c_float


class Params(C.Structure):
    """pyrsgm_gb300_params: pyrsgm::Params as a C struct."""
    _fields_ = [(n, _i) for n in (
        "num_disparities", "min_disparity", "block_size", "cost_mode",
        "p1", "p2", "uniqueness_ratio", "disp12_max_diff",
        "lr_check", "median_filter", "num_paths", "pre_filter_cap",
        "pyramid_levels", "pyramid_coarse_disparities", "pyramid_max_disparity")] + [
        ("pyramid_min_confidence", _f), ("adaptive_p2", _i),
        ("p2_alpha", _f), ("p2_beta", _f), ("p2_lower_mult", _f), ("p2_upper_mult", _f)]

    def as_dict(self) -> dict:
        return {n: getattr(self, n) for n, _ in self._fields_}


class Pair(C.Structure):
    """pyrsgm_gb300_pair: one stereo pair of a batch."""
    _fields_ = [("d_left", _vp), ("left_pitch", _sz), ("d_right", _vp), ("right_pitch", _sz),
                ("d_disp16", _vp), ("disp16_pitch", _sz), ("d_disp32", _vp), ("disp32_pitch", _sz),
                ("d_conf", _vp), ("conf_pitch", _sz), ("width", _i), ("height", _i), ("params", Params)]


class TuneEntry(C.Structure):
    """pyrsgm_gb300_tune_entry (include/pyrsgm/pyrsgm_gb300.h)."""
    _fields_ = [("num_labels", C.c_int), ("pyramid", C.c_int), ("rows", C.c_int), ("width", C.c_int),
                ("words", C.c_int), ("ms_wide", C.c_float), ("ms_spread", C.c_float)]


class Metrics(C.Structure):
    """pyrsgm_gb300_metrics: disparity metrics against ground truth."""
    _fields_ = [("evaluated", _i), ("valid", _i)] + [(n, C.c_double) for n in (
        "avg_err", "rms_err", "bad05", "bad1", "bad2", "bad4", "density", "invalid", "bad1_all", "bad2_all")]

    def as_dict(self) -> dict:
        return {n: getattr(self, n) for n, _ in self._fields_}


class Request(C.Structure):
    """pyrsgm_gb300_request: one served pair (host buffers, pitch = width)."""
    _fields_ = [("h_left", _vp), ("h_right", _vp), ("h_disp16", _vp), ("h_disp32", _vp), ("h_conf", _vp),
                ("width", _i), ("height", _i), ("params", Params)]


# name -> (restype, argtypes)
_SIGS = {
    "pyrsgm_create_workspace": (_vp, []),
    "pyrsgm_destroy_workspace": (None, [_vp]),
    "pyrsgm_workspace_reserve": (_i, [_vp, _i, _i, _i]),
    "pyrsgm_compute_single_scale": (_i, [_vp, _u8p, _u8p, _i16p, _f32p, _f32p, _sz, _sz, _sz, _sz, _sz,
                                         _i, _i, _i, _i, _i, _i, _i, _i, _i, _i, _i, _i, _i, _i,
                                         _f, _f, _f, _f, _vp]),
    "pyrsgm_compute_level": (_i, [_vp, _u8p, _u8p, _i16p, _f32p, _i16p, _f32p, _f32p,
                                  _sz, _sz, _sz, _sz, _sz, _sz, _sz,
                                  _i, _i, _i, _i, _i, _i, _i, _i, _i, _i, _i, _i, _i, _i, _i, _i, _i,
                                  _f, _i, _f, _f, _f, _f, _vp]),
    "pyrsgm_pyrdown_u8": (_i, [_u8p, _sz, _i, _i, _u8p, _sz, _i, _i, _vp]),
    "pyrsgm_gb300_compute_level_noalloc": (_i, [_u8p, _u8p, _i16p, _f32p, _i16p, _f32p, _f32p,
                                                _sz, _sz, _sz, _sz, _sz, _sz, _sz,
                                                _i, _i, _i, _i, _i, _i, _i, _i, _i, _i, _i, _i, _i, _i, _i, _i,
                                                _i, _f, _i, _f, _f, _f, _f, _vp]),
    "pyrsgm_gb300_workspace_set_debug": (_i, [_vp, _i]),
    "pyrsgm_gb300_workspace_volumes": (_i, [_vp, C.POINTER(_vp), C.POINTER(_vp), C.POINTER(_i),
                                            C.POINTER(_i), C.POINTER(_i)]),
    "pyrsgm_gb300_workspace_copy_volumes": (_i, [_vp, _i16p, _i16p, _vp]),
    "pyrsgm_gb300_workspace_bytes": (_sz, [_i, _i, _i]),
    "pyrsgm_gb300_p2_table": (_i, [_vp, _i, _f, _f, _f, _f, _vp]),
    "pyrsgm_gb300_default_params": (None, [C.POINTER(Params)]),
    "pyrsgm_gb300_validate_params": (_i, [C.POINTER(Params), C.POINTER(Params), C.c_char_p, _sz]),
    "pyrsgm_gb300_matcher_create": (_vp, [_i, _i, C.POINTER(Params), C.c_char_p, _sz]),
    "pyrsgm_gb300_matcher_destroy": (None, [_vp]),
    "pyrsgm_gb300_matcher_compute": (_i, [_vp, _u8p, _sz, _u8p, _sz, _i16p, _sz, _f32p, _sz, _f32p, _sz,
                                          _vp, C.c_char_p, _sz]),
    "pyrsgm_gb300_matcher_level_info": (_i, [_vp, _i, C.POINTER(_i)]),
    "pyrsgm_gb300_matcher_num_levels": (_i, [_vp]),
    "pyrsgm_gb300_level_geometry": (_i, [_i, _i, C.POINTER(Params), C.POINTER(_i), C.c_char_p, _sz]),
    "pyrsgm_gb300_matcher_device_bytes": (_sz, [_vp]),
    "pyrsgm_gb300_batch_create": (_vp, [_sz, C.c_char_p, _sz]),
    "pyrsgm_gb300_batch_destroy": (None, [_vp]),
    "pyrsgm_gb300_batch_run": (_i, [_vp, C.POINTER(Pair), _i, _i, _vp, C.c_char_p, _sz]),
    "pyrsgm_gb300_batch_bytes_in_use": (_sz, [_vp]),
    "pyrsgm_gb300_batch_reserve": (_i, [_vp, _i, _i, C.POINTER(Params), _i, _vp, C.c_char_p, _sz]),
    "pyrsgm_gb300_pair_bytes": (_sz, [_i, _i, C.POINTER(Params)]),
    "pyrsgm_gb300_server_create": (_vp, [_sz, _i, _i, _i, C.c_char_p, _sz]),
    "pyrsgm_gb300_server_destroy": (None, [_vp]),
    "pyrsgm_gb300_server_submit": (C.c_longlong, [_vp, C.POINTER(Request), C.c_char_p, _sz]),
    "pyrsgm_gb300_server_wait": (_i, [_vp, C.c_longlong, C.c_double, C.c_char_p, _sz]),
    "pyrsgm_gb300_server_drain": (_i, [_vp, C.c_double]),
    "pyrsgm_gb300_server_stats": (_i, [_vp, C.POINTER(C.c_double)]),
    "pyrsgm_gb300_server_reset_stats": (None, [_vp]),
    "pyrsgm_gb300_server_timeline": (_i, [_vp, C.POINTER(C.c_double)]),
    "pyrsgm_gb300_server_inject_failure": (_i, [_vp, _i]),
    "pyrsgm_gb300_server_register": (_i, [_vp, _vp, _sz, C.c_char_p, _sz]),
    "pyrsgm_gb300_server_unregister": (_i, [_vp, _vp]),
    "pyrsgm_gb300_server_reserve": (_i, [_vp, _i, _i, C.POINTER(Params), _i, C.c_char_p, _sz]),
    "pyrsgm_gb300_version": (C.c_char_p, []),
    "pyrsgm_gb300_launch_count": (C.c_ulonglong, []),
    "pyrsgm_gb300_checked": (_i, []),
    "pyrsgm_gb300_check_report": (_i, [C.c_char_p, _sz]),
    "pyrsgm_gb300_set_packed_words": (_i, [_i]),
    "pyrsgm_gb300_set_autotune": (_i, [_i]),
    "pyrsgm_gb300_set_fused": (_i, [_i]),
    "pyrsgm_gb300_set_tbw": (_i, [_i]),
    "pyrsgm_gb300_fused_stalls": (C.c_uint, [_i]),
    "pyrsgm_gb300_autotune_entries": (_i, [_vp, _i]),
    "pyrsgm_gb300_autotune_clear": (None, []),
    "pyrsgm_gb300_read_pfm": (_i, [C.c_char_p, _vp, _sz, C.POINTER(_i), C.POINTER(_i), C.c_char_p, _sz]),
    "pyrsgm_gb300_write_pfm": (_i, [C.c_char_p, _vp, _sz, _i, _i, C.c_char_p, _sz]),
    "pyrsgm_gb300_read_pgm": (_i, [C.c_char_p, _vp, _sz, C.POINTER(_i), C.POINTER(_i), C.c_char_p, _sz]),
    "pyrsgm_gb300_write_pgm": (_i, [C.c_char_p, _vp, _sz, _i, _i, C.c_char_p, _sz]),
    "pyrsgm_gb300_read_ndisp": (_i, [C.c_char_p]),
    "pyrsgm_gb300_filter_speckles": (_i, [_vp, _sz, _i, _i, C.c_short, _i, _i, _vp]),
    "pyrsgm_gb300_evaluate": (_i, [_vp, _sz, _vp, _sz, _vp, _sz, _i, _i, _f, C.POINTER(Metrics)]),
    "pyrsgm_gb300_profile": (_i, [_i]),
    "pyrsgm_gb300_profile_read": (_i, [_i, C.POINTER(C.c_double), C.POINTER(C.c_longlong), C.POINTER(C.c_double)]),
}
# the Tri3SGM engine's names for the same two entry points (pyrsgm_tri3sgm.h)
_SIGS["cuda_3sgm_compute_with_workspace"] = _SIGS["pyrsgm_compute_single_scale"]
_SIGS["cuda_3sgm_compute_pyramid_level_with_workspace"] = _SIGS["pyrsgm_compute_level"]

# Entry points declared in include/pyrsgm/*.h (checked by the tests).
EXPORTS = tuple(_SIGS)

_lib = None


def lib() -> C.CDLL:
    """Load the native library (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"pyrsgm-gb300 native library missing at {LIB_PATH}; "
                               "build it with pyrsgm_gb300.build.build()")
        h = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            fn = getattr(h, name)
            fn.restype = res
            fn.argtypes = args
        _lib = h
    return _lib


def optional_symbol(name: str, restype, argtypes):
    """Bind an entry point that not every build declares in _SIGS."""
    fn = getattr(lib(), name)
    fn.restype = restype
    fn.argtypes = argtypes
    return fn
