"""pyrsgm-gb300: coarse-to-fine Semi-Global Matching on NVIDIA GB300 (sm_103a).

The product is the native library libpyrsgm_gb300.so (C ABI in
include/pyrsgm/); this package builds it (pyrsgm_gb300.build) and exposes a
thin Python surface over it (pyrsgm_gb300.api).
"""
from .api import (COST_BT, COST_CENSUS, POST_LRCHECK, POST_MEDIAN, BatchEngine, LevelInfo, Params,
                  Server, StereoMatcher, Workspace, pair_bytes, compute_level, compute_single_scale, invalid_disparity16, level_geometry,
                  pyrdown, set_packed_words, validate_params, filter_speckles, set_autotune, set_fused, set_tbw, fused_stalls, check_report, is_checked, autotune_table,
                  autotune_clear)

__all__ = ["COST_BT", "COST_CENSUS", "POST_LRCHECK", "POST_MEDIAN", "BatchEngine", "LevelInfo", "pair_bytes", "Server", "Params", "StereoMatcher",
           "Workspace", "compute_level", "compute_single_scale", "invalid_disparity16", "level_geometry", "pyrdown",
           "set_packed_words", "validate_params", "filter_speckles", "set_autotune", "set_fused", "set_tbw", "fused_stalls", "check_report", "is_checked", "autotune_table",
           "autotune_clear"]
