"""Python surface over the C ABI, with torch CUDA tensors as device memory.

This mirrors the reference's two public surfaces for tests, the benchmark and
Python callers:

  * StereoMatcher / Params / validate_params / level geometry
    (reference include/pyrsgm/pyrsgm.h:27-146), through the pyrsgm_gb300_matcher_*
    C surface over the C++ class;
  * Workspace, compute_level, compute_single_scale, pyrdown
    (reference include/pyrsgm/pyrsgm_c.h:38-140).

Errors follow the reference: invalid parameters raise ValueError (the C++
std::invalid_argument), failed launches raise RuntimeError, and the C entry
points' -1 becomes RuntimeError.  torch supplies device memory and streams
only; all compute runs in libpyrsgm_gb300.so.
"""
from __future__ import annotations

import ctypes as C
import dataclasses

import torch

from . import _native
from ._native import lib

COST_BT = 0
COST_CENSUS = 1
POST_LRCHECK = 1
POST_MEDIAN = 2


@dataclasses.dataclass
class Params:
    """pyrsgm::Params (same field names and defaults)."""
    num_disparities: int = 128
    min_disparity: int = 0
    block_size: int = 5
    cost_mode: int = COST_BT
    p1: int = 300
    p2: int = 2400
    uniqueness_ratio: int = 10
    disp12_max_diff: int = 1
    lr_check: bool = True
    median_filter: bool = True
    num_paths: int = 3
    pre_filter_cap: int = 63
    pyramid_levels: int = 0
    pyramid_coarse_disparities: int = 128
    pyramid_max_disparity: int = 0
    pyramid_min_confidence: float = 0.05
    adaptive_p2: bool = False
    p2_alpha: float = 3.041
    p2_beta: float = 16.137
    p2_lower_mult: float = 0.601
    p2_upper_mult: float = 1.77

    def to_c(self) -> _native.Params:
        c = _native.Params()
        for f in dataclasses.fields(self):
            v = getattr(self, f.name)
            setattr(c, f.name, int(v) if isinstance(v, bool) else v)
        return c

    @classmethod
    def from_c(cls, c: _native.Params) -> "Params":
        kw = {}
        for f in dataclasses.fields(cls):
            v = getattr(c, f.name)
            kw[f.name] = bool(v) if f.type in (bool, "bool") else v
        return cls(**kw)


def validate_params(p: Params) -> Params:
    out = _native.Params()
    err = C.create_string_buffer(256)
    if lib().pyrsgm_gb300_validate_params(C.byref(p.to_c()), C.byref(out), err, 256) != 0:
        raise ValueError(err.value.decode())
    return Params.from_c(out)


def invalid_disparity16(p: Params) -> int:
    v = (p.min_disparity - 1) * 16
    return ((v + 0x8000) & 0xFFFF) - 0x8000


@dataclasses.dataclass
class LevelInfo:
    level: int
    width: int
    height: int
    num_labels: int
    max_disparity: int
    block_size: int
    refine: bool


def level_geometry(width: int, height: int, params: Params) -> list[LevelInfo]:
    """Per-level geometry of StereoMatcher(width, height, params); no device memory."""
    out = (C.c_int * 35)()
    err = C.create_string_buffer(256)
    n = lib().pyrsgm_gb300_level_geometry(width, height, C.byref(params.to_c()), out, err, 256)
    if n < 0:
        raise ValueError(err.value.decode())
    return [LevelInfo(out[7 * i], out[7 * i + 1], out[7 * i + 2], out[7 * i + 3], out[7 * i + 4], out[7 * i + 5],
                      bool(out[7 * i + 6])) for i in range(n)]


def _ptr(t: torch.Tensor | None) -> int | None:
    return None if t is None else t.data_ptr()


def _pitch(t: torch.Tensor | None) -> int:
    if t is None:
        return 0
    return t.stride(0) * t.element_size()


def _stream(stream) -> int | None:
    if stream is None:
        return torch.cuda.current_stream().cuda_stream
    return stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream)


class StereoMatcher:
    """pyrsgm::StereoMatcher: fixed image size, all device memory allocated here."""

    def __init__(self, width: int, height: int, params: Params):
        err = C.create_string_buffer(512)
        self._h = lib().pyrsgm_gb300_matcher_create(width, height, C.byref(params.to_c()), err, 512)
        if not self._h:
            msg = err.value.decode()
            raise (RuntimeError if "CUDA" in msg or "allocation" in msg else ValueError)(msg)
        self._width, self._height = width, height
        self._params = validate_params(params)

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().pyrsgm_gb300_matcher_destroy(self._h)
            self._h = None

    __del__ = close

    @property
    def width(self) -> int:
        return self._width

    @property
    def height(self) -> int:
        return self._height

    @property
    def params(self) -> Params:
        return self._params

    def num_levels(self) -> int:
        return lib().pyrsgm_gb300_matcher_num_levels(self._h)

    def level_info(self, level: int) -> LevelInfo:
        out = (C.c_int * 7)()
        if lib().pyrsgm_gb300_matcher_level_info(self._h, level, out) != 0:
            raise IndexError("pyrsgm: level")
        return LevelInfo(out[0], out[1], out[2], out[3], out[4], out[5], bool(out[6]))

    def device_memory_bytes(self) -> int:
        return lib().pyrsgm_gb300_matcher_device_bytes(self._h)

    def compute_into(self, left: torch.Tensor, right: torch.Tensor, disp16: torch.Tensor | None = None,
                     disp32: torch.Tensor | None = None, conf: torch.Tensor | None = None, stream=None) -> None:
        """StereoMatcher::compute with caller-owned (possibly pitched) outputs."""
        err = C.create_string_buffer(512)
        r = lib().pyrsgm_gb300_matcher_compute(
            self._h, _ptr(left), _pitch(left), _ptr(right), _pitch(right),
            _ptr(disp16), _pitch(disp16), _ptr(disp32), _pitch(disp32), _ptr(conf), _pitch(conf),
            _stream(stream), err, 512)
        if r != 0:
            msg = err.value.decode()
            raise (ValueError if "null" in msg or "pitch" in msg else RuntimeError)(msg)

    def compute(self, left: torch.Tensor, right: torch.Tensor, want16: bool = True, want32: bool = False,
                want_conf: bool = False, stream=None) -> dict:
        dev = left.device
        h, w = self._height, self._width
        out = {
            "disp16": torch.empty((h, w), dtype=torch.int16, device=dev) if want16 else None,
            "disp32": torch.empty((h, w), dtype=torch.float32, device=dev) if want32 else None,
            "conf": torch.empty((h, w), dtype=torch.float32, device=dev) if want_conf else None,
        }
        self.compute_into(left, right, out["disp16"], out["disp32"], out["conf"], stream)
        return out


def filter_speckles(disp16: torch.Tensor, new_val: int, max_speckle_size: int, max_diff: int,
                    stream=None) -> torch.Tensor:
    """In place on an int16 device map: regions (4-neighbours differing by at
    most max_diff, none equal to new_val) of at most max_speckle_size pixels
    become new_val (cv::filterSpeckles semantics).  Returns disp16."""
    if disp16.dtype != torch.int16 or disp16.dim() != 2 or not disp16.is_cuda:
        raise ValueError("pyrsgm: filter_speckles takes a 2-D int16 CUDA tensor")
    h, w = disp16.shape
    if lib().pyrsgm_gb300_filter_speckles(_ptr(disp16), _pitch(disp16), w, h, int(new_val), int(max_speckle_size),
                                          int(max_diff), _stream(stream)) != 0:
        raise RuntimeError("pyrsgm: filter_speckles failed")
    return disp16


def set_packed_words(words: int) -> int:
    """Shape of the 16/32/64-label aggregation kernels (0 per launch, 8, or 2/4);
    returns the previous setting.  Results do not depend on it."""
    r = lib().pyrsgm_gb300_set_packed_words(int(words))
    if r < 0:
        raise ValueError("pyrsgm: packed words must be 0, 2, 4 or 8")
    return r


def set_fused(on: bool) -> bool:
    """Fused aggregation passes for the 16-label pyramid levels
    (pyrsgm_gb300_set_fused); returns the previous setting."""
    return bool(lib().pyrsgm_gb300_set_fused(1 if on else 0))


def set_tbw(mode: int) -> int:
    """Winner-take-all inside the top-to-bottom pass of the 16-label pyramid
    levels (pyrsgm_gb300_set_tbw): 0 never, 1 for launches that fill the GPU
    (default), 2 always; returns the previous mode.  Results do not depend
    on it."""
    r = lib().pyrsgm_gb300_set_tbw(int(mode))
    if r < 0:
        raise ValueError("pyrsgm: tbw mode must be 0, 1 or 2")
    return r


def check_report() -> tuple[int, str]:
    """Failures seen by the checked build since load and the first one's
    description (pyrsgm_gb300_check_report); (0, "") in the default build."""
    buf = C.create_string_buffer(256)
    n = lib().pyrsgm_gb300_check_report(buf, 256)
    return int(n), buf.value.decode()


def is_checked() -> bool:
    """Whether the loaded library is the checked build (PYRSGM_GB300_CHECKED=1)."""
    return bool(lib().pyrsgm_gb300_checked())


def fused_stalls(reset: bool = False) -> int:
    """Waits of the fused pass that ran out of time (pyrsgm_gb300_fused_stalls)."""
    return int(lib().pyrsgm_gb300_fused_stalls(1 if reset else 0))


def set_autotune(on: bool) -> bool:
    """Measure the 16/32/64-label kernel shape per launch key on the batch
    engine's first run of each new batch (pyrsgm_gb300_set_autotune);
    returns the previous setting."""
    return bool(lib().pyrsgm_gb300_set_autotune(1 if on else 0))


def autotune_table() -> list[dict]:
    """Recorded shape choices: key (labels, pyramid, rows, width), chosen
    words per thread and the best time of each shape in ms."""
    n = lib().pyrsgm_gb300_autotune_entries(None, 0)
    arr = (_native.TuneEntry * max(n, 1))()
    n = min(n, lib().pyrsgm_gb300_autotune_entries(C.cast(arr, C.c_void_p), n))
    return [{f: (round(getattr(arr[i], f), 4) if f.startswith("ms") else getattr(arr[i], f))
             for f, _ in _native.TuneEntry._fields_} for i in range(n)]


def autotune_clear() -> None:
    lib().pyrsgm_gb300_autotune_clear()


def pair_bytes(width: int, height: int, params: Params) -> int:
    """Device bytes one pair of this shape occupies (StereoMatcher or batch slot)."""
    return lib().pyrsgm_gb300_pair_bytes(width, height, C.byref(params.to_c()))


class BatchEngine:
    """Many pairs of different shapes per launch (pyrsgm_gb300_batch_*).

    run(items) takes dicts with left, right (uint8 [h, w] device tensors),
    params (Params) and optional disp16 / disp32 / conf output tensors.
    """

    def __init__(self, budget_bytes: int):
        err = C.create_string_buffer(256)
        self._h = lib().pyrsgm_gb300_batch_create(budget_bytes, err, 256)
        if not self._h:
            raise RuntimeError(err.value.decode())

    def bytes_in_use(self) -> int:
        return lib().pyrsgm_gb300_batch_bytes_in_use(self._h)

    def reserve(self, width: int, height: int, params: Params, count: int, stream=None) -> None:
        """Allocate now the plans for `count` pairs of this shape (pyrsgm_gb300_batch_reserve)."""
        err = C.create_string_buffer(256)
        if lib().pyrsgm_gb300_batch_reserve(self._h, width, height, C.byref(params.to_c()), count, _stream(stream),
                                            err, 256) != 0:
            raise RuntimeError(err.value.decode())

    @staticmethod
    def make_pairs(items: list[dict]):
        arr = (_native.Pair * len(items))()
        for i, it in enumerate(items):
            L, R = it["left"], it["right"]
            p = arr[i]
            p.d_left, p.left_pitch = _ptr(L), _pitch(L)
            p.d_right, p.right_pitch = _ptr(R), _pitch(R)
            p.d_disp16, p.disp16_pitch = _ptr(it.get("disp16")), _pitch(it.get("disp16"))
            p.d_disp32, p.disp32_pitch = _ptr(it.get("disp32")), _pitch(it.get("disp32"))
            p.d_conf, p.conf_pitch = _ptr(it.get("conf")), _pitch(it.get("conf"))
            p.height, p.width = L.shape
            p.params = it["params"].to_c()
        return arr

    def run_pairs(self, arr, use_graph: bool = True, stream=None) -> None:
        err = C.create_string_buffer(512)
        if lib().pyrsgm_gb300_batch_run(self._h, arr, len(arr), 1 if use_graph else 0, _stream(stream), err, 512):
            raise RuntimeError(err.value.decode())

    def run(self, items: list[dict], use_graph: bool = True, stream=None) -> None:
        self.run_pairs(self.make_pairs(items), use_graph, stream)

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().pyrsgm_gb300_batch_destroy(self._h)
            self._h = None

    __del__ = close


class Server:
    """Continuous-batching server (pyrsgm_gb300_server_*) over host buffers.

    submit() takes uint8 numpy images and returns (request id, outputs dict);
    the outputs are filled when wait(id) returns 1.
    """

    STATS = ("completed", "failed", "p50_ms", "p99_ms", "p999_ms", "mean_batch", "pairs_per_s", "peak_inflight",
             "refused", "max_ms")

    def __init__(self, budget_bytes: int, max_batch: int = 16, streams: int = 2, max_queue: int = 4096):
        err = C.create_string_buffer(256)
        self._h = lib().pyrsgm_gb300_server_create(budget_bytes, max_batch, streams, max_queue, err, 256)
        if not self._h:
            raise RuntimeError(err.value.decode())
        self._keep: dict[int, tuple] = {}
        self._reg: dict[int, object] = {}

    def submit(self, left, right, params: Params, want16: bool = True, want32: bool = False,
               want_conf: bool = False, outputs: dict | None = None):
        import numpy as np
        h, w = left.shape
        left = np.ascontiguousarray(left, dtype=np.uint8)
        right = np.ascontiguousarray(right, dtype=np.uint8)
        out = outputs if outputs is not None else {
            "disp16": np.empty((h, w), np.int16) if want16 else None,
            "disp32": np.empty((h, w), np.float32) if want32 else None,
            "conf": np.empty((h, w), np.float32) if want_conf else None}
        r = _native.Request()
        r.h_left, r.h_right = left.ctypes.data, right.ctypes.data
        r.h_disp16 = out["disp16"].ctypes.data if out.get("disp16") is not None else None
        r.h_disp32 = out["disp32"].ctypes.data if out.get("disp32") is not None else None
        r.h_conf = out["conf"].ctypes.data if out.get("conf") is not None else None
        r.width, r.height = w, h
        r.params = params.to_c()
        err = C.create_string_buffer(256)
        rid = lib().pyrsgm_gb300_server_submit(self._h, C.byref(r), err, 256)
        if rid < 0:
            raise ValueError(err.value.decode())
        self._keep[rid] = (left, right, out)
        return rid, out

    def wait(self, rid: int, timeout: float = -1.0) -> int:
        err = C.create_string_buffer(256)
        s = lib().pyrsgm_gb300_server_wait(self._h, rid, timeout, err, 256)
        if s != 0:
            self._keep.pop(rid, None)
        if s < 0:
            self.last_error = err.value.decode()
        return s

    def drain(self, timeout: float = -1.0) -> bool:
        return lib().pyrsgm_gb300_server_drain(self._h, timeout) == 1

    def stats(self) -> dict:
        o = (C.c_double * 10)()
        lib().pyrsgm_gb300_server_stats(self._h, o)
        return dict(zip(self.STATS, list(o)))

    TIMELINE = ("queue_wait_ms", "enqueue_ms", "gpu_ms", "complete_ms", "batches", "enqueue_max_ms",
                "graph_fraction", "inputs_ms", "kernels_ms", "outputs_ms")

    def timeline(self) -> dict:
        """Mean per-stage times since the last reset (pyrsgm_gb300_server_timeline)."""
        o = (C.c_double * 10)()
        lib().pyrsgm_gb300_server_timeline(self._h, o)
        return dict(zip(self.TIMELINE, list(o)))

    def reset_stats(self) -> None:
        lib().pyrsgm_gb300_server_reset_stats(self._h)

    def inject_failure(self, batches: int) -> None:
        lib().pyrsgm_gb300_server_inject_failure(self._h, batches)

    def reserve(self, width: int, height: int, params: Params, count: int) -> None:
        """Keep plans for `count` pairs of this shape resident in the shared
        pool, and I/O buffers for a full batch of this size on every lane
        (pyrsgm_gb300_server_reserve)."""
        err = C.create_string_buffer(256)
        if lib().pyrsgm_gb300_server_reserve(self._h, width, height, C.byref(params.to_c()), count, err, 256) != 0:
            raise RuntimeError(err.value.decode())

    def register(self, arr) -> bool:
        """Page-lock a numpy array the caller reuses for images or outputs, so
        that requests using it skip the staging copies.  False if refused."""
        err = C.create_string_buffer(256)
        ok = lib().pyrsgm_gb300_server_register(self._h, arr.ctypes.data, arr.nbytes, err, 256) == 0
        if ok:
            self._reg[arr.ctypes.data] = arr
        return ok

    def unregister(self, arr) -> None:
        if self._reg.pop(arr.ctypes.data, None) is not None:
            lib().pyrsgm_gb300_server_unregister(self._h, arr.ctypes.data)

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().pyrsgm_gb300_server_destroy(self._h)
            self._h = None
            self._reg = {}

    __del__ = close


class Workspace:
    """Opaque C-API workspace (pyrsgm_create_workspace / destroy)."""

    def __init__(self):
        self._h = lib().pyrsgm_create_workspace()
        if not self._h:
            raise RuntimeError("pyrsgm: workspace allocation failed")

    @property
    def handle(self) -> int:
        return self._h

    def reserve(self, width: int, height: int, num_disparities: int) -> int:
        return lib().pyrsgm_workspace_reserve(self._h, width, height, num_disparities)

    def set_debug(self, flags: int) -> None:
        lib().pyrsgm_gb300_workspace_set_debug(self._h, flags)

    def volumes(self, stream=None) -> tuple[torch.Tensor, torch.Tensor]:
        """(cost, aggregated) volumes of the last call as [h, w, D] int16 tensors."""
        w, h, d = C.c_int(), C.c_int(), C.c_int()
        if lib().pyrsgm_gb300_workspace_volumes(self._h, None, None, C.byref(w), C.byref(h), C.byref(d)) != 0:
            raise RuntimeError("workspace has no volumes")
        cost = torch.empty((h.value, w.value, d.value), dtype=torch.int16, device="cuda")
        agg = torch.empty_like(cost)
        if lib().pyrsgm_gb300_workspace_copy_volumes(self._h, cost.data_ptr(), agg.data_ptr(), _stream(stream)) != 0:
            raise RuntimeError("volume copy failed")
        return cost, agg

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().pyrsgm_destroy_workspace(self._h)
            self._h = None

    __del__ = close


def pyrdown(src: torch.Tensor, dst: torch.Tensor | None = None, stream=None) -> torch.Tensor:
    h, w = src.shape
    if dst is None:
        dst = torch.empty(((h + 1) // 2, (w + 1) // 2), dtype=torch.uint8, device=src.device)
    r = lib().pyrsgm_pyrdown_u8(_ptr(src), _pitch(src), w, h, _ptr(dst), _pitch(dst),
                                dst.shape[1], dst.shape[0], _stream(stream))
    if r != 0:
        raise RuntimeError("pyrsgm_pyrdown_u8 failed")
    return dst


def compute_level(ws: Workspace, left, right, parent_disp=None, parent_conf=None, disp=None, disp_float=None,
                  conf_float=None, *, num_disparities, min_disparity=0, max_disparity, block_size=5, p1=300,
                  p2=2400, uniqueness=10, disp12_max_diff=1, pre_filter_cap=63, cost_mode=COST_BT,
                  post_flags=POST_LRCHECK, num_paths=3, refine=False, min_confidence=0.05, adaptive_p2=False,
                  p2_alpha=3.041, p2_beta=16.137, p2_lower=0.601, p2_upper=1.77, stream=None) -> int:
    """pyrsgm_compute_level with tensors; returns the C return code."""
    h, w = left.shape
    ph, pw = (parent_disp.shape if parent_disp is not None else (0, 0))
    return lib().pyrsgm_compute_level(
        ws.handle, _ptr(left), _ptr(right), _ptr(parent_disp), _ptr(parent_conf), _ptr(disp), _ptr(disp_float),
        _ptr(conf_float), _pitch(left), _pitch(right), _pitch(parent_disp), _pitch(parent_conf), _pitch(disp),
        _pitch(disp_float), _pitch(conf_float), w, h, pw, ph, num_disparities, min_disparity, max_disparity,
        block_size, p1, p2, uniqueness, disp12_max_diff, pre_filter_cap, cost_mode, post_flags, num_paths,
        1 if refine else 0, min_confidence, 1 if adaptive_p2 else 0, p2_alpha, p2_beta, p2_lower, p2_upper,
        _stream(stream))


def compute_single_scale(ws: Workspace, left, right, disp=None, disp_float=None, conf_float=None, *,
                         num_disparities, min_disparity=0, block_size=5, p1=300, p2=2400, uniqueness=10,
                         disp12_max_diff=1, pre_filter_cap=63, cost_mode=COST_BT,
                         post_flags=POST_LRCHECK | POST_MEDIAN, num_paths=3, adaptive_p2=False, p2_alpha=3.041,
                         p2_beta=16.137, p2_lower=0.601, p2_upper=1.77, stream=None) -> int:
    """pyrsgm_compute_single_scale with tensors; returns the C return code."""
    h, w = left.shape
    return lib().pyrsgm_compute_single_scale(
        ws.handle, _ptr(left), _ptr(right), _ptr(disp), _ptr(disp_float), _ptr(conf_float), _pitch(left),
        _pitch(right), _pitch(disp), _pitch(disp_float), _pitch(conf_float), w, h, num_disparities, min_disparity,
        block_size, p1, p2, uniqueness, disp12_max_diff, pre_filter_cap, cost_mode, post_flags, num_paths,
        1 if adaptive_p2 else 0, p2_alpha, p2_beta, p2_lower, p2_upper, _stream(stream))
