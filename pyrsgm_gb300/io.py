"""PFM / PGM files and disparity metrics (pyrsgm_io.h) for numpy arrays.

Host-only: these wrap the library's C functions and need no GPU.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from ._native import Metrics, lib


def _err() -> C.Array:
    return C.create_string_buffer(256)


def _size(fn, path: str) -> tuple[int, int]:
    w, h, e = C.c_int(), C.c_int(), _err()
    if fn(os.fsencode(path), None, 0, C.byref(w), C.byref(h), e, 256) != 0:
        raise OSError(e.value.decode())
    return w.value, h.value


def read_pfm(path: str) -> np.ndarray:
    """Grayscale PFM as float32 [h, w] (top row first; inf kept)."""
    w, h = _size(lib().pyrsgm_gb300_read_pfm, path)
    out = np.empty((h, w), np.float32)
    ww, hh, e = C.c_int(), C.c_int(), _err()
    if lib().pyrsgm_gb300_read_pfm(os.fsencode(path), out.ctypes.data, w, C.byref(ww), C.byref(hh), e, 256) != 0:
        raise OSError(e.value.decode())
    return out


def write_pfm(path: str, a: np.ndarray) -> None:
    """Little-endian grayscale PFM, bottom row first."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    e = _err()
    if lib().pyrsgm_gb300_write_pfm(os.fsencode(path), a.ctypes.data, a.shape[1], a.shape[1], a.shape[0], e, 256):
        raise OSError(e.value.decode())


def read_pgm(path: str) -> np.ndarray:
    """Binary 8-bit PGM as uint8 [h, w]."""
    w, h = _size(lib().pyrsgm_gb300_read_pgm, path)
    out = np.empty((h, w), np.uint8)
    ww, hh, e = C.c_int(), C.c_int(), _err()
    if lib().pyrsgm_gb300_read_pgm(os.fsencode(path), out.ctypes.data, w, C.byref(ww), C.byref(hh), e, 256) != 0:
        raise OSError(e.value.decode())
    return out


def write_pgm(path: str, a: np.ndarray) -> None:
    a = np.ascontiguousarray(a, dtype=np.uint8)
    e = _err()
    if lib().pyrsgm_gb300_write_pgm(os.fsencode(path), a.ctypes.data, a.shape[1], a.shape[1], a.shape[0], e, 256):
        raise OSError(e.value.decode())


def read_ndisp(path: str) -> int:
    """ndisp= of a MiddEval3 calib.txt (0 if absent)."""
    return lib().pyrsgm_gb300_read_ndisp(os.fsencode(path))


def evaluate(disp: np.ndarray, gt: np.ndarray, mask: np.ndarray | None = None, max_disp: float = 1e30) -> dict:
    """Disparity metrics (disp <= 0 invalid; gt non-finite, <= 0 or > max_disp unknown;
    mask 255 = evaluate)."""
    d = np.ascontiguousarray(disp, dtype=np.float32)
    g = np.ascontiguousarray(gt, dtype=np.float32)
    if d.shape != g.shape:
        raise ValueError("disparity and ground truth sizes differ")
    m = None
    if mask is not None:
        m = np.ascontiguousarray(mask, dtype=np.uint8)
        if m.shape != g.shape:
            raise ValueError("mask size differs")
    out = Metrics()
    h, w = g.shape
    if lib().pyrsgm_gb300_evaluate(d.ctypes.data, w, g.ctypes.data, w, m.ctypes.data if m is not None else None, w,
                                   w, h, float(max_disp), C.byref(out)) != 0:
        raise ValueError("evaluate: bad arguments")
    return out.as_dict()
