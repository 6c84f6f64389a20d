"""PFM / PGM files and disparity metrics (include/pyrsgm/pyrsgm_io.h), host
only.  The PFM conventions follow the reference's reader (bench/middlebury.h:
22-53: grayscale "Pf", negative scale = little-endian, bottom row first,
inf kept) and writer (examples/stereo_pair.cpp:37-44); the metrics its
evaluate() (bench/middlebury.h:78-120), restated here in numpy."""
from __future__ import annotations

import os

import numpy as np
import pytest

from pyrsgm_gb300 import io


def test_pfm_round_trip_keeps_every_value(tmp_path):
    rng = np.random.default_rng(1)
    a = rng.normal(0, 100, (37, 53)).astype(np.float32)
    a[3, 4] = np.inf
    a[5, 6] = -0.0
    p = str(tmp_path / "a.pfm")
    io.write_pfm(p, a)
    with open(p, "rb") as f:
        assert f.read(3) == b"Pf\n"
    b = io.read_pfm(p)
    assert b.dtype == np.float32 and b.shape == a.shape
    np.testing.assert_array_equal(b, a)


def test_pfm_file_layout_is_bottom_up_little_endian(tmp_path):
    a = np.arange(12, dtype=np.float32).reshape(3, 4)
    p = str(tmp_path / "a.pfm")
    io.write_pfm(p, a)
    data = open(p, "rb").read()
    assert data.startswith(b"Pf\n4 3\n-1.0\n")
    body = np.frombuffer(data[len(b"Pf\n4 3\n-1.0\n"):], dtype="<f4").reshape(3, 4)
    np.testing.assert_array_equal(body[::-1], a)


def test_big_endian_pfm_is_read(tmp_path):
    a = np.array([[1.5, -2.0, np.inf], [0.25, 7.0, 100.0]], np.float32)
    p = str(tmp_path / "be.pfm")
    with open(p, "wb") as f:
        f.write(b"Pf\n3 2\n1.0\n")
        f.write(a[::-1].astype(">f4").tobytes())
    np.testing.assert_array_equal(io.read_pfm(p), a)


def test_pgm_round_trip_and_header_comments(tmp_path):
    rng = np.random.default_rng(2)
    a = rng.integers(0, 256, (19, 31), dtype=np.uint8)
    p = str(tmp_path / "a.pgm")
    io.write_pgm(p, a)
    np.testing.assert_array_equal(io.read_pgm(p), a)
    q = str(tmp_path / "c.pgm")
    with open(q, "wb") as f:
        f.write(b"P5\n# made by hand\n31 19\n255\n" + a.tobytes())
    np.testing.assert_array_equal(io.read_pgm(q), a)


def test_bad_files_raise(tmp_path):
    with pytest.raises(OSError, match="cannot open"):
        io.read_pfm(str(tmp_path / "missing.pfm"))
    p = str(tmp_path / "color.pfm")
    with open(p, "wb") as f:
        f.write(b"PF\n2 2\n-1.0\n" + bytes(48))
    with pytest.raises(OSError, match="grayscale"):
        io.read_pfm(p)
    q = str(tmp_path / "short.pfm")
    with open(q, "wb") as f:
        f.write(b"Pf\n4 4\n-1.0\n" + bytes(20))
    with pytest.raises(OSError, match="truncated"):
        io.read_pfm(q)
    r = str(tmp_path / "ascii.pgm")
    with open(r, "wb") as f:
        f.write(b"P2\n2 2\n255\n1 2 3 4\n")
    with pytest.raises(OSError, match="P5"):
        io.read_pgm(r)


def test_read_ndisp(tmp_path):
    p = str(tmp_path / "calib.txt")
    with open(p, "w") as f:
        f.write("cam0=[1 0 0; 0 1 0; 0 0 1]\ndoffs=0\nbaseline=100\nwidth=640\nheight=480\nndisp=256\nvmin=10\n")
    assert io.read_ndisp(p) == 256
    assert io.read_ndisp(str(tmp_path / "none.txt")) == 0


def _metrics_np(d, g, mask, max_disp):
    known = np.isfinite(g) & (g > 0) & (g <= max_disp)
    if mask is not None:
        known &= mask == 255
    ev = int(known.sum())
    valid = known & (d > 0)
    nv = int(valid.sum())
    e = np.abs(d[valid].astype(np.float64) - g[valid].astype(np.float64))
    out = {"evaluated": ev, "valid": nv}
    if nv:
        out.update(avg_err=e.mean(), rms_err=np.sqrt((e * e).mean()),
                   bad05=100 * (e > 0.5).sum() / nv, bad1=100 * (e > 1).sum() / nv,
                   bad2=100 * (e > 2).sum() / nv, bad4=100 * (e > 4).sum() / nv)
    if ev:
        out.update(density=100 * nv / ev, invalid=100 - 100 * nv / ev,
                   bad1_all=100 * ((e > 1).sum() + ev - nv) / ev, bad2_all=100 * ((e > 2).sum() + ev - nv) / ev)
    return out


@pytest.mark.parametrize("with_mask", [False, True])
def test_evaluate_matches_the_metric_definitions(with_mask):
    rng = np.random.default_rng(3)
    g = rng.uniform(0, 80, (40, 60)).astype(np.float32)
    g[rng.random(g.shape) < 0.1] = np.inf
    g[rng.random(g.shape) < 0.05] = 0.0
    d = (g + rng.normal(0, 1.5, g.shape)).astype(np.float32)
    d[rng.random(g.shape) < 0.15] = 0.0
    d[rng.random(g.shape) < 0.02] = np.nan
    mask = np.where(rng.random(g.shape) < 0.7, 255, 128).astype(np.uint8) if with_mask else None
    got = io.evaluate(d, g, mask, max_disp=64.0)
    want = _metrics_np(d, g, mask, 64.0)
    for k, v in want.items():
        assert got[k] == pytest.approx(v, rel=1e-9, abs=1e-9), k


def test_evaluate_empty_ground_truth():
    g = np.full((4, 4), np.inf, np.float32)
    m = io.evaluate(np.ones((4, 4), np.float32), g)
    assert m["evaluated"] == 0 and m["valid"] == 0 and m["density"] == 0.0
