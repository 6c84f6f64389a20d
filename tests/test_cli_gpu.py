"""The headless stereo CLI (pyrsgm_gb300/pyrsgm_stereo_pair, the reference's
examples/stereo_pair.cpp without OpenCV): PGM in, PFM/PGM out, metrics
against a ground-truth PFM.  Its disparity file must hold exactly what
StereoMatcher::compute returns for the same pair and parameters."""
from __future__ import annotations

import os
import subprocess

import numpy as np
import pytest
import torch

import pyrsgm_gb300 as pg
from pyrsgm_gb300 import build, io, synth

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("cost", ["bt", "census"])
def test_cli_output_equals_compute(tmp_path, cost):
    w, h, D, L = 320, 200, 64, 2
    left, right, truth = synth.make_pair(w, h, D - 1, 6, 8100 + (cost == "census"))
    lp, rp, gp = str(tmp_path / "l.pgm"), str(tmp_path / "r.pgm"), str(tmp_path / "gt.pfm")
    io.write_pgm(lp, left)
    io.write_pgm(rp, right)
    io.write_pfm(gp, truth)
    prefix = str(tmp_path / "out")
    assert os.path.exists(build.CLI), "CLI not built"
    r = subprocess.run([build.CLI, lp, rp, prefix, str(D), str(L), cost, "--gt", gp],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert "ms per frame" in r.stdout and "bad1(all)" in r.stdout
    disp = io.read_pfm(prefix + "_disp.pfm")
    conf8 = io.read_pgm(prefix + "_conf.pgm")
    assert disp.shape == (h, w) and conf8.shape == (h, w)

    p = pg.Params(num_disparities=D, pyramid_levels=L)   # the CLI's parameters: defaults, Census with P1 8 / P2 32
    if cost == "census":
        p = pg.Params(num_disparities=D, pyramid_levels=L, cost_mode=1, p1=8, p2=32)
    m = pg.StereoMatcher(w, h, p)
    out = m.compute(torch.from_numpy(left).cuda(), torch.from_numpy(right).cuda(), False, True, True)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(disp, out["disp32"].cpu().numpy())
    # conf * 255 rounded to a byte (a fused multiply-add may round the .5 cases the other way)
    want8 = np.clip(out["conf"].cpu().numpy().astype(np.float64) * 255.0 + 0.5, 0, 255).astype(np.int32)
    assert np.abs(conf8.astype(np.int32) - want8).max() <= 1
    met = io.evaluate(disp, truth, None, float(D))
    assert met["evaluated"] > 0.5 * w * h and met["bad1_all"] < 60.0
    m.close()


def test_cli_rejects_bad_input(tmp_path):
    r = subprocess.run([build.CLI, str(tmp_path / "no.pgm"), str(tmp_path / "no.pgm"), str(tmp_path / "o")],
                       capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "cannot open" in r.stderr
    r = subprocess.run([build.CLI], capture_output=True, text=True, timeout=60)
    assert r.returncode == 2 and "usage" in r.stderr
