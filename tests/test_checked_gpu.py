"""The checked build (libpyrsgm_gb300_checked.so, compiled with
PYRSGM_CHECKED): range checks at the kernels' main global-memory accesses
(a failed check records its site and skips the access), a wait and an
error check after every launch, no CUDA graphs.  It stands in for a memory
checker.  Run in a child process (the library is chosen at import by
PYRSGM_GB300_CHECKED=1): every kind of level and kernel form, a batch of
real-size pairs and a matcher, each result equal to the oracle's or the
default library's, and no failure reported."""
from __future__ import annotations

import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r'''
import numpy as np
import torch
import pyrsgm_gb300 as pg
from pyrsgm_gb300 import synth
from tests import _runners, cases
assert pg.is_checked()
torch.cuda.set_device(0)
levels = [c for c in cases.LEVELS if c["D"] == 16][:2] + [cases.LEVELS[1]]
single = [c for c in cases.SINGLE_SCALE if c["D"] not in (16, 32, 64)][:1] + cases.SINGLE_SCALE[:1]
n = 0
# every form of the 16/32/64-label aggregation, and the other path kernels
for words, fused, tbw in ((8, False, 2), (8, False, 0), (8, True, 1), (2, False, 1)):
    pg.set_packed_words(words); pg.set_fused(fused); pg.set_tbw(tbw)
    for case in levels + single:
        mine = _runners.run_mine(case)
        bad = _runners.compare(mine, _runners.run_oracle(case, _runners.device_lut(case)))
        assert not bad, (case["name"], words, fused, tbw, bad)
        n += 1
pg.set_packed_words(0); pg.set_fused(False); pg.set_tbw(1)
# a batch of two 1080p D=256 pairs (Census, BT) against the same pairs computed alone
items, alone = [], []
for i, cost in enumerate((pg.COST_CENSUS, pg.COST_BT)):
    left, right, _ = synth.make_pair(1920, 1080, 255, 16, 7000 + i)
    p = pg.Params(num_disparities=256, pyramid_levels=3, cost_mode=cost, p1=8 if cost == pg.COST_CENSUS else 300,
                  p2=32 if cost == pg.COST_CENSUS else 2400, adaptive_p2=True, median_filter=True)
    L, R = torch.from_numpy(left).cuda(), torch.from_numpy(right).cuda()
    out = dict(disp16=torch.empty((1080, 1920), dtype=torch.int16, device="cuda"))
    items.append(dict(left=L, right=R, params=p, **out))
    m = pg.StereoMatcher(1920, 1080, p)
    d16 = torch.empty((1080, 1920), dtype=torch.int16, device="cuda")
    m.compute_into(L, R, d16, None, None)
    alone.append(d16)
eng = pg.BatchEngine(16 << 30)
eng.run(items, use_graph=True)
torch.cuda.synchronize()
for it, a in zip(items, alone):
    assert torch.equal(it["disp16"], a)
    assert int((a > 0).sum()) > 0
eng.close()
fails, first = pg.check_report()
assert fails == 0, first
print("checked ok", n)
'''


def test_checked_build_runs_clean():
    from pyrsgm_gb300 import build
    build.build(checked=True)
    env = dict(os.environ, PYRSGM_GB300_CHECKED="1")
    r = subprocess.run([sys.executable, "-c", CHILD], cwd=ROOT, env=env, capture_output=True, text=True, timeout=1200)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    assert "checked ok" in r.stdout
