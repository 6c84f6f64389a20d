"""Batched execution: a mixed batch (sizes, label counts, pyramid depths,
cost types, adaptive P2, output subsets) run through one BatchEngine must
give, pair by pair, exactly what StereoMatcher::compute gives for that pair
alone -- with and without CUDA-graph capture, and again on graph replay
with new image contents."""
from __future__ import annotations

import numpy as np
import pytest
import torch

import pyrsgm_gb300 as pg
from pyrsgm_gb300 import synth

pytestmark = pytest.mark.gpu

SIZES = [(160, 96), (200, 120), (240, 136), (128, 72), (96, 64)]


def mixed_batch(n: int, seed: int = 4000):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        w, h = SIZES[rng.integers(len(SIZES))]
        D = int(rng.choice([32, 64, 96, 128]))
        L = int(rng.integers(0, 5))
        cost = int(rng.integers(2))
        p = pg.Params(num_disparities=D, pyramid_levels=L, cost_mode=cost,
                      p1=8 if cost else 300, p2=32 if cost else 2400,
                      adaptive_p2=bool(rng.integers(2)), median_filter=bool(rng.integers(2)),
                      num_paths=int(rng.choice([1, 2, 3, 3])))
        left, right, _ = synth.make_pair(w, h, max(4, min(D - 1, w // 3)), 5, seed + i)
        want = [True, True, True] if i % 4 else [bool(rng.integers(2)), True, bool(rng.integers(2))]
        out.append((p, left, right, want))
    return out


def _alloc(h, w, want):
    return dict(disp16=torch.full((h, w), 1234, dtype=torch.int16, device="cuda") if want[0] else None,
                disp32=torch.full((h, w), -1.0, dtype=torch.float32, device="cuda") if want[1] else None,
                conf=torch.full((h, w), -1.0, dtype=torch.float32, device="cuda") if want[2] else None)


def _alone(p, left, right, want):
    h, w = left.shape
    m = pg.StereoMatcher(w, h, p)
    o = _alloc(h, w, want)
    m.compute_into(torch.from_numpy(left).cuda(), torch.from_numpy(right).cuda(), o["disp16"], o["disp32"], o["conf"])
    torch.cuda.synchronize()
    m.close()
    return {k: (v.cpu().numpy() if v is not None else None) for k, v in o.items()}


def _check(got, want, tag):
    for k in ("disp16", "disp32", "conf"):
        if want[k] is None:
            continue
        if k == "disp16":
            np.testing.assert_array_equal(got[k], want[k], err_msg=f"{tag} {k}")
        else:
            np.testing.assert_allclose(got[k], want[k], rtol=0, atol=1e-6, err_msg=f"{tag} {k}")


@pytest.mark.parametrize("use_graph", [True, False])
def test_batch_matches_each_pair_alone(use_graph):
    batch = mixed_batch(12)
    eng = pg.BatchEngine(8 << 30)
    st = torch.cuda.Stream()
    items, dev = [], []
    for p, left, right, want in batch:
        h, w = left.shape
        L, R = torch.from_numpy(left).cuda(), torch.from_numpy(right).cuda()
        o = _alloc(h, w, want)
        items.append(dict(left=L, right=R, params=p, **o))
        dev.append(o)
    torch.cuda.synchronize()
    eng.run(items, use_graph=use_graph, stream=st)
    torch.cuda.synchronize()
    for i, (p, left, right, want) in enumerate(batch):
        got = {k: (v.cpu().numpy() if v is not None else None) for k, v in dev[i].items()}
        _check(got, _alone(p, left, right, want), f"pair {i}")
    # same buffers, new contents: the cached graph replays on the new images
    batch2 = mixed_batch(12, seed=4500)
    for i, (p, left, right, want) in enumerate(batch):
        h, w = left.shape
        l2, r2, _ = synth.make_pair(w, h, max(4, min(p.num_disparities - 1, w // 3)), 5, 9000 + i)
        items[i]["left"].copy_(torch.from_numpy(l2))
        items[i]["right"].copy_(torch.from_numpy(r2))
        batch2[i] = (p, l2, r2, want)
    torch.cuda.synchronize()
    eng.run(items, use_graph=use_graph, stream=st)
    torch.cuda.synchronize()
    for i, (p, left, right, want) in enumerate(batch2):
        got = {k: (v.cpu().numpy() if v is not None else None) for k, v in dev[i].items()}
        _check(got, _alone(p, left, right, want), f"replay pair {i}")
    eng.close()


def test_batch_budget_is_enforced():
    eng = pg.BatchEngine(4096)  # far too small for any pair
    p, left, right, want = mixed_batch(1)[0]
    h, w = left.shape
    item = dict(left=torch.from_numpy(left).cuda(), right=torch.from_numpy(right).cuda(), params=p,
                disp16=torch.zeros((h, w), dtype=torch.int16, device="cuda"))
    with pytest.raises(RuntimeError, match="budget"):
        eng.run([item])
    eng.close()


def test_batch_rejects_invalid_params():
    eng = pg.BatchEngine(1 << 30)
    L = torch.zeros((48, 64), dtype=torch.uint8, device="cuda")
    with pytest.raises(RuntimeError, match="pyramid_levels"):
        eng.run([dict(left=L, right=L, params=pg.Params(pyramid_levels=7),
                      disp16=torch.zeros((48, 64), dtype=torch.int16, device="cuda"))])
    eng.close()


def test_autotuned_batch_matches_each_pair_alone():
    """With the measuring shape choice on, the first run of a batch times
    both shapes of every 16/32/64-label aggregation launch, records the
    faster, and the captured graph uses it; results are unchanged."""
    prev = pg.set_autotune(True)
    pg.autotune_clear()
    try:
        batch = mixed_batch(12, seed=4700)
        eng = pg.BatchEngine(8 << 30)
        st = torch.cuda.Stream()
        items, dev = [], []
        for p, left, right, want in batch:
            h, w = left.shape
            o = _alloc(h, w, want)
            items.append(dict(left=torch.from_numpy(left).cuda(), right=torch.from_numpy(right).cuda(), params=p, **o))
            dev.append(o)
        torch.cuda.synchronize()
        for _ in range(2):   # tuning run + capture, then a replay
            eng.run(items, use_graph=True, stream=st)
        torch.cuda.synchronize()
        table = pg.autotune_table()
        assert table, "no shape was measured"
        for t in table:
            assert t["num_labels"] in (16, 32, 64) and t["rows"] > 0 and t["width"] > 0
            assert t["words"] in (8, 4 if t["num_labels"] == 64 else 2)
            assert t["ms_wide"] > 0 and t["ms_spread"] > 0
            assert (t["words"] == 8) == (t["ms_wide"] <= t["ms_spread"])
        for i, (p, left, right, want) in enumerate(batch):
            got = {k: (v.cpu().numpy() if v is not None else None) for k, v in dev[i].items()}
            _check(got, _alone(p, left, right, want), f"pair {i}")
        eng.close()
    finally:
        pg.set_autotune(prev)
        pg.autotune_clear()
