"""Opt-in speckle filter (pyrsgm_gb300_filter_speckles): the oracle's
sequential flood fill on hand-made maps (CPU), and the GPU union-find
version against the oracle, bit for bit (GPU)."""
from __future__ import annotations

import numpy as np
import pytest

from tests import _oracle

INV = -16


def test_oracle_speckle_rules():
    img = np.full((6, 8), 100, np.int16)
    img[2, 3] = 200            # isolated pixel: a region of one
    img[4, 5:7] = 150          # a region of two
    img[0, 0] = INV            # invalid pixels never join a region
    img[0, 1] = 101            # within max_diff of its neighbours: part of the big region
    out = _oracle.orc_speckles(img, INV, 2, 1)
    want = img.copy()
    want[2, 3] = INV
    want[4, 5:7] = INV
    np.testing.assert_array_equal(out, want)
    # max_size 1 keeps the pair; max_diff 100 merges everything into one region
    out1 = _oracle.orc_speckles(img, INV, 1, 1)
    assert out1[2, 3] == INV and (out1[4, 5:7] == 150).all()
    out2 = _oracle.orc_speckles(img, INV, 2, 100)
    np.testing.assert_array_equal(out2, img)
    # max_size <= 0: nothing changes
    np.testing.assert_array_equal(_oracle.orc_speckles(img, INV, 0, 1), img)


def _blocky(h, w, seed):
    rng = np.random.default_rng(seed)
    img = (rng.integers(0, 8, (h // 4 + 1, w // 4 + 1)) * 20).repeat(4, 0).repeat(4, 1)[:h, :w]
    img = img + rng.integers(0, 3, (h, w))                    # small jitter within regions
    img[rng.random((h, w)) < 0.05] = rng.integers(0, 400)     # speckles
    img[rng.random((h, w)) < 0.08] = INV
    return img.astype(np.int16)


@pytest.mark.gpu
@pytest.mark.parametrize("h,w,max_size,max_diff", [(64, 96, 20, 2), (97, 131, 5, 0), (200, 160, 100, 16),
                                                   (33, 257, 1, 3)])
def test_gpu_speckle_filter_matches_oracle(h, w, max_size, max_diff):
    import torch
    import pyrsgm_gb300 as pg
    img = _blocky(h, w, h * 1000 + w)
    want = _oracle.orc_speckles(img, INV, max_size, max_diff)
    big = torch.full((h, w + 7), 5, dtype=torch.int16, device="cuda")   # pitched view
    d = big[:, :w]
    d.copy_(torch.from_numpy(img))
    pg.filter_speckles(d, INV, max_size, max_diff)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(d.cpu().numpy(), want)
    assert int((big[:, w:] != 5).sum()) == 0


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["ramp", "checker", "blocky_1080p"])
def test_gpu_speckle_filter_large_and_extreme_maps(kind):
    """One region spanning every tile (a ramp whose steps are within
    max_diff), no region larger than one pixel (a checkerboard of far-apart
    values), and a 1080p map."""
    import torch
    import pyrsgm_gb300 as pg
    if kind == "ramp":
        h, w = 300, 517
        img = (np.add.outer(np.arange(h), np.arange(w)) % 700).astype(np.int16)
        max_size, max_diff = 100, 1
    elif kind == "checker":
        h, w = 129, 250
        img = np.where(np.add.outer(np.arange(h), np.arange(w)) % 2 == 0, 10, 500).astype(np.int16)
        max_size, max_diff = 1, 5
    else:
        h, w = 1080, 1920
        img = _blocky(h, w, 77)
        max_size, max_diff = 100, 20          # neighbouring blocks join or not depending on the jitter
    want = _oracle.orc_speckles(img, INV, max_size, max_diff)
    d = torch.from_numpy(img).cuda()
    pg.filter_speckles(d, INV, max_size, max_diff)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(d.cpu().numpy(), want)
