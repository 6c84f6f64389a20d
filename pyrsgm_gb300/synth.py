"""Seeded synthetic stereo pairs standing in for the Middlebury scenes.

The reference benchmarks on Middlebury MiddEval3 (not available offline);
these pairs reproduce its sizes and disparity ranges with a known ground
truth:

  left   = 0.6 * value noise (4 octaves, 0..255) + 0.4 * uniform noise
  truth  = K planar slanted patches on a Voronoi partition,
           d = a*x + b*y + c clamped to [0, d_max]
  right  = left forward-warped by -d (nearer surfaces win, unfilled
           occluded pixels get fresh noise) + N(0, sigma), rounded to uint8

Pair i of configuration k uses seed 1000*k + i.  numpy only; deterministic for
a given seed on any machine.
"""
from __future__ import annotations

import numpy as np


def _value_noise(rng: np.random.Generator, h: int, w: int, octaves: int = 4, cell: int = 32) -> np.ndarray:
    out = np.zeros((h, w), np.float64)
    amp, total = 1.0, 0.0
    ys = np.arange(h, dtype=np.float64)
    xs = np.arange(w, dtype=np.float64)
    for o in range(octaves):
        c = max(2, cell >> o)
        gh, gw = h // c + 2, w // c + 2
        grid = rng.random((gh, gw))
        fy, fx = ys / c, xs / c
        y0, x0 = np.floor(fy).astype(int), np.floor(fx).astype(int)
        ty, tx = fy - y0, fx - x0
        ty, tx = ty * ty * (3 - 2 * ty), tx * tx * (3 - 2 * tx)  # smoothstep
        g00 = grid[np.ix_(y0, x0)]
        g01 = grid[np.ix_(y0, x0 + 1)]
        g10 = grid[np.ix_(y0 + 1, x0)]
        g11 = grid[np.ix_(y0 + 1, x0 + 1)]
        top = g00 + (g01 - g00) * tx[None, :]
        bot = g10 + (g11 - g10) * tx[None, :]
        out += amp * (top + (bot - top) * ty[:, None])
        total += amp
        amp *= 0.5
    return out / total * 255.0


def ground_truth(rng: np.random.Generator, h: int, w: int, d_max: float, patches: int) -> np.ndarray:
    """K slanted planes on a Voronoi partition, clamped to [0, d_max]."""
    sy = rng.uniform(0, h, patches)
    sx = rng.uniform(0, w, patches)
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float64)
    best = np.full((h, w), np.inf)
    label = np.zeros((h, w), np.int32)
    for k in range(patches):
        dist = (yy - sy[k]) ** 2 + (xx - sx[k]) ** 2
        m = dist < best
        best[m] = dist[m]
        label[m] = k
    c = rng.uniform(0.1 * d_max, 0.9 * d_max, patches)
    a = rng.uniform(-0.15, 0.15, patches) * d_max / w
    b = rng.uniform(-0.15, 0.15, patches) * d_max / h
    d = a[label] * (xx - sx[label]) + b[label] * (yy - sy[label]) + c[label]
    return np.clip(d, 0.0, d_max)


def make_pair(width: int, height: int, d_max: int, patches: int, seed: int,
              noise_sigma: float = 2.0) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Returns (left u8 [h,w], right u8 [h,w], truth float32 [h,w])."""
    rng = np.random.default_rng(seed)
    h, w = height, width
    left = 0.6 * _value_noise(rng, h, w) + 0.4 * rng.uniform(0, 255, (h, w))
    left_u8 = np.clip(np.rint(left), 0, 255).astype(np.uint8)
    d = ground_truth(rng, h, w, float(d_max), patches)
    # forward warp: right(x - d(x)) = left(x); the nearer (larger d) surface wins
    yy, xx = np.mgrid[0:h, 0:w]
    xr = np.rint(xx - d).astype(np.int64)
    ok = (xr >= 0) & (xr < w)
    target = (yy * w + xr)[ok]
    key = (np.rint(d * 16).astype(np.int64)[ok] << 20) | xx[ok].astype(np.int64)
    order = np.lexsort((key, target))          # by target, then key ascending
    ts, ks = target[order], key[order]
    last = np.flatnonzero(np.r_[ts[1:] != ts[:-1], True])  # largest key of each target
    best = np.full(h * w, -1, np.int64)
    best[ts[last]] = ks[last]
    filled = best >= 0
    src_x = (best & ((1 << 20) - 1)).reshape(h, w)
    right = rng.uniform(0, 255, (h, w))
    rows = np.repeat(np.arange(h)[:, None], w, axis=1)
    fm = filled.reshape(h, w)
    right[fm] = left_u8[rows[fm], src_x[fm]]
    right += rng.normal(0.0, noise_sigma, (h, w))
    right_u8 = np.clip(np.rint(right), 0, 255).astype(np.uint8)
    return left_u8, right_u8, d.astype(np.float32)


# Named workloads (width, height, num_disparities, pyramid_levels, patches)
WORKLOADS = {
    "640x480_D64_L0_bt": (640, 480, 64, 0, 6),
    "1280x720_D128_L2_census": (1280, 720, 128, 2, 10),
    "1920x1080_D256_L3": (1920, 1080, 256, 3, 16),
    "1920x1080_D256_L2_census": (1920, 1080, 256, 2, 16),
}
