"""The tiled contact pass skips a staged block of 32 bodies when the FP32
gap between its bounding box and the warp's box gives gap2 >= 1
(gi_grid.cu, box_gap2).  The skip is sound only if no pair drawn from the
two boxes can pass the pair filter r2 < 1 in the filter's own rounding.
This restates both computations in numpy (float32 subtractions; the
filter's fma(dz, dz, fma(dx, dx, dy * dy)) emulated in float64, where the
float32 products are exact and the sum rounds once more before the float32
rounding, so it can differ from a true fma in the last place, rarely; every
rounding step is monotone either way, which is what the bound rests on) and
searches adversarial boxes a few ulps around distance 1 at large
coordinates."""
from __future__ import annotations

import numpy as np

f32 = np.float32


def fma32(a, b, c):
    return (np.asarray(a, np.float64) * np.asarray(b, np.float64) + np.asarray(c, np.float64)).astype(np.float32)


def r2_filter(pj, pi):
    dx = (pj[..., 0] - pi[..., 0]).astype(np.float32)
    dy = (pj[..., 1] - pi[..., 1]).astype(np.float32)
    dz = (pj[..., 2] - pi[..., 2]).astype(np.float32)
    return fma32(dz, dz, fma32(dx, dx, (dy * dy).astype(np.float32)))


def gap2(ilo, ihi, jlo, jhi):
    g = np.maximum(np.maximum((jlo - ihi).astype(np.float32), (ilo - jhi).astype(np.float32)), f32(0))
    return fma32(g[..., 2], g[..., 2], fma32(g[..., 0], g[..., 0], (g[..., 1] * g[..., 1]).astype(np.float32)))


def test_skip_never_drops_a_pair():
    rng = np.random.default_rng(17)
    m = 200000
    base = (rng.uniform(-1, 1, size=(m, 1, 3)) * 10.0 ** rng.integers(0, 4, size=(m, 1, 1))).astype(np.float32)
    # i box: a point cloud near base; j box offset so the gap is about 1 +- a few ulps along a
    # random axis mix
    direction = rng.normal(size=(m, 1, 3))
    direction /= np.linalg.norm(direction, axis=-1, keepdims=True)
    ulps = rng.integers(-6, 7, size=(m, 1, 1))
    dist = (1.0 + ulps * 2.0 ** -23).astype(np.float64)
    pi = (base + rng.uniform(0, 0.25, size=(m, 4, 3))).astype(np.float32)
    ihi = pi.max(axis=1, keepdims=True)
    ilo = pi.min(axis=1, keepdims=True)
    corner = np.where(direction > 0, ihi, ilo).astype(np.float64)
    jstart = (corner + direction * dist).astype(np.float32)
    pj = (jstart + np.where(direction > 0, 1, -1) * rng.uniform(0, 0.25, size=(m, 4, 3))).astype(np.float32)
    pj[:, 0, :] = jstart[:, 0, :]  # the nearest corner itself
    jlo = pj.min(axis=1, keepdims=True)
    jhi = pj.max(axis=1, keepdims=True)
    g2 = gap2(ilo[:, 0], ihi[:, 0], jlo[:, 0], jhi[:, 0])
    # every (i, j) pair's filter value
    r2 = r2_filter(pj[:, None, :, :], pi[:, :, None, :]).reshape(m, -1)
    skipped = g2 >= 1.0
    assert skipped.any() and (~skipped).any()
    assert np.all(r2[skipped] >= 1.0)
    # the bound is a lower bound for every pair, skipped or not
    assert np.all(r2 >= g2[:, None])
