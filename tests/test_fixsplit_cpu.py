"""The contact pass rounds each FP32 pair term to a 64-bit fixed-point
integer on the FP32 pipe (gi_grid.cu, fix_split / fix_value): a magic-number
split into hi * 2^23 + lo.  These tests restate that arithmetic in numpy
float32 (IEEE round-to-nearest-even, no FMA) and check it against exact
round-half-even over every binade the split takes, the tie cases, and a
256-term sum taken mod 2^32 as the kernels do."""
from __future__ import annotations

import numpy as np

M = np.float32(1.5 * 2.0 ** 46)
C = np.float32(1.5 * 2.0 ** 23)
LIMIT = np.float32(2.0 ** 45)


def bits(a):
    return np.asarray(a, np.float32).view(np.uint32).astype(np.int64)


def split(x):
    x = np.asarray(x, np.float32)
    s = (x + M).astype(np.float32)
    lo = (x - (s - M).astype(np.float32)).astype(np.float32)
    l = (lo + C).astype(np.float32)
    return bits(s), bits(l)


def value(h, l, n):
    hi = ((h - n * int(bits(M))) + 2 ** 31) % 2 ** 32 - 2 ** 31
    lo = ((l - n * int(bits(C))) + 2 ** 31) % 2 ** 32 - 2 ** 31
    return hi * (1 << 23) + lo


def exact(x):
    return np.rint(np.asarray(x, np.float32).astype(np.float64)).astype(np.int64)


def test_every_binade_below_the_limit():
    rng = np.random.default_rng(7)
    exps = np.arange(0, 127 + 45)          # biased exponents: 0 (zero, subnormals) .. 2^44
    mant = rng.integers(0, 1 << 23, size=(len(exps), 4000), dtype=np.uint32)
    u = (exps[:, None].astype(np.uint32) << 23) | mant
    u = np.concatenate([u.ravel(), u.ravel() | np.uint32(0x80000000)])
    x = u.view(np.float32)
    assert np.all(np.abs(x) < LIMIT)
    h, l = split(x)
    assert np.array_equal(value(h, l, 1), exact(x))


def test_ties_and_edges():
    pts = [0.0, -0.0, 0.5, 1.5, 2.5, -0.5, -1.5, -2.5, 2.0 ** 22, 2.0 ** 22 + 0.5, 2.0 ** 22 + 1.5,
           2.0 ** 23 - 0.5, 2.0 ** 23 - 1.5, 2.0 ** 23, 2.0 ** 23 + 1, 2.0 ** 24 + 2, 2.0 ** 44,
           np.nextafter(np.float32(2.0 ** 45), np.float32(0)), 3 * 2.0 ** 22, 5 * 2.0 ** 22,
           2.0 ** 22 * 1.5 + 0.5, 1e-45, 1e-30]
    x = np.array(pts + [-p for p in pts], np.float32)
    assert np.all(np.abs(x) < LIMIT)
    # every multiple of 2^22 +- a few ulp around the hi boundaries
    k = np.arange(-(1 << 23), (1 << 23) + 1, 4099, dtype=np.int64)
    near = np.concatenate([(k * 2.0 ** 22 + d) for d in (-1.5, -1.0, -0.5, 0.0, 0.5, 1.0, 1.5)])
    near = near[np.abs(near) < 2.0 ** 45].astype(np.float32)
    x = np.concatenate([x, near])
    h, l = split(x)
    assert np.array_equal(value(h, l, 1), exact(x))


def test_sum_of_256_terms_mod_2_32():
    rng = np.random.default_rng(11)
    for scale in (2.0 ** 44, 2.0 ** 30, 2.0 ** 23, 3.0, 0.7):
        x = (rng.uniform(-1, 1, size=(50, 256)) * scale).astype(np.float32)
        h, l = split(x)
        hs = h.sum(axis=1) % 2 ** 32
        ls = l.sum(axis=1) % 2 ** 32
        assert np.array_equal(value(hs, ls, 256), exact(x).sum(axis=1))


def test_pair_term_is_the_exact_negation():
    """A pair of two crowded cells is evaluated once: body j receives the
    negation of body i's rounded term.  Body j's own evaluation would round
    -x (dp and dv change sign exactly, the coefficient is symmetric), so the
    negation must equal round(-x), ties included."""
    rng = np.random.default_rng(13)
    x = np.concatenate([
        (rng.uniform(-1, 1, size=200000) * 2.0 ** rng.uniform(-2, 44, size=200000)),
        np.arange(-64, 65) * 0.5,                       # every tie near zero
        (np.arange(-64, 65) + 0.5) * 2.0 ** 22,         # ties at the largest fractional binade
    ]).astype(np.float32)
    x = x[np.abs(x) < LIMIT]
    h, l = split(x)
    hn, ln = split(-x)
    assert np.array_equal(-value(h, l, 1), value(hn, ln, 1))
    assert np.array_equal(-value(h, l, 1), exact(-x))
