"""The paired far field's decomposition, checked on the host (no GPU).

gi_debug_pair_plan returns the library's own numbers for a run of n bodies:
log2 of the j-chunks per work item (cpi = 2^pcl), the run's 64-body j-chunks
and 1,024-body i-blocks, its work items and the stride of the item
permutation.  The tests restate the kernel's rules (gi_force_pair.cu):

  * i-block a takes the j-chunks from its own first body to the end of the
    run, cpi at a time, so it has ceil((C - 16 a) / cpi) items;
  * CTA t takes item (t * stride) mod items, decoded into (a, k) by the
    arithmetic series of the items before each block;
  * in an item, warp w (rows a 1024 + 256 w .. + 256) skips the chunks that
    end at or before its first row, keeps only i < j on the chunks that
    overlap its rows, and takes every pair of the chunks after them;

and check that the item count, the permutation and the decode are
consistent, and that every unordered pair i < j is evaluated exactly once
(a lane holds two j-bodies of a chunk, slots l and l + 32; the rules above
are per chunk, so the lane split does not enter them).
"""
from __future__ import annotations

import math

import numpy as np
import pytest

ROWS, CHUNK, WARP_ROWS, BLOCK_CHUNKS = 1024, 64, 256, 16


def _items_before(a, k0, q):
    return a * k0 - q * (a * (a - 1) // 2)


def _decode(t, plan):
    """(i-block, first chunk, chunks) of permuted item t, as the kernel does."""
    cpi = 1 << plan["pcl"]
    q = BLOCK_CHUNKS // cpi
    u = (t * plan["stride"]) % plan["items"]
    lo, hi = 0, plan["iblocks"] - 1
    while lo < hi:
        mid = (lo + hi + 1) >> 1
        if _items_before(mid, plan["items_block0"], q) <= u:
            lo = mid
        else:
            hi = mid - 1
    c0 = lo * BLOCK_CHUNKS + (u - _items_before(lo, plan["items_block0"], q)) * cpi
    return lo, c0, min(cpi, plan["chunks"] - c0)


@pytest.mark.parametrize("n", [1, 2, 31, 32, 33, 255, 1023, 1024, 1025, 3000, 4600, 8192, 25000,
                               32767, 32768, 66000, 131071, 131072, 1153434])
def test_default_plan_counts(gi, n):
    plan = gi.pair_plan(n)
    cpi = 1 << plan["pcl"]
    # the default: 4 chunks of 64 per item below 32,768 bodies, 8 below 131,072, 16 above
    assert cpi == (4 if n < 32768 else 8 if n < 131072 else 16)
    C = -(-n // CHUNK)
    nb = -(-n // ROWS)
    assert plan["chunks"] == C and plan["iblocks"] == nb
    assert plan["items_block0"] == -(-C // cpi)
    assert plan["items"] == sum(-(-(C - BLOCK_CHUNKS * a) // cpi) for a in range(nb))
    assert math.gcd(plan["stride"], plan["items"]) == 1


@pytest.mark.parametrize("pcl", [0, 1, 2, 3, 4])
@pytest.mark.parametrize("n", [1, 33, 65, 1000, 1025, 2049, 5000])
def test_permutation_and_decode_cover_every_item_once(gi, n, pcl):
    plan = gi.pair_plan(n, pcl)
    assert plan["pcl"] == pcl
    seen = set()
    for t in range(plan["items"]):
        a, c0, nch = _decode(t, plan)
        assert 0 <= a < plan["iblocks"] and nch >= 1
        assert a * BLOCK_CHUNKS <= c0 < plan["chunks"]
        assert (c0 - a * BLOCK_CHUNKS) % (1 << pcl) == 0
        seen.add((a, c0))
    assert len(seen) == plan["items"]


@pytest.mark.parametrize("pcl", [0, 2, 4])
@pytest.mark.parametrize("n", [2, 40, 100, 257, 1030, 2600])
def test_every_pair_once(gi, n, pcl):
    plan = gi.pair_plan(n, pcl)
    count = np.zeros((n, n), np.uint8)
    for t in range(plan["items"]):
        a, c0, nch = _decode(t, plan)
        for w in range(ROWS // WARP_ROWS):
            r0 = a * ROWS + w * WARP_ROWS
            rows = np.arange(r0, min(r0 + WARP_ROWS, n))
            if len(rows) == 0:
                continue
            for c in range(c0, c0 + nch):
                j0 = c * CHUNK
                if j0 + CHUNK <= r0:
                    continue  # before the warp's rows: the warp owning them covers it
                cols = np.arange(j0, min(j0 + CHUNK, n))
                ii, jj = np.meshgrid(rows, cols, indexing="ij")
                keep = ii < jj
                np.add.at(count, (ii[keep], jj[keep]), 1)
    upper = np.triu(np.ones((n, n), bool), 1)
    assert (count[upper] == 1).all()
    assert (count[~upper] == 0).all()
