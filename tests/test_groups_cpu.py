"""CPU tests of the Earth / Moon grouping oracles: the literal restatement of
the reference's group loop (findEarthAndMoon) against an independent
union-find, on clumps, chains, debris and ties."""
from __future__ import annotations

import numpy as np
import pytest


def clumps(seed, sizes, spacing=1.2, debris=0, far=60.0):
    """Lattice clumps (neighbours 1.2 apart: touching at 1.5) far apart, plus
    isolated debris; shuffled so that group numbers are not contiguous."""
    rng = np.random.default_rng(seed)
    pts = []
    for k, m in enumerate(sizes):
        side = int(np.ceil(m ** (1 / 3)))
        g = np.stack(np.meshgrid(*[np.arange(side)] * 3, indexing="ij"), -1).reshape(-1, 3)[:m]
        pts.append(g * spacing + np.array([k * far, 0.0, 0.0]))
    for _ in range(debris):
        pts.append(rng.uniform(-500, 500, size=(1, 3)) + np.array([0.0, 800.0, 0.0]))
    p = np.concatenate(pts)
    p = p[rng.permutation(len(p))]
    out = np.zeros((len(p), 4), np.float32)
    out[:, :3] = p
    return out


def test_literal_and_union_find_agree(orc):
    pos = clumps(1, [700, 300, 120, 5], debris=40)
    a = orc.groups_ref(pos)
    b = orc.groups_uf(pos)
    assert np.array_equal(a, b)
    # a group is named by its smallest member
    for g in np.unique(a):
        assert g == np.flatnonzero(a == g).min()
    em = orc.earth_moon_ref(a, [100, 200, 600])
    assert em["n_earth"] == 700 and em["n_moon"] == 300
    assert em["n_groups"] == 4 + 40
    assert sum(em["earth_counts"]) == 700 and sum(em["moon_counts"]) == 300


def test_touch_threshold_is_strict(orc):
    # two bodies exactly 1.5 apart do not touch; a hair closer they do
    pos = np.zeros((3, 4), np.float32)
    pos[1, 0] = 1.5
    pos[2, 0] = np.nextafter(np.float32(-1.5), np.float32(0))
    g = orc.groups_ref(pos)
    assert g.tolist() == [0, 1, 0]
    assert np.array_equal(orc.groups_uf(pos), g)


def test_ties_pick_the_smallest_group_number(orc):
    pos = clumps(2, [50, 50, 50])
    g = orc.groups_ref(pos)
    em = orc.earth_moon_ref(g, [0, 0, 0])
    names = sorted(set(g.tolist()))
    assert em["earth"] == names[0] and em["moon"] == names[1]
    assert em["n_earth"] == em["n_moon"] == 50


def test_single_group_has_no_moon(orc):
    pos = clumps(3, [64])
    em = orc.earth_moon_ref(orc.groups_ref(pos), [10, 20, 30])
    assert em["earth"] == 0 and em["moon"] == -1 and em["n_moon"] == 0
    assert em["moon_counts"] == [0, 0, 0, 0]


@pytest.mark.parametrize("seed", [5, 6])
def test_chains_and_random_gas(orc, seed):
    """Random gas near the percolation density: long, branched groups."""
    rng = np.random.default_rng(seed)
    n = 2500
    pos = np.zeros((n, 4), np.float32)
    pos[:, :3] = rng.uniform(0, 23.0, size=(n, 3))
    a = orc.groups_ref(pos)
    assert np.array_equal(a, orc.groups_uf(pos))
    assert len(np.unique(a)) > 1
