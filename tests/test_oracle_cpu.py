"""CPU tests of the oracle: known answers of the pair law, conservation,
agreement of the two restatements, and (when present) the golden vectors
produced by the reference's own CUDA kernels."""
from __future__ import annotations

import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN, config1_params, reference_unit_params, rel_l2


def two_bodies(r, v1=(0.0, 0.0, 0.0)):
    pos = np.zeros((2, 4), np.float32)
    vel = np.zeros((2, 4), np.float32)
    pos[1, 0] = r
    vel[1, :3] = v1
    return pos, vel


def expected_mag(p, test, r, dpdv, sep_mode=0):
    """Pair law (impactAddTime.cu:298-366) evaluated in float64."""
    G = [p.GMassSiSi, p.GMassFeSi, p.GMassFeFe][test]
    K = [p.KSiSi, p.KFeSi, p.KFeFe][test]
    sep = (dpdv > 0) if sep_mode == 1 else (dpdv >= 1.0)
    if r >= 1.0:
        return G / r**2
    if test == 0:
        if r >= p.ShellBreakSi:
            return G - K * (1 - r * r)
        return G - (p.KRSiSi if sep else K) * (1 - r * r)
    if test == 2:
        if r >= p.ShellBreakFe:
            return G - K * (1 - r * r)
        return G - (p.KRFeFe if sep else K) * (1 - r * r)
    if r >= p.ShellBreakFeSi1:
        return G - K * (1 - r * r)
    if r >= p.ShellBreakFeSi2:
        return G - (p.KRMix if sep else K) * (1 - r * r)
    return G - (p.KRFeSi if sep else K) * (1 - r * r)


CASES = [
    # (r, v1x, nfe, test)
    (2.0, 0.0, 0, 0),        # Si-Si gravity
    (0.9995, 0.0, 0, 0),     # Si-Si full-K band
    (0.99, 0.5, 0, 0),       # Si-Si shell, dp.dv = 0.495 < 1: K (reference int test)
    (0.99, 2.0, 0, 0),       # Si-Si shell, dp.dv = 1.98: KR
    (3.0, 0.0, 1, 1),        # Fe-Si gravity
    (0.9995, 2.0, 1, 1),     # Fe-Si outer band: K
    (0.9985, 2.0, 1, 1),     # Fe-Si middle band separating: KRMix
    (0.9985, 0.1, 1, 1),     # Fe-Si middle band approaching: K
    (0.99, 2.0, 1, 1),       # Fe-Si inner, separating: KRFeSi
    (1.5, 0.0, 2, 2),        # Fe-Fe gravity
    (0.9985, 0.0, 2, 2),     # Fe-Fe band
    (0.99, 3.0, 2, 2),       # Fe-Fe shell, separating: KR
]


@pytest.mark.parametrize("r,v1x,nfe,test", CASES)
@pytest.mark.parametrize("which", ["config1", "reference_units"])
def test_two_body_known_answers(gi, orc, r, v1x, nfe, test, which):
    p = config1_params(gi) if which == "config1" else reference_unit_params(gi)
    pos, vel = two_bodies(r, (v1x, 0.0, 0.0))
    runs = [(0, 2, nfe, 0, 0.0, 0.0, 0.0, 0.0)]
    rr = float(np.float32(r))
    dpdv = rr * float(np.float32(v1x))
    want = expected_mag(p, test, rr, dpdv)
    f64, absf = orc.forces_fp64(pos, vel, runs, p)
    assert f64[0, 0] == pytest.approx(want, rel=1e-12, abs=1e-15)
    assert f64[1, 0] == pytest.approx(-want, rel=1e-12, abs=1e-15)
    assert np.all(f64[:, 1:] == 0.0)
    assert absf[0] == pytest.approx(abs(want), rel=1e-12)
    f32 = orc.forces_ref(pos, vel, runs, p)
    assert f32[0, 0] == pytest.approx(want, rel=2e-6, abs=1e-6)
    assert f32[1, 0] == pytest.approx(-want, rel=2e-6, abs=1e-6)


def test_separation_test_modes(gi, orc):
    """dp.dv in (0, 1): the reference's int truncation keeps K, the sign
    test switches to KR (impactAddTime.cu:313-315)."""
    p = config1_params(gi)
    pos, vel = two_bodies(0.99, (0.5, 0.0, 0.0))
    runs = [(0, 2, 0, 0, 0.0, 0.0, 0.0, 0.0)]
    ref_int, _ = orc.forces_fp64(pos, vel, runs, p, sep_test=orc.SEP_REF_INT)
    sign, _ = orc.forces_fp64(pos, vel, runs, p, sep_test=orc.SEP_SIGN)
    rr = float(np.float32(0.99))
    assert ref_int[0, 0] == pytest.approx(expected_mag(p, 0, rr, 0.495, 0), rel=1e-12)
    assert sign[0, 0] == pytest.approx(expected_mag(p, 0, rr, 0.495, 1), rel=1e-12)
    assert ref_int[0, 0] != sign[0, 0]


def test_self_pair_and_single_body(gi, orc):
    p = config1_params(gi)
    pos = np.array([[1.0, 2.0, 3.0, 0.0]], np.float32)
    vel = np.zeros((1, 4), np.float32)
    f = orc.forces_ref(pos, vel, [(0, 1, 0, 0, 0, 0, 0, 0)], p)
    assert np.all(f[0, :3] == 0.0)
    f64, _ = orc.forces_fp64(pos, vel, [(0, 1, 0, 0, 0, 0, 0, 0)], p)
    assert np.all(f64 == 0.0)


def ball(gi, n=2000, seed=7):
    pos, vel, nfe = gi.ic_uniform_ball(seed, n, radius=20.0 * (n / 8192.0) ** (1 / 3))
    return pos, vel, nfe


def test_momentum_conservation(gi, orc):
    """Pair forces are antisymmetric (same band, class and dp.dv both ways),
    so the FP64 net force vanishes to round-off."""
    p = config1_params(gi)
    pos, vel, nfe = gi.ic_lattice(3, 512, spacing=0.999, jitter=0.004, vel_sigma=1.0)
    runs = [(0, 512, nfe, 0, 0, 0, 0, 0)]
    f64, absf = orc.forces_fp64(pos, vel, runs, p)
    assert np.abs(f64.sum(0)).max() < 1e-9 * absf.sum()


def test_ref_exact_vs_fp64(gi, orc):
    p = config1_params(gi)
    pos, vel, nfe = ball(gi)
    runs = [(0, len(pos), nfe, 0, 0, 0, 0, 0)]
    f32 = orc.forces_ref(pos, vel, runs, p)
    f64, _ = orc.forces_fp64(pos, vel, runs, p)
    assert rel_l2(f32[:, :3], f64) < 1e-5


def test_subset_matches_full(gi, orc):
    p = config1_params(gi)
    pos, vel, nfe = gi.ic_lattice(5, 729, vel_sigma=1.5)
    runs = [(0, 729, nfe, 0, 0, 0, 0, 0)]
    full = orc.forces_ref(pos, vel, runs, p)
    idx = np.array([0, 5, 100, 728, nfe, nfe - 1], np.int32)
    sub = orc.forces_ref_subset(pos, vel, idx, runs, p)
    assert np.array_equal(sub[:, :3], full[idx, :3])
    f64, _ = orc.forces_fp64(pos, vel, runs, p)
    s64, _ = orc.forces_fp64(pos, vel, runs, p, idx=idx)
    assert np.array_equal(s64, f64[idx])


def test_separate_runs_skip_cross_pairs(gi, orc):
    """Two copies of a body far apart but listed as separate runs give the
    same forces as each alone (generateTargetImpactor.cu:529)."""
    p = config1_params(gi)
    pos, vel, nfe = gi.ic_lattice(11, 300, vel_sigma=1.0)
    pos2 = pos.copy()
    pos2[:, 0] += 3.0  # overlapping in space: only run separation keeps them apart
    both_p = np.concatenate([pos, pos2])
    both_v = np.concatenate([vel, vel])
    runs = [(0, 300, nfe, 0, 0, 0, 0, 0), (300, 300, nfe, 0, 0, 0, 0, 0)]
    f = orc.forces_ref(both_p, both_v, runs, p)
    alone = orc.forces_ref(pos, vel, [(0, 300, nfe, 0, 0, 0, 0, 0)], p)
    assert np.array_equal(f[:300, :3], alone[:, :3])
    alone2 = orc.forces_ref(pos2, vel, [(0, 300, nfe, 0, 0, 0, 0, 0)], p)
    assert np.array_equal(f[300:, :3], alone2[:, :3])


def test_move_matches_numpy(orc):
    rng = np.random.default_rng(0)
    pos = rng.normal(size=(100, 4)).astype(np.float32)
    vel = rng.normal(size=(100, 4)).astype(np.float32)
    force = rng.normal(size=(100, 4)).astype(np.float32)
    run = (0, 100, 30, 0, 1e-3, 1e-3 / 2.5, 1e-3, 0.0)
    p2, v2 = orc.move_ref(pos, vel, force, [run])
    dtm = np.where(np.arange(100) < 30, np.float32(1e-3 / 2.5), np.float32(1e-3)).astype(np.float32)
    v_want = (vel[:, :3].astype(np.float64) + force[:, :3] * dtm[:, None].astype(np.float64))
    assert np.allclose(v2[:, :3], v_want, rtol=1e-6, atol=1e-7)
    assert np.array_equal(v2[:, 3], vel[:, 3]) and np.array_equal(p2[:, 3], pos[:, 3])
    assert np.allclose(p2[:, :3], pos[:, :3] + v2[:, :3].astype(np.float64) * 1e-3, rtol=1e-6,
                       atol=1e-7)


def test_r2_threshold(orc):
    for s in [0.999, 0.998, 0.9995, 1.0, 0.5, 0.123456]:
        t = np.float32(orc.r2_threshold(s))
        s32 = np.float32(s)
        assert np.sqrt(t) >= s32
        assert np.sqrt(np.nextafter(t, np.float32(0))) < s32
    assert orc.r2_threshold(1.0) == 1.0


def test_potential_gradient_is_force(gi, orc):
    """With no separating pairs (v = 0) the law is conservative: the FP64
    force equals -dU/dx of the FP64 potential (central differences)."""
    p = config1_params(gi)
    pos, vel, nfe = gi.ic_lattice(13, 64, spacing=0.99, jitter=0.01, vel_sigma=0.0)
    runs = [(0, 64, nfe, 0, 0, 0, 0, 0)]
    f64, _ = orc.forces_fp64(pos, vel, runs, p)
    i = 21
    h = 2.0 ** -16  # small enough not to straddle the r = 1 kink of U
    grad = []
    for a in range(3):
        pp, pm = pos.copy(), pos.copy()
        pp[i, a] += h
        pm[i, a] -= h
        up = orc.potential_fp64(pp, runs, p).sum() / 2
        um = orc.potential_fp64(pm, runs, p).sum() / 2
        grad.append(-(up - um) / (float(pp[i, a]) - float(pm[i, a])))
    assert np.allclose(grad, f64[i], rtol=1e-4, atol=1e-5 * np.abs(f64[i]).max())


def test_diag_simple(gi, orc):
    p = config1_params(gi)
    pos = np.array([[1, 0, 0, 0], [-1, 0, 0, 0], [0, 2, 0, 0]], np.float32)
    vel = np.array([[0, 1, 0, 0], [0, -1, 0, 0], [0, 0, 0, 0]], np.float32)
    run = (0, 3, 2, 0, 0, 0, 0, 0)
    d = orc.diag_fp64(pos, vel, run, p)
    m = 1.0 + 1.0 + float(np.float32(0.4))
    assert d[0] == pytest.approx(m)
    assert d[2] == pytest.approx(0.8 / m)
    # L_z about the com: two Fe bodies counter-moving at +-1 around the x axis
    cy = 0.8 / m
    lz = (1 * 1 - (0 - cy) * 0) + (-1 * -1 - (0 - cy) * 0)
    assert d[9] == pytest.approx(lz)
    assert d[10] == pytest.approx(1.0)
    assert d[14] == 3


def test_flip_counter_runs(gi, orc):
    p = config1_params(gi)
    pos, vel, nfe = gi.ic_lattice(17, 512, spacing=0.9985, jitter=0.002, vel_sigma=1.0)
    runs = [(0, 512, nfe, 0, 0, 0, 0, 0)]
    bf, sf = orc.count_flips(pos, vel, np.arange(512), runs, p)
    assert bf >= 0 and sf >= 0


# ------------------------------------------------------------ golden vectors --

GOLDEN_FILES = sorted(glob.glob(os.path.join(GOLDEN, "ref_*.npz")))


@pytest.mark.skipif(not GOLDEN_FILES, reason="no golden vectors committed")
@pytest.mark.parametrize("path", GOLDEN_FILES, ids=[os.path.basename(p) for p in GOLDEN_FILES])
def test_oracle_matches_reference_golden(orc, path):
    """The ref-exact oracle reproduces the reference's own CUDA kernels
    (run on a GB300, outputs committed) bit for bit."""
    g = np.load(path)
    kind = str(g["kind"])
    params = {k[2:]: float(g[k]) for k in g.files if k.startswith("p_")}
    runs = [tuple(int(x) if i < 4 else float(x) for i, x in enumerate(r)) for r in g["runs"]]
    if kind in ("collision", "separate"):
        f = orc.forces_ref(g["pos"], g["vel"], runs, params)
        mism = np.argwhere(f[:, :3] != g["force"][:, :3])
        assert len(mism) == 0, f"{len(mism)} mismatching components, first {mism[:5]}"
    if "pos_after" in g.files:
        force = g["force"]
        p2, v2 = orc.move_ref(g["pos"], g["vel"], force, runs)
        assert np.array_equal(v2, g["vel_after"])
        assert np.array_equal(p2, g["pos_after"])


def test_material_params_match_library(gi, orc):
    """The oracle's own pair table (used where the library must not load)
    equals gi_params_from_material field for field, both orders of the
    shell depths."""
    for sd in ((0.002, 0.001), (0.001, 0.002)):
        a = orc.material_params(1.0, 1.0, 1.0, 0.4, 5.0, 1.5, 0.02, 0.01, *sd)
        b = gi.params_from_material(1.0, 1.0, 1.0, 0.4, 5.0, 1.5, 0.02, 0.01, *sd)
        for name in orc.PARAM_FIELDS:
            assert np.float32(a[name]) == np.float32(getattr(b, name)), name


def test_integrate_fp64_first_step_and_invariants(gi, orc):
    """One step of the FP64 integrator is the FP64 force (double predicates)
    followed by the double kick-drift; its log holds E = KE + PE, L and P of
    the state; momentum is conserved (the law is antisymmetric pair by pair)
    and, with KR = K, energy is conserved to the integrator's order."""
    pos, vel, nfe = gi.ic_lattice(17, 600, spacing=0.97, jitter=0.01, vel_sigma=0.8)
    p = config1_params(gi)
    run = [(0, 600, nfe, 0, 0, 0, 0, 0)]
    dt = 1e-3
    X, V, log = orc.integrate_fp64(pos, vel, nfe, p, dt, 1, 1)
    f64, _ = orc.forces_fp64(pos, vel, run, p, branch=orc.BRANCH_F64)
    m = np.where(np.arange(600) < nfe, p.MassFe, p.MassSi).astype(np.float64)[:, None]
    v1 = vel[:, :3].astype(np.float64) + f64 * dt / m
    x1 = pos[:, :3].astype(np.float64) + v1 * dt
    assert np.allclose(V, v1, rtol=1e-13, atol=1e-15)
    assert np.allclose(X, x1, rtol=1e-15, atol=1e-13)
    d = orc.diag_fp64(pos, vel, run[0], p)
    pe = orc.potential_fp64(pos, run, p).sum() / 2.0
    assert abs(log[0, 0] - (d[10] + pe)) <= 1e-12 * abs(log[0, 0])
    assert np.allclose(log[0, 4:7], d[11:14], rtol=1e-12, atol=1e-12)
    # conservative control (KR = K): 200 steps
    q = gi.params_from_material(1.0, 1.0, 1.0, 0.4, 5.0, 1.5, 1.0, 1.0, 0.002, 0.001)
    _, _, lg = orc.integrate_fp64(pos, vel, nfe, q, dt, 200, 50)
    scale = np.abs(m[:, 0] * vel[:, :3].astype(np.float64).T).sum()
    assert np.abs(lg[:, 4:7] - lg[0, 4:7]).max() <= 1e-11 * scale
    assert np.abs(lg[:, 0] - lg[0, 0]).max() <= 1e-3 * abs(lg[0, 0])
