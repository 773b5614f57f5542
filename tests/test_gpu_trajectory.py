"""Trajectories and the hard force case against the FP64 oracle.

  * The 8,192-body settle workload stepped 1,000 times through the library's
    fused step, against (a) the FP64 oracle integrated with the same
    kick-drift in double and (b) the reference's own kernels
    (getForcesCollisionSingleGPU + moveBodiesCollisionSingleGPU,
    impactAddTime.cu:245-394) stepped 1,000 times on the same input.  Max
    position deviation and FP64 energy / angular-momentum drift of all three
    are printed and bounded.
  * Interpenetrating bodies, where a body's contact terms cancel
    (sum_j |f_ij| >> |F_i|): the force error against the FP64 oracle with
    the reference's FP32 branch decisions, and the branch flips between FP32
    and FP64 decisions reported beside the error with FP64 decisions.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

FORCE_TOL = 1e-5


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _energy_l(orc, pos, vel, run, p):
    """FP64 E (KE + pair potential) and L = sum m x cross v of a float state."""
    d = orc.diag_fp64(pos, vel, run, p)
    pe = orc.potential_fp64(pos, [run], p).sum() / 2.0
    M, c, u = d[0], d[1:4], d[4:7]
    L = d[7:10] + M * np.cross(c, u)
    return d[10] + pe, L


def _drift(log):
    E0, L0 = log[0][0], np.asarray(log[0][1])
    dE = max(abs(e - E0) / abs(E0) for e, _ in log)
    dL = max(float(np.linalg.norm(np.asarray(l) - L0)) for _, l in log)
    return dE, dL


def test_config1_trajectory_against_fp64_and_reference(gi, orc, torch_cuda):
    """All three run in the reference's units (m_Si = 1: masses / 0.4, K /
    0.4^2, dt x sqrt(0.4), velocities / sqrt(0.4)), because its separation
    test, int inout = dp.dv, is not unit-free: in other units the three
    paths would not make the same K / KR decisions."""
    torch = torch_cuda
    import gi_workloads as wl
    steps, every = 1000, 100
    pos0, vel0, nfe = wl.config1(gi)
    n = len(pos0)
    mu = wl.MATERIAL["mass_si"]
    p = gi.params_from_material(1.0, 1.0, 1.0 / mu, 1.0, 5.0 / mu**2, 1.5 / mu**2, 0.02, 0.01,
                                0.002, 0.001)
    dt = 1e-3 * mu ** 0.5
    vel0 = vel0 * np.float32([mu ** -0.5] * 3 + [1.0])  # at rest: zero either way
    run = gi.Run(0, n, nfe, 0, dt, dt / p.MassFe, dt / p.MassSi, 0.0)
    orun = (0, n, nfe, 0, 0, 0, 0, 0)
    # ---- this library: fused force + kick-drift steps
    ctx = gi.Context(0)
    dp, dv = _dev(torch, pos0), _dev(torch, vel0)
    ours, ours_log = [], []
    for k in range(0, steps + 1, every):
        if k:
            ctx.step(dp.data_ptr(), dv.data_ptr(), [run], p, every)
            torch.cuda.synchronize()
        P, V = dp.cpu().numpy(), dv.cpu().numpy()
        ours.append(P[:, :3].astype(np.float64))
        ours_log.append(_energy_l(orc, P, V, orun, p))
    ctx.close()
    # ---- the reference's kernels on the same input
    ref = orc.ref_lib()
    assert ref is not None, "reference kernels not built"
    fc = gi.collision_consts(p, nfe)
    mc = gi.MoveCollisionConsts(dt, dt / p.MassFe, dt / p.MassSi, nfe)
    rpos, rvel = _dev(torch, pos0), _dev(torch, vel0)
    rfor = torch.zeros_like(rpos)
    s = torch.cuda.current_stream().cuda_stream
    refs, ref_log = [], []
    for k in range(0, steps + 1, every):
        if k:
            for _ in range(every):
                assert ref.giref_forces_collision(rpos.data_ptr(), rvel.data_ptr(),
                                                  rfor.data_ptr(), C.byref(fc), n, s) == 0
                assert ref.giref_move_collision(rpos.data_ptr(), rvel.data_ptr(),
                                                rfor.data_ptr(), C.byref(mc), n, s) == 0
            torch.cuda.synchronize()
        P, V = rpos.cpu().numpy(), rvel.cpu().numpy()
        refs.append(P[:, :3].astype(np.float64))
        ref_log.append(_energy_l(orc, P, V, orun, p))
    # ---- FP64 oracle trajectory (double state, double branch decisions), in
    # pieces of `every` steps so that the positions at the record points are
    # kept; each piece logs E, L, P at its start and end
    f64 = [pos0[:, :3].astype(np.float64)]
    f64_log = []
    Xk, Vk = pos0, vel0
    for k in range(every, steps + 1, every):
        Xk, Vk, lg = orc.integrate_fp64(Xk, Vk, nfe, p, dt, every, every)
        if not f64_log:
            f64_log.append((lg[0, 0], lg[0, 1:4]))
        f64_log.append((lg[1, 0], lg[1, 1:4]))
        f64.append(Xk.copy())

    def maxdev(a, b):
        return [float(np.abs(x - y).max()) for x, y in zip(a, b)]

    d_ours, d_ref, d_or = maxdev(ours, f64), maxdev(refs, f64), maxdev(ours, refs)
    dE_o, dL_o = _drift(ours_log)
    dE_r, dL_r = _drift(ref_log)
    dE_f, dL_f = _drift(f64_log)
    print(f"\nmax |dx| vs FP64 every {every} steps:\n  ours      {np.array(d_ours)}\n"
          f"  reference {np.array(d_ref)}\n  ours vs reference {np.array(d_or)}")
    print(f"FP64 drift over {steps} steps: max |dE|/|E0| ours {dE_o:.3e}, reference {dE_r:.3e}, "
          f"FP64 oracle {dE_f:.3e}; max |dL| ours {dL_o:.3e}, reference {dL_r:.3e}, "
          f"FP64 oracle {dL_f:.3e}")
    # Every body stays within a small fraction of a diameter of the FP64
    # trajectory, and no farther than the reference path's own trajectory.
    assert d_ours[-1] < 1e-2
    assert d_ours[-1] <= max(2.0 * d_ref[-1], 1e-4)
    # Energy: the integrator's error is the same on every path (dt-limited).
    assert dE_o <= max(2.0 * dE_r, 2.0 * dE_f) + 1e-9
    # Angular momentum: no force of the law changes it, and the bodies start
    # at rest, so any |dL| is numerical.
    assert dL_o <= max(2.0 * dL_r, 1e-5)


def _overlapping_balls(seed, n_each, radius, sep, vscale):
    """Two uniform balls of n_each bodies (inner 30 % by radius Fe), centres
    `sep` apart, random velocities."""
    rng = np.random.default_rng(seed)
    parts = []
    for k in range(2):
        d = rng.normal(size=(n_each, 3))
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        r = radius * rng.uniform(0, 1, size=(n_each, 1)) ** (1 / 3)
        x = d * r
        x[:, 0] += (k - 0.5) * sep
        parts.append((x, r[:, 0] < 0.3 * radius))
    fe = np.concatenate([parts[0][0][parts[0][1]], parts[1][0][parts[1][1]]])
    si = np.concatenate([parts[0][0][~parts[0][1]], parts[1][0][~parts[1][1]]])
    pos = np.zeros((2 * n_each, 4), np.float32)
    pos[:, :3] = np.concatenate([fe, si])
    vel = np.zeros_like(pos)
    vel[:, :3] = rng.normal(scale=vscale, size=(2 * n_each, 3))
    nfe = len(fe)
    vel[:nfe, 3], vel[nfe:, 3] = 1.0, 0.4
    return pos, vel, nfe


def test_interpenetrating_bodies_force_error_and_flips(gi, orc, torch_cuda):
    """Two config-1 balls of 8,192 bodies each, compressed to radius 1.5 and
    overlapping (centres 1 apart), with random velocities so that the KR
    branch fires: thousands of contacts per body whose terms largely cancel.
    Bar: global relative L2 <= 1e-5 against the FP64 oracle with the
    reference's FP32 branch decisions.  Flips between FP32 and FP64
    decisions are counted and reported with the error against FP64
    decisions, and the reference kernel's error on the same state beside
    it (in its own units)."""
    torch = torch_cuda
    import gi_workloads as wl
    pos, vel, nfe = _overlapping_balls(41, 8192, 1.5, 1.0, 1.5)
    n = len(pos)
    p = wl.params(gi)
    run = wl.run_desc(gi, 0, n, nfe)
    orun = [(0, n, nfe, 0, 0, 0, 0, 0)]
    ctx = gi.Context(0)
    dp, dv = _dev(torch, pos), _dev(torch, vel)
    df = torch.full_like(dp, float("nan"))
    ctx.forces(dp.data_ptr(), dv.data_ptr(), df.data_ptr(), [run], p)
    torch.cuda.synchronize()
    f = df.cpu().numpy()[:, :3].astype(np.float64)
    ctx.close()
    idx = np.sort(np.random.default_rng(5).choice(n, 4096, replace=False)).astype(np.int32)
    f64, absf = orc.forces_fp64(pos, vel, orun, p, idx=idx, branch=orc.BRANCH_F32)
    f64d, _ = orc.forces_fp64(pos, vel, orun, p, idx=idx, branch=orc.BRANCH_F64)
    band_flips, sep_flips = orc.count_flips(pos, vel, idx, orun, p)
    contacts = 0
    for c0 in range(0, len(idx), 256):
        xi = pos[idx[c0:c0 + 256], None, :3].astype(np.float64)
        contacts += int((((xi - pos[None, :, :3]) ** 2).sum(-1) < 1.0).sum())
    contacts -= len(idx)  # the self pairs
    err = rel_l2(f[idx], f64)
    err_d = rel_l2(f[idx], f64d)
    cancel = float(np.median(absf / np.maximum(np.linalg.norm(f64, axis=1), 1e-300)))
    # the reference's kernel, in its own units (m_Si = 1), against the FP64
    # oracle in the same units (its int dp.dv separation test is not unit-free)
    mu = p.MassSi
    rp = gi.params_from_material(1.0, 1.0, p.MassFe / mu, 1.0, 5.0 / mu**2, 1.5 / mu**2, 0.02,
                                 0.01, 0.002, 0.001)
    ref = orc.ref_lib()
    rerr = None
    if ref is not None:
        rf = torch.zeros_like(dp)
        rvel = vel * np.float32([mu ** -0.5] * 3 + [1.0])
        rv = _dev(torch, rvel)
        assert ref.giref_forces_collision(dp.data_ptr(), rv.data_ptr(), rf.data_ptr(),
                                          C.byref(gi.collision_consts(rp, nfe)), n,
                                          torch.cuda.current_stream().cuda_stream) == 0
        torch.cuda.synchronize()
        r64, _ = orc.forces_fp64(pos, rvel, orun, rp, idx=idx, branch=orc.BRANCH_F32)
        rerr = rel_l2(rf.cpu().numpy()[idx, :3].astype(np.float64), r64)
    print(f"\ninterpenetrating {n} bodies: {contacts / len(idx):.0f} contacts per body, median "
          f"sum|f_ij| / |F| {cancel:.1f}; rel L2 vs FP64 (FP32 decisions) {err:.3e}, vs FP64 "
          f"(FP64 decisions) {err_d:.3e}; flips over {len(idx)} x {n} pairs: band {band_flips}, "
          f"separation {sep_flips}; reference kernel vs FP64 {rerr}")
    assert contacts / len(idx) > 1000 and cancel > 5
    assert err < FORCE_TOL
