"""Seeded synthetic workloads with the shapes of the Giant-Impact runs.

  config1(...)   8,192 bodies uniform in a ball of radius 20 D, inner 30 % by
                 radius Fe; mFe = 1, mSi = 0.4, KFe = 5, KSi = 1.5,
                 KR 0.02 / 0.01, shell depth 0.002 / 0.001 D; v = 0; dt = 1e-3.
  sweep(...)     a parameter sweep of many impacts packed into one array (one
                 run per impact): target N log-uniform in [4,096, 131,072],
                 impactor 0.1 x target, angle U[0, 60] deg, speed U[1.0, 1.5]
                 x escape, spin U[0, 0.8] x breakup; bodies settled together
                 in one batched damped step call.
  precision_impact(...)  1,048,576-body target + 104,858-body impactor,
                 each a config-1 ball scaled to the same density (radius
                 20 (N / 8192)^(1/3) D), not settled, spun, placed and
                 moving as in impact().
  impact(...)    two-body impact: target (60,000) and impactor (6,000), each
                 built as a seeded ball and settled on the GPU with the damped
                 separate-body step (the reference's generate-target-impactor
                 damping phase, generateTargetImpactor.cu:666-749), spun about
                 z at a fraction of breakup, placed at 45 degrees and moving at
                 1.2 x the mutual escape speed, reordered [Fe1, Fe2, Si1, Si2]
                 (impactInitialization.cu:329-371).
Code units: G = 1, particle diameter D = 1.
"""
from __future__ import annotations

import math

import numpy as np

MATERIAL = dict(G=1.0, diameter=1.0, mass_fe=1.0, mass_si=0.4, k_fe=5.0, k_si=1.5, kr_fe=0.02,
                kr_si=0.01, sd_fe=0.002, sd_si=0.001)
DT = 1e-3


def params(gi):
    m = MATERIAL
    return gi.params_from_material(m["G"], m["diameter"], m["mass_fe"], m["mass_si"], m["k_fe"],
                                   m["k_si"], m["kr_fe"], m["kr_si"], m["sd_fe"], m["sd_si"])


def run_desc(gi, offset, n, nfe, damp=0.0, dt=DT):
    m = MATERIAL
    return gi.Run(offset, n, nfe, 0, dt, dt / m["mass_fe"], dt / m["mass_si"], damp)


def config1(gi, seed=1, n=8192, radius=20.0):
    pos, vel, nfe = gi.ic_uniform_ball(seed, n, radius, 0.3, MATERIAL["mass_fe"],
                                       MATERIAL["mass_si"], 0.0, 1.0)
    return pos, vel, nfe


def body_mass(n, nfe):
    return nfe * MATERIAL["mass_fe"] + (n - nfe) * MATERIAL["mass_si"]


def raw_body(gi, seed, n, tag_fe, tag_si):
    """Seeded ball at ~50 % volume fraction, Fe inner 30 % by radius."""
    radius = (n / 4.0) ** (1.0 / 3.0)
    return gi.ic_uniform_ball(seed, n, radius, 0.3, MATERIAL["mass_fe"], MATERIAL["mass_si"],
                              tag_fe, tag_si)


def settle_pair(gi, torch, n_t, n_i, seed=2, steps=1500, damp=8.0, ctx=None):
    """Build and settle target and impactor together on the GPU (separate
    runs: no cross-body forces), reference order [Fe1, Si1, Fe2, Si2]."""
    pt, vt, fet = raw_body(gi, seed, n_t, 0.0, 1.0)
    pi, vi, fei = raw_body(gi, seed + 1000, n_i, 2.0, 3.0)
    pos = np.concatenate([pt, pi])
    vel = np.concatenate([vt, vi])
    own = ctx is None
    if own:
        ctx = gi.Context(0)
    p = params(gi)
    runs = [run_desc(gi, 0, n_t, fet, damp), run_desc(gi, n_t, n_i, fei, damp)]
    dp = torch.from_numpy(pos).cuda()
    dv = torch.from_numpy(vel).cuda()
    ctx.step(dp.data_ptr(), dv.data_ptr(), runs, p, steps)
    # a short undamped rest, as in the reference's rest phase
    runs0 = [run_desc(gi, 0, n_t, fet, 0.0), run_desc(gi, n_t, n_i, fei, 0.0)]
    ctx.step(dp.data_ptr(), dv.data_ptr(), runs0, p, max(1, steps // 10))
    torch.cuda.synchronize()
    pos, vel = dp.cpu().numpy(), dv.cpu().numpy()
    if own:
        ctx.close()
    return pos, vel, fet, fei


def _com(pos, vel, n0, n, nfe):
    m = np.where(np.arange(n) < nfe, MATERIAL["mass_fe"], MATERIAL["mass_si"])
    x = pos[n0:n0 + n, :3].astype(np.float64)
    v = vel[n0:n0 + n, :3].astype(np.float64)
    M = m.sum()
    return (m[:, None] * x).sum(0) / M, (m[:, None] * v).sum(0) / M, M


def spin_and_place(pos, vel, n_t, n_i, fet, fei, spin_fraction=0.5, angle_deg=45.0,
                   speed_factor=1.2, spin_t=None, spin_i=None):
    """Zero each body's drift, spin about z, place the impactor at the given
    impact angle and speed, reorder to [Fe1, Fe2, Si1, Si2].  Returns
    (pos, vel, nfe_total)."""
    pos = pos.astype(np.float64).copy()
    vel = vel.astype(np.float64).copy()
    radii = []
    masses = []
    for (n0, n, nfe), frac in (((0, n_t, fet), spin_t if spin_t is not None else spin_fraction),
                               ((n_t, n_i, fei), spin_i if spin_i is not None else spin_fraction)):
        c, v, M = _com(pos.astype(np.float32), vel.astype(np.float32), n0, n, nfe)
        pos[n0:n0 + n, :3] -= c
        vel[n0:n0 + n, :3] -= v
        r = np.linalg.norm(pos[n0:n0 + n, :3], axis=1)
        R = float(np.percentile(r, 99.0)) + 0.5
        w = frac * math.sqrt(MATERIAL["G"] * M / R**3)
        vel[n0:n0 + n, 0] += -w * pos[n0:n0 + n, 1]
        vel[n0:n0 + n, 1] += w * pos[n0:n0 + n, 0]
        radii.append(R)
        masses.append(M)
    Rt, Ri = radii
    Mt, Mi = masses
    d = Rt + Ri
    vesc = math.sqrt(2 * MATERIAL["G"] * (Mt + Mi) / d)
    b = d * math.sin(math.radians(angle_deg))
    start = 1.25 * d
    pos[n_t:, 0] += -start
    pos[n_t:, 1] += b
    vel[n_t:, 0] += speed_factor * vesc
    # centre-of-mass frame
    M = Mt + Mi
    c_i = np.array([-start, b, 0.0])
    v_i = np.array([speed_factor * vesc, 0.0, 0.0])
    pos[:, :3] -= (Mi * c_i) / M
    vel[:, :3] -= (Mi * v_i) / M
    # reorder [Fe1, Si1, Fe2, Si2] -> [Fe1, Fe2, Si1, Si2]
    order = np.concatenate([np.arange(0, fet), np.arange(n_t, n_t + fei), np.arange(fet, n_t),
                            np.arange(n_t + fei, n_t + n_i)])
    return (pos[order].astype(np.float32), vel[order].astype(np.float32), fet + fei)


def impact(gi, torch, n_t=60000, n_i=6000, seed=2, settle_steps=1500, spin_fraction=0.5,
           angle_deg=45.0, speed_factor=1.2, ctx=None):
    pos, vel, fet, fei = settle_pair(gi, torch, n_t, n_i, seed=seed, steps=settle_steps, ctx=ctx)
    return spin_and_place(pos, vel, n_t, n_i, fet, fei, spin_fraction, angle_deg, speed_factor)


def sweep(gi, torch, nruns=64, seed=4, settle_steps=100, nmin=4096, nmax=131072, ctx=None,
          spin_max=0.8, angle_max=60.0, speed_range=(1.0, 1.5)):
    """Returns (pos, vel, runs, specs): all impacts packed back to back, one
    gi.Run per impact (material order [Fe1, Fe2, Si1, Si2] inside each)."""
    rng = np.random.default_rng(seed)
    specs = []
    for r in range(nruns):
        nt = int(round(math.exp(rng.uniform(math.log(nmin), math.log(nmax)))))
        ni = max(64, int(round(0.1 * nt)))
        specs.append(dict(n_target=nt, n_impactor=ni, angle=float(rng.uniform(0.0, angle_max)),
                          speed=float(rng.uniform(*speed_range)),
                          spin=float(rng.uniform(0.0, spin_max))))
    # raw bodies, all settled together: every body is its own run
    bodies = []
    for r, sp in enumerate(specs):
        bodies.append(raw_body(gi, seed * 100003 + 2 * r, sp["n_target"], 0.0, 1.0))
        bodies.append(raw_body(gi, seed * 100003 + 2 * r + 1, sp["n_impactor"], 2.0, 3.0))
    pos = np.concatenate([b[0] for b in bodies])
    vel = np.concatenate([b[1] for b in bodies])
    offs = np.concatenate([[0], np.cumsum([len(b[0]) for b in bodies])[:-1]]).astype(int)
    own = ctx is None
    if own:
        ctx = gi.Context(0)
    p = params(gi)
    if settle_steps > 0:
        runs = [run_desc(gi, int(o), len(b[0]), b[2], 8.0) for o, b in zip(offs, bodies)]
        dp = torch.from_numpy(pos).cuda()
        dv = torch.from_numpy(vel).cuda()
        ctx.step(dp.data_ptr(), dv.data_ptr(), runs, p, settle_steps)
        torch.cuda.synchronize()
        pos, vel = dp.cpu().numpy(), dv.cpu().numpy()
    if own:
        ctx.close()
    out_p, out_v, out_runs = [], [], []
    off = 0
    for r, sp in enumerate(specs):
        bt, bi = 2 * r, 2 * r + 1
        nt, ni = sp["n_target"], sp["n_impactor"]
        pp = np.concatenate([pos[offs[bt]:offs[bt] + nt], pos[offs[bi]:offs[bi] + ni]])
        vv = np.concatenate([vel[offs[bt]:offs[bt] + nt], vel[offs[bi]:offs[bi] + ni]])
        P, V, nfe = spin_and_place(pp, vv, nt, ni, bodies[bt][2], bodies[bi][2],
                                   spin_fraction=sp["spin"], angle_deg=sp["angle"],
                                   speed_factor=sp["speed"])
        out_p.append(P)
        out_v.append(V)
        out_runs.append(run_desc(gi, off, nt + ni, nfe))
        off += nt + ni
    return np.concatenate(out_p), np.concatenate(out_v), out_runs, specs


N3_TARGET, N3_IMPACTOR = 1_048_576, 104_858


def precision_impact(gi, seed=3, n_t=N3_TARGET, n_i=N3_IMPACTOR):
    """The large-N impact state (returns pos, vel, nfe in [Fe1, Fe2, Si1, Si2]
    order): two uniform balls at the config-1 density, spun at 0.5 of
    breakup, 45 degrees, 1.2 x the mutual escape speed."""
    m = MATERIAL
    rt = 20.0 * (n_t / 8192.0) ** (1.0 / 3.0)
    ri = 20.0 * (n_i / 8192.0) ** (1.0 / 3.0)
    pt, vt, fet = gi.ic_uniform_ball(seed, n_t, rt, 0.3, m["mass_fe"], m["mass_si"], 0.0, 1.0)
    pi, vi, fei = gi.ic_uniform_ball(seed + 1000, n_i, ri, 0.3, m["mass_fe"], m["mass_si"], 2.0,
                                     3.0)
    return spin_and_place(np.concatenate([pt, pi]), np.concatenate([vt, vi]), n_t, n_i, fet, fei)
