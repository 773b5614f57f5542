"""Generate golden vectors from the reference's own CUDA kernels.

Runs on a GB300 with oracle/_ref/libgiref.so built (the reference kernels cut
from Code/ImpactCode/impactAddTime.cu:245-394 and
Code/GenerateTargetImpactorCode/generateTargetImpactor.cu:486-664).  Inputs are
seeded; for every case the inputs, the pair table, the reference force and
the state after one reference kick-drift are saved to tests/golden/ref_*.npz.

    python tests/golden/make_golden.py [outdir]
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "tests"))

import oracle as orc  # noqa: E402
from conftest import load_gi, reference_unit_params  # noqa: E402


def main(outdir: str) -> None:
    import torch
    gi = load_gi()
    ref = orc.ref_lib()
    assert ref is not None, "oracle/_ref/libgiref.so is not built"
    os.makedirs(outdir, exist_ok=True)
    p = reference_unit_params(gi)  # the reference hard-codes m_Si = 1
    mu = 0.4
    dt = 1e-3 * mu ** 0.5
    cases = []
    # 1. contact-rich lattice, random velocities: every band and both K / KR
    pos, vel, nfe = gi.ic_lattice(101, 512, spacing=0.999, jitter=0.004, vel_sigma=2.0, nfe=170,
                                  mass_fe=p.MassFe, mass_si=p.MassSi)
    cases.append(("collision_lattice512", pos, vel, nfe))
    # 2. a config-1-like random ball (overlaps of every depth), random velocities
    pos, vel, nfe = gi.ic_uniform_ball(102, 1024, 20.0 * (1024 / 8192) ** (1 / 3), 0.3, p.MassFe,
                                       p.MassSi, 0.0, 1.0)
    rng = np.random.default_rng(102)
    vel[:, :3] = rng.normal(scale=1.5, size=(1024, 3)).astype(np.float32)
    cases.append(("collision_ball1024", pos, vel, nfe))
    # 3. tighter lattice: deep shells, Fe-Fe and Fe-Si heavy
    pos, vel, nfe = gi.ic_lattice(103, 768, spacing=0.9975, jitter=0.003, vel_sigma=3.0, nfe=400,
                                  mass_fe=p.MassFe, mass_si=p.MassSi)
    cases.append(("collision_lattice768", pos, vel, nfe))

    s = torch.cuda.current_stream().cuda_stream
    for name, pos, vel, nfe in cases:
        n = len(pos)
        fc = gi.collision_consts(p, nfe)
        mc = gi.MoveCollisionConsts(dt, dt / p.MassFe, dt / p.MassSi, nfe)
        dp = torch.from_numpy(pos).cuda()
        dv = torch.from_numpy(vel).cuda()
        df = torch.full_like(dp, float("nan"))
        assert ref.giref_forces_collision(dp.data_ptr(), dv.data_ptr(), df.data_ptr(),
                                          C.byref(fc), n, s) == 0
        torch.cuda.synchronize()
        force = df.cpu().numpy()
        assert ref.giref_move_collision(dp.data_ptr(), dv.data_ptr(), df.data_ptr(), C.byref(mc),
                                        n, s) == 0
        torch.cuda.synchronize()
        runs = np.array([[0, n, nfe, 0, dt, dt / p.MassFe, dt / p.MassSi, 0.0]], np.float64)
        save(outdir, name, "collision", pos, vel, force, dp.cpu().numpy(), dv.cpu().numpy(), runs,
             p)

    # 4. two separate bodies (settle kernel), damped move
    pa, va, fa = gi.ic_lattice(104, 384, spacing=0.999, jitter=0.004, vel_sigma=1.5, nfe=128,
                               mass_fe=p.MassFe, mass_si=p.MassSi)
    pb, vb, fb = gi.ic_lattice(105, 128, spacing=0.999, jitter=0.004, vel_sigma=1.5, nfe=40,
                               mass_fe=p.MassFe, mass_si=p.MassSi)
    pb[:, 0] += 2.5  # interpenetrating in space; only the body split keeps them apart
    pos = np.concatenate([pa, pb])
    vel = np.concatenate([va, vb])
    b1, b2, b3 = fa, 384, 384 + fb
    n = 512
    sc = gi.separate_consts(p, b1, b2, b3)
    ms = gi.MoveSeparateConsts(dt, dt / p.MassFe, dt / p.MassSi, b1, b2, b3)
    dp = torch.from_numpy(pos).cuda()
    dv = torch.from_numpy(vel).cuda()
    df = torch.full_like(dp, float("nan"))
    assert ref.giref_forces_separate(dp.data_ptr(), dv.data_ptr(), df.data_ptr(), C.byref(sc), n,
                                     s) == 0
    torch.cuda.synchronize()
    force = df.cpu().numpy()
    assert ref.giref_move_damped_separate(dp.data_ptr(), dv.data_ptr(), df.data_ptr(),
                                          C.byref(ms), 8.0, 3.0, n, s) == 0
    torch.cuda.synchronize()
    runs = np.array([[0, b2, b1, 0, dt, dt / p.MassFe, dt / p.MassSi, 8.0],
                     [b2, n - b2, b3 - b2, 0, dt, dt / p.MassFe, dt / p.MassSi, 3.0]], np.float64)
    save(outdir, "separate_two_bodies512", "separate", pos, vel, force, dp.cpu().numpy(),
         dv.cpu().numpy(), runs, p)


def save(outdir, name, kind, pos, vel, force, pos_after, vel_after, runs, p):
    extra = {f"p_{k}": np.float32(v) for k, v in p.as_dict().items()}
    # runs: offset, n, nfe, params, dt, dt/mFe, dt/mSi, damp (floats stored as float32 values)
    runs = runs.copy()
    runs[:, 4:] = runs[:, 4:].astype(np.float32)
    np.savez_compressed(os.path.join(outdir, f"ref_{name}.npz"), kind=kind, pos=pos, vel=vel,
                        force=force, pos_after=pos_after, vel_after=vel_after, runs=runs, **extra)
    print("wrote", name, pos.shape)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else HERE)
