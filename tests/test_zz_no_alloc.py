"""gi_forces_collision_noalloc: the force pass for callers that cannot
allocate device memory (a fixed device-memory budget or pool, or a step loop
that must not stall on the device-wide synchronisation cudaMalloc can cause).
It keeps all scratch in one static device array, so it must give the same
forces as the regular drop-in gi_forces_collision, within the 1e-5 force
tolerance the other tests use, call after call: the array keeps the previous
call's contents, and a second call must not be disturbed by them.

This file is collected last so that a run stopping at the first failure has
already run every other test."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import reference_unit_params, rel_l2

pytestmark = pytest.mark.gpu

FORCE_TOL = 1e-5


def _forces(gi, torch, fn, pos, vel, consts):
    dp = torch.from_numpy(np.ascontiguousarray(pos)).cuda()
    dv = torch.from_numpy(np.ascontiguousarray(vel)).cuda()
    df = torch.full_like(dp, float("nan"))
    fn(dp.data_ptr(), dv.data_ptr(), df.data_ptr(), consts, len(pos),
       torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return df.cpu().numpy()


def test_noalloc_matches_drop_in_on_two_calls_in_a_row(gi, orc, torch_cuda):
    torch = torch_cuda
    p = reference_unit_params(gi)
    # two different inputs, called back to back: a contact-rich lattice with
    # random velocities (every band, K and KR), then a larger random ball
    lat = gi.ic_lattice(61, 20000, spacing=0.999, jitter=0.004, vel_sigma=2.0,
                        mass_fe=p.MassFe, mass_si=p.MassSi)
    ball_pos, ball_vel, ball_nfe = gi.ic_uniform_ball(62, gi.NOALLOC_MAX_BODIES,
                                                      20.0 * 4.0 ** (1 / 3), 0.3, p.MassFe,
                                                      p.MassSi, 0.0, 1.0)
    rng = np.random.default_rng(62)
    ball_vel[:, :3] = rng.normal(scale=1.5, size=(len(ball_pos), 3)).astype(np.float32)
    for pos, vel, nfe in (lat, (ball_pos, ball_vel, ball_nfe)):
        c = gi.collision_consts(p, nfe)
        mine = _forces(gi, torch, gi.forces_collision_noalloc, pos, vel, c)
        regular = _forces(gi, torch, gi.forces_collision, pos, vel, c)
        assert np.isfinite(mine[:, :3]).all()
        assert np.isnan(mine[:, 3]).all()  # .w left untouched
        err = rel_l2(mine[:, :3], regular[:, :3])
        print(f"n={len(pos)}: no-alloc vs gi_forces_collision rel L2 {err:.3e}")
        assert err < FORCE_TOL
        idx = np.arange(0, len(pos), 97)
        f64, _ = orc.forces_fp64(pos, vel, [(0, len(pos), nfe, 0, 0, 0, 0, 0)], p, idx=idx)
        assert rel_l2(mine[idx, :3], f64) < FORCE_TOL
    # a repeat of the first input after the second call left the array dirty
    c = gi.collision_consts(p, lat[2])
    again = _forces(gi, torch, gi.forces_collision_noalloc, lat[0], lat[1], c)
    first = _forces(gi, torch, gi.forces_collision, lat[0], lat[1], c)
    assert rel_l2(again[:, :3], first[:, :3]) < FORCE_TOL


def test_noalloc_refuses_more_than_its_maximum(gi, torch_cuda):
    torch = torch_cuda
    n = gi.NOALLOC_MAX_BODIES + 1
    p = reference_unit_params(gi)
    buf = torch.zeros((n, 4), device="cuda")
    with pytest.raises(gi.GIError) as e:
        gi.forces_collision_noalloc(buf.data_ptr(), buf.data_ptr(), buf.data_ptr(),
                                    gi.collision_consts(p, 0), n)
    assert e.value.status == 2
    assert "32768" in str(e.value)
