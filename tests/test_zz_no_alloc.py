"""gi_forces_collision_noalloc: the force pass for callers that cannot
allocate device memory (a fixed device-memory budget or pool, or a step loop
that must not stall on the device-wide synchronisation cudaMalloc can cause).
It keeps all scratch in one static device array and runs the regular
drop-in's kernels with the same default decomposition, so it must give the
same forces as gi_forces_collision bit for bit, call after call: the array
keeps the previous call's contents, and a second call must not be disturbed
by them.

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
        assert np.array_equal(mine[:, :3], regular[:, :3])
        idx = np.arange(0, len(pos), 97)
        f64, _ = orc.forces_fp64(pos, vel, [(0, len(pos), nfe, 0, 0, 0, 0, 0)], p, idx=idx)
        assert rel_l2(mine[idx, :3], f64) < FORCE_TOL
    # a repeat of the first input after the second call left the array dirty
    c = gi.collision_consts(p, lat[2])
    again = _forces(gi, torch, gi.forces_collision_noalloc, lat[0], lat[1], c)
    first = _forces(gi, torch, gi.forces_collision, lat[0], lat[1], c)
    assert np.array_equal(again[:, :3], first[:, :3])


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


@pytest.mark.parametrize("n", [3000, 1])
def test_noalloc_small_runs_match(gi, orc, torch_cuda, n):
    """3,000 bodies: not a multiple of the far field's 64-body j-chunk or
    1,024-body i-block, with the Fe/Si boundary inside a chunk.  n = 1 is
    the self pair alone (zero force)."""
    torch = torch_cuda
    p = reference_unit_params(gi)
    pos, vel, nfe = gi.ic_lattice(63, n, spacing=0.999, jitter=0.004, vel_sigma=2.0,
                                  nfe=n // 3, mass_fe=p.MassFe, mass_si=p.MassSi)
    c = gi.collision_consts(p, nfe)
    for _ in range(2):
        mine = _forces(gi, torch, gi.forces_collision_noalloc, pos, vel, c)
        regular = _forces(gi, torch, gi.forces_collision, pos, vel, c)
        assert np.isnan(mine[:, 3]).all()
        if n == 1:
            assert np.array_equal(mine[:, :3], np.zeros((1, 3), np.float32))
            continue
        assert np.array_equal(mine[:, :3], regular[:, :3])
        f64, _ = orc.forces_fp64(pos, vel, [(0, n, nfe, 0, 0, 0, 0, 0)], p)
        assert rel_l2(mine[:, :3], f64) < FORCE_TOL


_FRESH = r'''
# Device memory through the CUDA runtime directly (no torch: with every
# module loaded up front, torch's own kernels would take minutes to load).
import ctypes as C, glob, json, os, sys
sys.path.insert(0, sys.argv[1])
import numpy as np
import gi
gi.lib()
home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
rt = C.CDLL(sorted(glob.glob(os.path.join(home, "lib64", "libcudart.so*")))[0])

def ok(e):
    assert e == 0, f"CUDA runtime error {e}"

def free_bytes():
    f, t = C.c_size_t(), C.c_size_t()
    ok(rt.cudaMemGetInfo(C.byref(f), C.byref(t)))
    return f.value

ok(rt.cudaSetDevice(0))
p = gi.params_from_material(1.0, 1.0, 2.5, 1.0, 31.25, 9.375, 0.02, 0.01, 0.002, 0.001)
bufs = []
for n, seed in ((3000, 71), (gi.NOALLOC_MAX_BODIES, 72), (1, 73)):
    pos, vel, nfe = gi.ic_lattice(seed, n, spacing=0.999, jitter=0.004, vel_sigma=2.0,
                                  nfe=n // 3, mass_fe=2.5, mass_si=1.0)
    ptrs = []
    for host in (pos, vel, np.zeros_like(pos)):
        d = C.c_void_p()
        ok(rt.cudaMalloc(C.byref(d), C.c_size_t(host.nbytes)))
        ok(rt.cudaMemcpy(d, host.ctypes.data_as(C.c_void_p), C.c_size_t(host.nbytes), 1))
        ptrs.append(d)
    bufs.append((ptrs, gi.collision_consts(p, nfe), n))
ok(rt.cudaDeviceSynchronize())
free = [free_bytes()]
finite = True
for (dp, dv, df), c, n in bufs:
    gi.forces_collision_noalloc(dp.value, dv.value, df.value, c, n)
    ok(rt.cudaDeviceSynchronize())
    free.append(free_bytes())
    f = np.zeros((n, 4), np.float32)
    ok(rt.cudaMemcpy(f.ctypes.data_as(C.c_void_p), df, C.c_size_t(f.nbytes), 2))
    finite &= bool(np.isfinite(f).all())
print(json.dumps({"free": free, "finite": finite}))
'''


def test_noalloc_allocates_nothing_in_a_fresh_process(gi, torch_cuda, tmp_path):
    """The defining property, in a process that calls nothing else of the
    library: with every module loaded up front (CUDA_MODULE_LOADING=EAGER),
    free device memory stays the same from the end of the first call (3,000
    bodies) through a maximum-size call and a one-body call.  A hidden
    library context would have to grow its scratch for the larger run.  The
    child process allocates its inputs through the CUDA runtime itself."""
    import json
    import os
    import subprocess
    import sys
    from conftest import PKG
    script = tmp_path / "fresh_noalloc.py"
    script.write_text(_FRESH)
    env = dict(os.environ, CUDA_MODULE_LOADING="EAGER")
    out = subprocess.run([sys.executable, str(script), PKG], env=env, capture_output=True,
                         text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-3000:]
    res = json.loads(out.stdout.strip().splitlines()[-1])
    free = res["free"]
    print("free device bytes before / after each call:", free)
    assert res["finite"]
    assert free[1] == free[2] == free[3]
