"""CPU tests of the C ABI: the library loads, exports everything the header
declares, its host-only helpers compute what the reference computes, and its
seeded generators are reproducible.  No kernel is launched here."""
from __future__ import annotations

import ctypes as C
import hashlib

import numpy as np
import pytest


def test_exports_every_header_symbol(gi):
    names = gi.header_symbols()
    assert len(names) >= 20
    L = gi.lib()
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    assert L.gi_version() == 1


def test_status_strings(gi):
    L = gi.lib()
    for s in range(12):
        assert L.gi_status_string(s)
    assert L.gi_status_string(0) == b"ok"


def test_struct_layouts_match_reference(gi):
    # forceCollisionKernalConstantsStruct: 13 float + int; move: 3 float + int;
    # separate: 13 float + 3 int; move separate: 3 float + 3 int.
    assert C.sizeof(gi.ForceCollisionConsts) == 56
    assert C.sizeof(gi.MoveCollisionConsts) == 16
    assert C.sizeof(gi.ForceSeparateConsts) == 64
    assert C.sizeof(gi.MoveSeparateConsts) == 24
    assert C.sizeof(gi.PairParams) == 64
    assert C.sizeof(gi.Run) == 32


def test_params_from_material_matches_reference_formulas(gi):
    """loadKernalConstantStructures (impactAddTime.cu:128-170) in double,
    stored as float."""
    G, D, mfe, msi, kfe, ksi, krfe, krsi, sdfe, sdsi = 1.0, 1.0, 2.5, 1.0, 31.25, 9.375, 0.02, 0.01, 0.002, 0.001
    p = gi.params_from_material(G, D, mfe, msi, kfe, ksi, krfe, krsi, sdfe, sdsi)
    f = np.float32
    assert p.GMassFeFe == f(mfe * mfe) and p.GMassFeSi == f(mfe) and p.GMassSiSi == 1.0
    assert p.KFeFe == f(2 * kfe) and p.KSiSi == f(2 * ksi) and p.KFeSi == f(kfe + ksi)
    assert p.KRFeFe == f(2 * kfe * krfe) and p.KRSiSi == f(2 * ksi * krsi)
    assert p.KRFeSi == f(kfe * krfe + ksi * krsi)
    assert p.KRMix == f(kfe + ksi * krsi)  # SDFe >= SDSi
    assert p.ShellBreakFe == f(D - D * sdfe) and p.ShellBreakSi == f(D - D * sdsi)
    assert p.ShellBreakFeSi1 == f(D - D * sdsi) and p.ShellBreakFeSi2 == f(D - D * sdfe)
    q = gi.params_from_material(G, D, mfe, msi, kfe, ksi, krfe, krsi, 0.001, 0.002)
    assert q.KRMix == f(kfe * krfe + ksi)
    assert q.ShellBreakFeSi1 == f(D - D * 0.001) and q.ShellBreakFeSi2 == f(D - D * 0.002)


def test_params_from_collision_consts(gi):
    p = gi.params_from_material(1.0, 1.0, 2.5, 1.0, 31.25, 9.375, 0.02, 0.01, 0.002, 0.001)
    c = gi.collision_consts(p, 10)
    q = gi.params_from_collision_consts(c)
    assert q.GMassSiSi == 1.0 and q.MassSi == 1.0 and q.MassFe == p.GMassFeSi
    for n in ("KFeFe", "KRMix", "ShellBreakFeSi2"):
        assert getattr(q, n) == getattr(p, n)


def test_uniform_ball_reproducible_and_pinned(gi):
    a = gi.ic_uniform_ball(1, 8192)
    b = gi.ic_uniform_ball(1, 8192)
    assert np.array_equal(a[0], b[0]) and a[2] == b[2]
    pos, vel, nfe = a
    r = np.linalg.norm(pos[:, :3].astype(np.float64), axis=1)
    assert r.max() <= 20.0 + 1e-4
    assert np.all(r[:nfe] < 6.0 + 1e-5) and np.all(r[nfe:] >= 6.0 - 1e-5)
    # (0.3)^3 of the volume is Fe
    assert abs(nfe / 8192 - 0.027) < 0.006
    assert np.all(vel[:nfe, 3] == 1.0) and np.allclose(vel[nfe:, 3], 0.4)
    # Same bytes on every host (x86-64 here, aarch64 on the GPU host).
    h = hashlib.sha256(pos.tobytes() + vel.tobytes()).hexdigest()
    assert h == BALL_SHA256, h


BALL_SHA256 = "1fb4614d35e3866e8337e4cfe5ef9d1c99dfcfc98deacf900c54f98a80dee9eb"


def test_lattice_generator(gi):
    pos, vel, nfe = gi.ic_lattice(3, 1000, spacing=1.0, jitter=0.0, vel_sigma=0.0, nfe=100)
    assert nfe == 100
    assert np.all(vel[:, :3] == 0) and np.all(vel[:100, 3] == 1.0)
    assert pos[1, 0] == 1.0 and pos[10, 1] == 1.0 and pos[100, 2] == 1.0


def test_no_device_errors_cleanly(gi):
    """Without a GPU, device calls return an error status, never crash."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    st = gi.lib().gi_ctx_create(C.byref(h), 0)
    assert st in (4, 6)
    assert gi.lib().gi_last_error()


def test_invalid_arguments_rejected_before_device(gi):
    c = gi.ForceCollisionConsts()
    st = gi.lib().gi_forces_collision(None, None, None, C.byref(c), -1, None)
    assert st == 2
    st = gi.lib().gi_forces_collision(None, None, None, None, 10, None)
    assert st == 1
    m = gi.MoveSeparateConsts()
    m.boarder1, m.boarder2, m.boarder3 = 5, 3, 8
    assert gi.lib().gi_move_damped_separate(None, None, None, C.byref(m), 0.0, 0.0, 10, None) == 2
