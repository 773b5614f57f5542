"""GPU parity tests: libgi's sm_103a kernels, called through the C ABI, against
the FP64 oracle, the reference-exact CPU restatement and the reference's own
CUDA kernels on identical seeded inputs.

Tolerances (force): global relative L2 error against the FP64 oracle
<= 1e-5 (the stated force-error bound), and against the reference's own
kernels <= 1e-5.  Kick-drift: bit-exact.  Integer/index work (run
decomposition, batch invariance): bit-exact."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from conftest import config1_params, reference_unit_params, rel_l2

pytestmark = pytest.mark.gpu

FORCE_TOL = 1e-5


def dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    return t.cpu().numpy()


def stream(torch):
    return torch.cuda.current_stream().cuda_stream


@pytest.fixture(scope="module")
def ctx(gi, torch_cuda):
    c = gi.Context(0)
    yield c
    c.close()


def gpu_forces(gi, torch, ctx, pos, vel, runs, params):
    dp, dv = dev(torch, pos), dev(torch, vel)
    df = torch.full_like(dp, float("nan"))
    ctx.forces(dp.data_ptr(), dv.data_ptr(), df.data_ptr(), runs, params, stream(torch))
    torch.cuda.synchronize()
    return host(df)


def ball_with_velocities(gi, n, seed, vscale=1.5):
    pos, vel, nfe = gi.ic_uniform_ball(seed, n, 20.0 * (n / 8192.0) ** (1 / 3), 0.3, 1.0, 0.4,
                                       0.0, 1.0)
    rng = np.random.default_rng(seed)
    vel[:, :3] = rng.normal(scale=vscale, size=(n, 3)).astype(np.float32)
    return pos, vel, nfe


def test_config1_force_vs_fp64(gi, orc, torch_cuda, ctx):
    """The 8,192-body settle workload: per-step force error vs FP64."""
    import gi_workloads as wl
    pos, vel, nfe = wl.config1(gi)
    p = wl.params(gi)
    run = wl.run_desc(gi, 0, len(pos), nfe)
    f = gpu_forces(gi, torch_cuda, ctx, pos, vel, [run], p)
    f64, absf = orc.forces_fp64(pos, vel, [run], p)
    err = rel_l2(f[:, :3], f64)
    per_body = np.abs(f[:, :3] - f64).max(1) / absf
    print(f"config1 rel L2 {err:.3e}, max per-body err / sum|f| {per_body.max():.3e}")
    assert err < FORCE_TOL
    assert per_body.max() < 1e-5
    assert np.all(np.isnan(f[:, 3]))  # .w untouched


@pytest.mark.parametrize("kind", ["lattice", "ball"])
def test_drop_in_collision_vs_reference_kernel(gi, orc, torch_cuda, kind):
    """gi_forces_collision vs the reference's getForcesCollisionSingleGPU on
    the same inputs (reference units, N a multiple of 256)."""
    torch = torch_cuda
    p = reference_unit_params(gi)
    if kind == "lattice":
        pos, vel, nfe = gi.ic_lattice(7, 4096, spacing=0.999, jitter=0.004, vel_sigma=2.0,
                                      mass_fe=p.MassFe, mass_si=p.MassSi)
    else:
        pos, vel, nfe = ball_with_velocities(gi, 8192, 8)
    n = len(pos)
    c = gi.collision_consts(p, nfe)
    dp, dv = dev(torch, pos), dev(torch, vel)
    mine = torch.full_like(dp, float("nan"))
    theirs = torch.full_like(dp, float("nan"))
    gi.forces_collision(dp.data_ptr(), dv.data_ptr(), mine.data_ptr(), c, n, stream(torch))
    ref = orc.ref_lib()
    if ref is None:
        pytest.skip("reference kernels not built (oracle/_ref absent)")
    assert ref.giref_forces_collision(dp.data_ptr(), dv.data_ptr(), theirs.data_ptr(), C.byref(c),
                                      n, stream(torch)) == 0
    torch.cuda.synchronize()
    mine, theirs = host(mine)[:, :3], host(theirs)[:, :3]
    run = (0, n, nfe, 0, 0, 0, 0, 0)
    f64, _ = orc.forces_fp64(pos, vel, [run], p)
    e_mine, e_ref, e_mr = rel_l2(mine, f64), rel_l2(theirs, f64), rel_l2(mine, theirs)
    print(f"{kind}: mine vs fp64 {e_mine:.3e}, reference vs fp64 {e_ref:.3e}, mine vs ref {e_mr:.3e}")
    assert e_mine < FORCE_TOL
    assert e_mr < FORCE_TOL
    # the reference-exact oracle reproduces the reference kernel
    assert np.array_equal(orc.forces_ref(pos, vel, [run], p)[:, :3], theirs)


def test_drop_in_separate_vs_reference_kernel(gi, orc, torch_cuda):
    torch = torch_cuda
    p = reference_unit_params(gi)
    pa, va, fa = gi.ic_lattice(21, 3072, vel_sigma=1.5, nfe=1000, mass_fe=p.MassFe, mass_si=p.MassSi)
    pb, vb, fb = gi.ic_lattice(22, 1024, vel_sigma=1.5, nfe=300, mass_fe=p.MassFe, mass_si=p.MassSi)
    pb[:, 0] += 4.0
    pos, vel = np.concatenate([pa, pb]), np.concatenate([va, vb])
    n, b1, b2, b3 = 4096, fa, 3072, 3072 + fb
    sc = gi.separate_consts(p, b1, b2, b3)
    dp, dv = dev(torch, pos), dev(torch, vel)
    mine = torch.zeros_like(dp)
    gi.forces_separate(dp.data_ptr(), dv.data_ptr(), mine.data_ptr(), sc, n, stream(torch))
    torch.cuda.synchronize()
    runs = [(0, b2, b1, 0, 0, 0, 0, 0), (b2, n - b2, b3 - b2, 0, 0, 0, 0, 0)]
    f64, _ = orc.forces_fp64(pos, vel, runs, p)
    assert rel_l2(host(mine)[:, :3], f64) < FORCE_TOL
    ref = orc.ref_lib()
    if ref is None:
        pytest.skip("reference kernels not built")
    theirs = torch.zeros_like(dp)
    assert ref.giref_forces_separate(dp.data_ptr(), dv.data_ptr(), theirs.data_ptr(), C.byref(sc),
                                     n, stream(torch)) == 0
    torch.cuda.synchronize()
    assert rel_l2(host(mine)[:, :3], host(theirs)[:, :3]) < FORCE_TOL


def test_move_bitwise_vs_reference_kernel(gi, orc, torch_cuda):
    torch = torch_cuda
    rng = np.random.default_rng(3)
    n, nfe = 2048, 700
    pos = rng.normal(size=(n, 4)).astype(np.float32)
    vel = rng.normal(size=(n, 4)).astype(np.float32)
    force = rng.normal(size=(n, 4)).astype(np.float32) * 50
    mc = gi.MoveCollisionConsts(6.3e-4, 6.3e-4 / 2.5, 6.3e-4, nfe)
    a = [dev(torch, x) for x in (pos, vel, force)]
    gi.move_collision(a[0].data_ptr(), a[1].data_ptr(), a[2].data_ptr(), mc, n, stream(torch))
    torch.cuda.synchronize()
    run = (0, n, nfe, 0, mc.Dt, mc.DtOverMassFe, mc.DtOverMassSi, 0.0)
    p2, v2 = orc.move_ref(pos, vel, force, [run])
    assert np.array_equal(host(a[0]), p2) and np.array_equal(host(a[1]), v2)
    ref = orc.ref_lib()
    if ref is not None:
        b = [dev(torch, x) for x in (pos, vel, force)]
        assert ref.giref_move_collision(b[0].data_ptr(), b[1].data_ptr(), b[2].data_ptr(),
                                        C.byref(mc), n, stream(torch)) == 0
        torch.cuda.synchronize()
        assert np.array_equal(host(a[0]), host(b[0])) and np.array_equal(host(a[1]), host(b[1]))
    # damped, two bodies
    ms = gi.MoveSeparateConsts(1e-3, 1e-3, 2.5e-3, 300, 1500, 1800)
    c = [dev(torch, x) for x in (pos, vel, force)]
    gi.move_damped_separate(c[0].data_ptr(), c[1].data_ptr(), c[2].data_ptr(), ms, 8.0, 2.0, n,
                            stream(torch))
    torch.cuda.synchronize()
    runs = [(0, 1500, 300, 0, 1e-3, 1e-3, 2.5e-3, 8.0), (1500, 548, 300, 0, 1e-3, 1e-3, 2.5e-3, 2.0)]
    p3, v3 = orc.move_ref(pos, vel, force, runs)
    assert np.array_equal(host(c[0]), p3) and np.array_equal(host(c[1]), v3)
    if ref is not None:
        d = [dev(torch, x) for x in (pos, vel, force)]
        assert ref.giref_move_damped_separate(d[0].data_ptr(), d[1].data_ptr(), d[2].data_ptr(),
                                              C.byref(ms), 8.0, 2.0, n, stream(torch)) == 0
        torch.cuda.synchronize()
        assert np.array_equal(host(c[1]), host(d[1]))


@pytest.mark.parametrize("n", [1, 2, 3, 31, 127, 128, 129, 255, 257, 1000, 4099])
def test_ragged_sizes(gi, orc, torch_cuda, ctx, n):
    p = config1_params(gi)
    pos, vel, nfe = gi.ic_lattice(n, n, spacing=0.999, jitter=0.004, vel_sigma=1.0, nfe=n // 3)
    run = (0, n, nfe, 0, 0.0, 0.0, 0.0, 0.0)
    f = gpu_forces(gi, torch_cuda, ctx, pos, vel, [gi.Run(*run)], p)
    f64, absf = orc.forces_fp64(pos, vel, [run], p)
    if n == 1:
        assert np.all(f[:, :3] == 0)
    else:
        assert rel_l2(f[:, :3], f64) < FORCE_TOL
        assert np.all(np.abs(f[:, :3] - f64).max(1) <= 1e-5 * absf + 1e-30)


def test_empty_and_invalid(gi, torch_cuda, ctx):
    torch = torch_cuda
    p = config1_params(gi)
    dp = torch.zeros((16, 4), device="cuda")
    # empty run: no-op
    ctx.forces(dp.data_ptr(), dp.data_ptr(), dp.data_ptr(), [gi.Run(0, 0, 0, 0, 0, 0, 0, 0)], p)
    with pytest.raises(gi.GIError) as e:
        ctx.forces(dp.data_ptr() + 4, dp.data_ptr(), dp.data_ptr(), [gi.Run(0, 8, 0, 0, 0, 0, 0, 0)], p)
    assert e.value.status == 3
    with pytest.raises(gi.GIError) as e:
        ctx.forces(dp.data_ptr(), dp.data_ptr(), dp.data_ptr(),
                   [gi.Run(0, 8, 0, 0, 0, 0, 0, 0), gi.Run(4, 8, 0, 0, 0, 0, 0, 0)], p)
    assert e.value.status == 1
    with pytest.raises(gi.GIError) as e:
        ctx.forces(dp.data_ptr(), dp.data_ptr(), dp.data_ptr(), [gi.Run(0, 8, 9, 0, 0, 0, 0, 0)], p)
    assert e.value.status == 2
    bad = gi.PairParams.from_buffer_copy(bytes(p))
    bad.GMassFeSi = 3.0 * bad.GMassFeSi
    with pytest.raises(gi.GIError) as e:
        ctx.forces(dp.data_ptr(), dp.data_ptr(), dp.data_ptr(), [gi.Run(0, 8, 2, 0, 0, 0, 0, 0)], bad)
    assert e.value.status == 8


def test_fused_step_equals_force_then_move(gi, torch_cuda, ctx):
    torch = torch_cuda
    import gi_workloads as wl
    p = wl.params(gi)
    pos, vel, nfe = gi.ic_lattice(5, 6000, vel_sigma=1.0)
    run = wl.run_desc(gi, 0, 6000, nfe)
    dp, dv = dev(torch, pos), dev(torch, vel)
    for _ in range(3):
        df = torch.zeros_like(dp)
        ctx.forces(dp.data_ptr(), dv.data_ptr(), df.data_ptr(), [run], p)
        ctx.move(dp.data_ptr(), dv.data_ptr(), df.data_ptr(), [run])
    ep, ev = dev(torch, pos), dev(torch, vel)
    ctx.step(ep.data_ptr(), ev.data_ptr(), [run], p, 3)
    torch.cuda.synchronize()
    assert torch.equal(dp, ep) and torch.equal(dv, ev)


def test_pingpong_matches_in_place_step(gi, torch_cuda, ctx):
    torch = torch_cuda
    import gi_workloads as wl
    p = wl.params(gi)
    pos, vel, nfe = gi.ic_lattice(15, 7000, vel_sigma=1.0)
    run = wl.run_desc(gi, 0, 7000, nfe)
    a = (dev(torch, pos), dev(torch, vel))
    b = (torch.zeros_like(a[0]), torch.zeros_like(a[1]))
    ctx.step_pingpong(a[0].data_ptr(), a[1].data_ptr(), b[0].data_ptr(), b[1].data_ptr(), [run], p, 3)
    c = (dev(torch, pos), dev(torch, vel))
    ctx.step(c[0].data_ptr(), c[1].data_ptr(), [run], p, 3)
    torch.cuda.synchronize()
    assert torch.equal(b[0], c[0]) and torch.equal(b[1], c[1])  # odd step count ends in b
    with pytest.raises(gi.GIError):
        ctx.step_pingpong(a[0].data_ptr(), a[1].data_ptr(), a[0].data_ptr(), b[1].data_ptr(), [run], p, 1)


def test_contacts_deterministic_and_bucket_independent(gi, torch_cuda):
    """Contact corrections are summed in fixed point: repeated passes (whose
    bucket order varies with the atomics) give bit-identical forces, also
    for a dense clump where hundreds of bodies overlap."""
    torch = torch_cuda
    import gi_workloads as wl
    p = wl.params(gi)
    pos, vel, nfe = ball_with_velocities(gi, 30000, 19)
    # a dense clump: 600 bodies squeezed into a ball of radius 2
    rng = np.random.default_rng(3)
    cl = rng.normal(size=(600, 3))
    cl = cl / np.linalg.norm(cl, axis=1, keepdims=True) * rng.uniform(0, 2.0, size=(600, 1))
    pos[:600, :3] = cl.astype(np.float32)
    run = wl.run_desc(gi, 0, 30000, nfe)
    c = gi.Context(0)
    f1 = gpu_forces(gi, torch, c, pos, vel, [run], p)
    f2 = gpu_forces(gi, torch, c, pos, vel, [run], p)
    c.close()
    assert np.array_equal(f1[:, :3], f2[:, :3])


def test_graph_step_loop_matches_pingpong(gi, torch_cuda):
    """A captured graph of 4 fused steps over a small sweep gives exactly the
    state of gi_step_pingpong, launch after launch."""
    torch = torch_cuda
    import gi_workloads as wl
    p = wl.params(gi)
    pos, vel, runs, _ = wl.sweep(gi, torch, nruns=5, seed=9, settle_steps=10, nmin=500, nmax=3000)
    c = gi.Context(0)
    s = torch.cuda.Stream()
    a = (dev(torch, pos), dev(torch, vel))
    b = (torch.empty_like(a[0]), torch.empty_like(a[1]))
    with torch.cuda.stream(s):
        g = c.graph(a[0].data_ptr(), a[1].data_ptr(), b[0].data_ptr(), b[1].data_ptr(), runs, p, 4,
                    s.cuda_stream)
        g.launch(s.cuda_stream)
        g.launch(s.cuda_stream)
    torch.cuda.synchronize()
    x = (dev(torch, pos), dev(torch, vel))
    y = (torch.empty_like(x[0]), torch.empty_like(x[1]))
    c.step_pingpong(x[0].data_ptr(), x[1].data_ptr(), y[0].data_ptr(), y[1].data_ptr(), runs, p, 8)
    torch.cuda.synchronize()
    g.close()
    c.close()
    for r in runs:  # bodies outside runs are untouched either way
        sl = slice(r.offset, r.offset + r.n)
        assert torch.equal(a[0][sl], x[0][sl]) and torch.equal(a[1][sl], x[1][sl])


def test_batch_invariance(gi, torch_cuda, ctx):
    """A run's forces are bit-identical alone and inside a batch."""
    torch = torch_cuda
    import gi_workloads as wl
    p = wl.params(gi)
    sizes = [5000, 12000, 700, 33000]
    bodies = [gi.ic_lattice(s + 1, s, vel_sigma=1.0) for s in sizes]
    pos = np.concatenate([b[0] for b in bodies])
    vel = np.concatenate([b[1] for b in bodies])
    offs = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(int)
    runs = [wl.run_desc(gi, int(o), s, b[2]) for o, s, b in zip(offs, sizes, bodies)]
    mixed = gpu_forces(gi, torch, ctx, pos, vel, runs, p)
    for k, (o, s) in enumerate(zip(offs, sizes)):
        alone = gpu_forces(gi, torch, ctx, bodies[k][0], bodies[k][1],
                           [wl.run_desc(gi, 0, s, bodies[k][2])], p)
        assert np.array_equal(alone[:, :3], mixed[o:o + s, :3]), k


def test_more_runs_than_one_launch_table(gi, orc, torch_cuda, ctx):
    """70 runs in one call: more than a launch table holds (64), so the call
    runs two tables one after the other, each clearing and filling the
    far-field sums.  Every run equals the run alone, bit for bit, and the
    batch matches the FP64 oracle."""
    torch = torch_cuda
    import gi_workloads as wl
    p = wl.params(gi)
    sizes = [300 + 37 * (k % 11) for k in range(70)]
    bodies = [gi.ic_lattice(200 + k, n, vel_sigma=1.0) for k, n in enumerate(sizes)]
    pos = np.concatenate([b[0] for b in bodies])
    vel = np.concatenate([b[1] for b in bodies])
    offs = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(int)
    runs = [wl.run_desc(gi, int(o), n, b[2]) for o, n, b in zip(offs, sizes, bodies)]
    mixed = gpu_forces(gi, torch, ctx, pos, vel, runs, p)
    for k in (0, 33, 64, 69):
        o, n = int(offs[k]), sizes[k]
        alone = gpu_forces(gi, torch, ctx, bodies[k][0], bodies[k][1],
                           [wl.run_desc(gi, 0, n, bodies[k][2])], p)
        assert np.array_equal(alone[:, :3], mixed[o:o + n, :3]), k
    f64, _ = orc.forces_fp64(pos, vel, [(int(o), n, b[2], 0, 0, 0, 0, 0) for o, n, b in
                                        zip(offs, sizes, bodies)], p)
    assert rel_l2(mixed[:, :3], f64) < FORCE_TOL


def test_mixed_pair_tables_and_mass_scales(gi, orc, torch_cuda, ctx):
    """Three runs in one call, each with its own pair table, the masses 10^3
    apart from table to table (forces 10^6 apart; stiffness scaled with
    m^2): each run's far field sums in a fixed-point unit of its own table.
    Every run matches the FP64 oracle and is bit-identical to the run alone."""
    torch = torch_cuda
    scales = [1e-3, 1.0, 1e3]
    ps = [gi.params_from_material(1.0, 1.0, s, 0.4 * s, 5.0 * s * s, 1.5 * s * s, 0.02, 0.01,
                                  0.002, 0.001) for s in scales]
    sizes, nfes = [2500, 3300, 1800], [700, 1000, 0]
    bodies = [gi.ic_lattice(80 + k, n, vel_sigma=1.0, nfe=f) for k, (n, f) in
              enumerate(zip(sizes, nfes))]
    pos = np.concatenate([b[0] for b in bodies])
    vel = np.concatenate([b[1] for b in bodies])
    offs = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(int)
    runs = [gi.Run(int(o), n, f, k, 0, 0, 0, 0) for k, (o, n, f) in
            enumerate(zip(offs, sizes, nfes))]
    mixed = gpu_forces(gi, torch, ctx, pos, vel, runs, ps)
    f64, _ = orc.forces_fp64(pos, vel, [(int(o), n, f, k, 0, 0, 0, 0) for k, (o, n, f) in
                                        enumerate(zip(offs, sizes, nfes))], ps)
    for k, (o, n, f) in enumerate(zip(offs, sizes, nfes)):
        err = rel_l2(mixed[o:o + n, :3], f64[o:o + n])
        print(f"table {k} (mass x {scales[k]:g}): rel L2 {err:.3e}, |F| ~ "
              f"{np.abs(f64[o:o + n]).mean():.3e}")
        assert err < FORCE_TOL
        alone = gpu_forces(gi, torch, ctx, bodies[k][0], bodies[k][1],
                           [gi.Run(0, n, f, 0, 0, 0, 0, 0)], ps[k])
        assert np.array_equal(alone[:, :3], mixed[o:o + n, :3]), k


def test_side_by_side_and_serial_paths_agree(gi, torch_cuda, ctx):
    """Tables of fewer than 2^34 pairs run the contact pass beside the far
    field and finish in a separate kernel; larger ones run it first and take
    the fused epilogue.  Three 80,000-body runs (6.4e9 pairs each) alone take
    the first path, batched (1.9e10 pairs) the second: forces and a fused step
    agree bit for bit."""
    torch = torch_cuda
    import gi_workloads as wl
    p = wl.params(gi)
    n = 80000
    bodies = [gi.ic_lattice(40 + k, n, vel_sigma=1.0) for k in range(3)]
    pos = np.concatenate([b[0] for b in bodies])
    vel = np.concatenate([b[1] for b in bodies])
    runs = [wl.run_desc(gi, k * n, n, bodies[k][2]) for k in range(3)]
    assert 3 * n * n >= 1 << 34 > n * n
    batched = gpu_forces(gi, torch, ctx, pos, vel, runs, p)
    s = stream(torch)
    dp, dv = dev(torch, pos), dev(torch, vel)
    ctx.step(dp.data_ptr(), dv.data_ptr(), runs, p, 1, s)
    torch.cuda.synchronize()
    for k in range(3):
        one = [wl.run_desc(gi, 0, n, bodies[k][2])]
        alone = gpu_forces(gi, torch, ctx, bodies[k][0], bodies[k][1], one, p)
        assert np.array_equal(alone[:, :3], batched[k * n:(k + 1) * n, :3]), k
        ap, av = dev(torch, bodies[k][0]), dev(torch, bodies[k][1])
        ctx.step(ap.data_ptr(), av.data_ptr(), one, p, 1, s)
        torch.cuda.synchronize()
        assert np.array_equal(host(ap), host(dp)[k * n:(k + 1) * n]), k
        assert np.array_equal(host(av), host(dv)[k * n:(k + 1) * n]), k


@pytest.mark.parametrize("ipt,jchunk", [(1, 0), (2, 1024), (4, 2048), (4, 128), (1, 512), (8, 256)])
def test_decompositions_agree(gi, orc, torch_cuda, ipt, jchunk):
    """The one-sided kernel's decompositions (i-bodies per thread, split
    j-chunks) against the FP64 oracle."""
    p = config1_params(gi)
    pos, vel, nfe = gi.ic_lattice(9, 5000, vel_sigma=1.5)
    run = gi.Run(0, 5000, nfe, 0, 0, 0, 0, 0)
    c = gi.Context(0, accum=gi.GI_ACCUM_KAHAN)
    c.set_tuning(ipt, jchunk)
    f = gpu_forces(gi, torch_cuda, c, pos, vel, [run], p)
    c.close()
    f64, _ = orc.forces_fp64(pos, vel, [(0, 5000, nfe, 0, 0, 0, 0, 0)], p)
    assert rel_l2(f[:, :3], f64) < FORCE_TOL


# Sizes around the paired kernel's 64-body chunks (two bodies a lane),
# 256-row warps and 1024-row i-blocks, with the Fe/Si boundary inside a
# chunk, on a chunk boundary, at 0 and at n.
PAIRED_CASES = [(1, 1), (2, 1), (31, 7), (32, 32), (33, 0), (63, 40), (64, 64), (65, 33),
                (255, 255), (256, 100), (257, 257), (1023, 511), (1024, 64), (1025, 1000),
                (2047, 1040), (3000, 1100), (5000, 0)]


@pytest.mark.parametrize("n,nfe", PAIRED_CASES)
def test_paired_far_field_sizes(gi, orc, torch_cuda, ctx, n, nfe):
    """Every unordered pair exactly once: any pair missed or counted twice
    would move the force by a whole pair term, far above the tolerance."""
    p = config1_params(gi)
    pos, vel, _ = gi.ic_lattice(60 + n % 17, n, vel_sigma=1.2, nfe=nfe)
    run = gi.Run(0, n, nfe, 0, 0, 0, 0, 0)
    f = gpu_forces(gi, torch_cuda, ctx, pos, vel, [run], p)
    f64, absf = orc.forces_fp64(pos, vel, [(0, n, nfe, 0, 0, 0, 0, 0)], p)
    if n == 1:
        assert np.all(f[:, :3] == 0)
    else:
        assert rel_l2(f[:, :3], f64) < FORCE_TOL
        assert np.all(np.abs(f[:, :3] - f64).max(1) <= 1e-5 * absf + 1e-30)


@pytest.mark.parametrize("jchunk", [32, 64, 128, 512, 1024, 0])
def test_paired_chunks_per_item(gi, orc, torch_cuda, jchunk):
    """Forced j-bodies per work item (1 to 16 chunks of 64): each stays
    within tolerance, and repeated calls are bit-identical."""
    p = config1_params(gi)
    n, nfe = 4500, 1337
    pos, vel, _ = gi.ic_lattice(77, n, vel_sigma=1.5, nfe=nfe)
    run = gi.Run(0, n, nfe, 0, 0, 0, 0, 0)
    c = gi.Context(0)
    c.set_tuning(1, jchunk)
    assert c.get_tuning(n) == (8, max(64, min(jchunk or 1024, 1024)))
    f = gpu_forces(gi, torch_cuda, c, pos, vel, [run], p)
    g = gpu_forces(gi, torch_cuda, c, pos, vel, [run], p)
    c.close()
    assert np.array_equal(f[:, :3], g[:, :3])
    f64, _ = orc.forces_fp64(pos, vel, [(0, n, nfe, 0, 0, 0, 0, 0)], p)
    assert rel_l2(f[:, :3], f64) < FORCE_TOL


@pytest.mark.parametrize("accum", ["PAIRED", "FP32", "FP64", "KAHAN"])
def test_accumulation_modes(gi, orc, torch_cuda, accum):
    p = config1_params(gi)
    pos, vel, nfe = ball_with_velocities(gi, 20000, 4)
    c = gi.Context(0, accum=getattr(gi, "GI_ACCUM_" + accum))
    run = gi.Run(0, len(pos), nfe, 0, 0, 0, 0, 0)
    c.set_tuning(4, 0)  # one chunk: the accumulation mode alone decides the error
    f = gpu_forces(gi, torch_cuda, c, pos, vel, [run], p)
    c.close()
    idx = np.arange(0, len(pos), 7)
    f64, _ = orc.forces_fp64(pos, vel, [(0, len(pos), nfe, 0, 0, 0, 0, 0)], p, idx=idx)
    err = rel_l2(f[idx, :3], f64)
    print(f"accum {accum}: rel L2 {err:.3e}")
    assert err < (2e-5 if accum == "FP32" else FORCE_TOL)


@pytest.mark.parametrize("accum", ["PAIRED", "KAHAN"])
def test_autotune_keeps_results_within_tolerance(gi, orc, torch_cuda, accum):
    torch = torch_cuda
    import gi_workloads as wl
    p = wl.params(gi)
    pos, vel, nfe = ball_with_velocities(gi, 20000, 23)
    run = wl.run_desc(gi, 0, 20000, nfe)
    c = gi.Context(0, accum=getattr(gi, "GI_ACCUM_" + accum))
    dp, dv = dev(torch, pos), dev(torch, vel)
    c.autotune(dp.data_ptr(), dv.data_ptr(), [run], p)
    tuned = c.get_tuning(20000)
    f = gpu_forces(gi, torch, c, pos, vel, [run], p)
    c.close()
    idx = np.arange(0, 20000, 11)
    f64, _ = orc.forces_fp64(pos, vel, [(0, 20000, nfe, 0, 0, 0, 0, 0)], p, idx=idx)
    print("tuned", tuned)
    assert tuned[0] in ((8,) if accum == "PAIRED" else (1, 2, 4))
    assert rel_l2(f[idx, :3], f64) < FORCE_TOL


def test_sign_separation_mode(gi, orc, torch_cuda):
    p = config1_params(gi)
    pos, vel, nfe = gi.ic_lattice(31, 3000, vel_sigma=0.3)
    c = gi.Context(0, sep_test=gi.GI_SEP_SIGN)
    f = gpu_forces(gi, torch_cuda, c, pos, vel, [gi.Run(0, 3000, nfe, 0, 0, 0, 0, 0)], p)
    c.close()
    run = (0, 3000, nfe, 0, 0, 0, 0, 0)
    f64, _ = orc.forces_fp64(pos, vel, [run], p, sep_test=orc.SEP_SIGN)
    f64_int, _ = orc.forces_fp64(pos, vel, [run], p, sep_test=orc.SEP_REF_INT)
    assert rel_l2(f[:, :3], f64) < FORCE_TOL
    assert rel_l2(f64_int, f64) > 1e-4  # the two tests really differ here


def test_diag_and_potential_vs_oracle(gi, orc, torch_cuda, ctx):
    torch = torch_cuda
    import gi_workloads as wl
    p = wl.params(gi)
    pos, vel, nfe = ball_with_velocities(gi, 9000, 12)
    run = wl.run_desc(gi, 0, 9000, nfe)
    dp, dv = dev(torch, pos), dev(torch, vel)
    d = np.array(ctx.diag(dp.data_ptr(), dv.data_ptr(), run, p))
    want = orc.diag_fp64(pos, vel, (0, 9000, nfe, 0, 0, 0, 0, 0), p)
    assert np.allclose(d, want, rtol=1e-12, atol=1e-9 * np.abs(want).max())
    label = np.zeros(9000, np.uint8)
    label[:4000] = 1
    label[4000:5000] = 2
    dl = dev(torch, label)
    for scope in (1, 2, 3):
        d = np.array(ctx.diag(dp.data_ptr(), dv.data_ptr(), run, p, label=dl.data_ptr(), scope=scope))
        want = orc.diag_fp64(pos, vel, (0, 9000, nfe, 0, 0, 0, 0, 0), p, label=label, scope=scope)
        assert np.allclose(d, want, rtol=1e-12, atol=1e-9 * np.abs(want).max()), scope
    u = ctx.potential(dp.data_ptr(), [run], p)[0]
    u64 = orc.potential_fp64(pos, [(0, 9000, nfe, 0, 0, 0, 0, 0)], p).sum() / 2
    print(f"potential {u:.10e} vs {u64:.10e}")
    assert u == pytest.approx(u64, rel=1e-7)


def test_diag_far_from_origin_and_moving(gi, orc, torch_cuda, ctx):
    """The FP64 diagnostics keep their per-body sums in float-float pairs on
    the FP32 pipe.  Here 300,000 bodies sit 1.1e4 D from the origin, move at
    a bulk 32 D per time unit and spin slowly, so the angular momentum about
    the centre of mass is far smaller than the orbital term M c x u, and the
    centre of mass is a small difference of large sums.  Against the FP64
    oracle (sequential double sums): every quantity to about 1e-12 of its
    own scale, the angular momentum to 1e-10 of sum |m r x w|."""
    torch = torch_cuda
    n = 300000
    rng = np.random.default_rng(21)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r = 30.0 * rng.uniform(0, 1, size=(n, 1)) ** (1 / 3)
    x = d * r
    w = 0.01 * np.stack([-x[:, 1], x[:, 0], np.zeros(n)], 1)  # spin about z
    pos = np.zeros((n, 4), np.float32)
    vel = np.zeros((n, 4), np.float32)
    pos[:, :3] = x + np.array([1.0e4, -5.0e3, 2.0e3])
    vel[:, :3] = w + rng.normal(scale=0.5, size=(n, 3)) + np.array([30.0, -10.0, 5.0])
    nfe = n // 10
    p = config1_params(gi)
    run = gi.Run(0, n, nfe, 0, 0, 0, 0, 0)
    dp, dv = dev(torch, pos), dev(torch, vel)
    got = np.array(ctx.diag(dp.data_ptr(), dv.data_ptr(), run, p))
    want = orc.diag_fp64(pos, vel, (0, n, nfe, 0, 0, 0, 0, 0), p)
    m = np.where(np.arange(n) < nfe, p.MassFe, p.MassSi).astype(np.float64)
    P64, V64 = pos[:, :3].astype(np.float64), vel[:, :3].astype(np.float64)
    assert got[14] == want[14] == n
    assert abs(got[0] - want[0]) <= 1e-13 * want[0]
    assert np.abs(got[1:4] - want[1:4]).max() <= 1e-12 * np.abs(P64).max()
    assert np.abs(got[4:7] - want[4:7]).max() <= 1e-12 * np.abs(V64).max()
    assert abs(got[10] - want[10]) <= 1e-12 * want[10]
    assert np.abs(got[11:14] - want[11:14]).max() <= 1e-12 * (m[:, None] * np.abs(V64)).sum()
    rr, ww = P64 - want[1:4], V64 - want[4:7]
    scale = (m[:, None] * np.abs(np.cross(rr, ww))).sum()
    err = np.abs(got[7:10] - want[7:10]).max()
    print(f"L about the com {want[7:10]}, |error| {err:.3e}, sum |m r x w| {scale:.3e}")
    assert err <= 1e-10 * scale
    # the same call twice gives the same bits
    again = np.array(ctx.diag(dp.data_ptr(), dv.data_ptr(), run, p))
    assert np.array_equal(got, again)


@pytest.mark.parametrize("nsteps", [0, 1, 4])
def test_run_host_matches_device_path(gi, torch_cuda, ctx, nsteps):
    """Host buffers in and out, with two runs and a gap between them that no
    run covers (left as it was): the same bits as the device path, for an
    even and an odd number of steps."""
    torch = torch_cuda
    import gi_workloads as wl
    p = wl.params(gi)
    pos, vel, nfe = gi.ic_lattice(77, 3000, vel_sigma=1.0)
    pos2, vel2, nfe2 = gi.ic_lattice(78, 1200, vel_sigma=1.0)
    gap = np.full((100, 4), 7.0, np.float32)
    P = np.concatenate([pos, gap, pos2])
    V = np.concatenate([vel, gap, vel2])
    runs = [wl.run_desc(gi, 0, 3000, nfe), wl.run_desc(gi, 3100, 1200, nfe2)]
    hp, hv = P.copy(), V.copy()
    ctx.run_host(hp.ctypes.data, hv.ctypes.data, len(P), runs, p, nsteps)
    dp, dv = dev(torch, P), dev(torch, V)
    ctx.step(dp.data_ptr(), dv.data_ptr(), runs, p, nsteps)
    torch.cuda.synchronize()
    assert np.array_equal(hp, host(dp)) and np.array_equal(hv, host(dv))
    assert np.array_equal(hp[3000:3100], gap) and np.array_equal(hv[3000:3100], gap)


def test_large_n_subsample_vs_fp64(gi, orc, torch_cuda, ctx):
    """1,153,434 bodies (the precision-study size): FP64 oracle on a seeded
    subsample of i-bodies against all j."""
    n = 1_153_434
    p = config1_params(gi)
    pos, vel, nfe = gi.ic_uniform_ball(5, n, 20.0 * (n / 8192.0) ** (1 / 3), 0.3, 1.0, 0.4, 0.0, 1.0)
    run = gi.Run(0, n, nfe, 0, 0, 0, 0, 0)
    f = gpu_forces(gi, torch_cuda, ctx, pos, vel, [run], p)
    idx = np.random.default_rng(5).choice(n, 96, replace=False).astype(np.int32)
    f64, _ = orc.forces_fp64(pos, vel, [(0, n, nfe, 0, 0, 0, 0, 0)], p, idx=idx)
    err = rel_l2(f[idx, :3], f64)
    print(f"N={n}: subsample rel L2 {err:.3e}")
    assert err < FORCE_TOL
    assert np.isfinite(f[:, :3]).all()


def test_dense_contact_path_matches_sparse_path(gi, orc, torch_cuda):
    """A collapsed remnant (cells of hundreds of bodies, thousands of contacts
    per body) next to a sparse ball: the shared-memory tiled contact pass
    (dense cells) and the warp-per-body pass give bit-identical forces, and
    both stay within the force tolerance of the FP64 oracle."""
    torch = torch_cuda
    import gi_workloads as wl
    p = wl.params(gi)
    n_dense, n_sparse = 12000, 8000
    rng = np.random.default_rng(23)
    d = rng.normal(size=(n_dense, 3))
    d = d / np.linalg.norm(d, axis=1, keepdims=True) * (rng.uniform(0, 1, size=(n_dense, 1)) ** (1 / 3)) * 4.0
    sp, _, _ = ball_with_velocities(gi, n_sparse, 24)
    pos = np.zeros((n_dense + n_sparse, 4), np.float32)
    pos[:n_dense, :3] = d
    pos[n_dense:] = sp
    pos[n_dense:, 0] += 60.0
    vel = np.zeros_like(pos)
    vel[:, :3] = rng.normal(scale=2.0, size=(len(pos), 3)).astype(np.float32)
    vel[:, 3] = 0.4
    nfe = 1500
    run = wl.run_desc(gi, 0, len(pos), nfe)
    tiled = gi.Context(0, dense_min=64)
    warp = gi.Context(0, dense_min=1 << 30)
    ft = gpu_forces(gi, torch, tiled, pos, vel, [run], p)
    fw = gpu_forces(gi, torch, warp, pos, vel, [run], p)
    ft2 = gpu_forces(gi, torch, tiled, pos, vel, [run], p)
    tiled.close()
    warp.close()
    assert np.isfinite(ft[:, :3]).all()
    assert np.array_equal(ft[:, :3], fw[:, :3])
    assert np.array_equal(ft[:, :3], ft2[:, :3])
    idx = np.concatenate([np.arange(0, n_dense, 61), np.arange(n_dense, len(pos), 97)]).astype(np.int32)
    f64, _ = orc.forces_fp64(pos, vel, [(0, len(pos), nfe, 0, 0, 0, 0, 0)], p, idx=idx)
    err = rel_l2(ft[idx, :3], f64)
    print(f"dense remnant: rel L2 vs FP64 {err:.3e}")
    assert err < FORCE_TOL


@pytest.mark.gpu
def test_dense_contact_path_crowded_cells(gi, orc, torch_cuda):
    """Cells of hundreds of bodies (several 128-body chunks and neighbour
    tiles, reordered by sub-cell), one cell of 9,000 bodies (above the
    in-bucket sort's capacity, so left in scatter order) and two runs laid
    over the same space (their buckets must stay apart): the tiled path
    equals the warp path bit for bit, repeats bit for bit, and stays within
    the force tolerance of the FP64 oracle."""
    torch = torch_cuda
    import gi_workloads as wl
    p = wl.params(gi)
    rng = np.random.default_rng(29)

    def ball(n, radius, centre):
        d = rng.normal(size=(n, 3))
        d = d / np.linalg.norm(d, axis=1, keepdims=True) * (rng.uniform(0, 1, size=(n, 1)) ** (1 / 3))
        return d * radius + np.asarray(centre)

    run_a = np.concatenate([ball(10000, 1.8, (0.0, 0.0, 0.0)),
                            rng.uniform(0.05, 0.95, size=(9000, 3)) + np.array([30.0, 0.0, 0.0])])
    run_b = ball(6000, 1.6, (0.3, 0.2, 0.1))
    pos = np.zeros((len(run_a) + len(run_b), 4), np.float32)
    pos[:len(run_a), :3] = run_a
    pos[len(run_a):, :3] = run_b
    vel = np.zeros_like(pos)
    vel[:, :3] = rng.normal(scale=2.0, size=(len(pos), 3)).astype(np.float32)
    vel[:, 3] = 0.4
    nfe_a, nfe_b = 3000, 1000
    runs = [wl.run_desc(gi, 0, len(run_a), nfe_a), wl.run_desc(gi, len(run_a), len(run_b), nfe_b)]
    tiled = gi.Context(0, dense_min=64)
    warp = gi.Context(0, dense_min=1 << 30)
    ft = gpu_forces(gi, torch, tiled, pos, vel, runs, p)
    fw = gpu_forces(gi, torch, warp, pos, vel, runs, p)
    ft2 = gpu_forces(gi, torch, tiled, pos, vel, runs, p)
    tiled.close()
    warp.close()
    assert np.isfinite(ft[:, :3]).all()
    assert np.array_equal(ft[:, :3], fw[:, :3])
    assert np.array_equal(ft[:, :3], ft2[:, :3])
    na = len(run_a)
    for off, n, nfe, step in ((0, na, nfe_a, 37), (na, len(run_b), nfe_b, 29)):
        idx = np.arange(off, off + n, step).astype(np.int32)
        sub_pos, sub_vel = pos[off:off + n], vel[off:off + n]
        f64, _ = orc.forces_fp64(sub_pos, sub_vel, [(0, n, nfe, 0, 0, 0, 0, 0)], p, idx=idx - off)
        err = rel_l2(ft[idx, :3], f64)
        print(f"crowded cells, run at {off}: rel L2 vs FP64 {err:.3e}")
        assert err < FORCE_TOL
