"""GPU tests of Earth / Moon grouping (gi_find_earth_moon) against the
oracle's literal restatement of the reference's group loop, and of the three
headless drivers against a step-by-step replay of the reference's schedule
through the library's public calls."""
from __future__ import annotations

import os

import numpy as np
import pytest

import formats_oracle as fo
from test_formats_cpu import SETUP_GENERATING, SETUP_IMPACT_INIT
from test_groups_cpu import clumps

pytestmark = pytest.mark.gpu


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _groups(gi, torch, ctx, pos, bounds, touch=1.5):
    d = _dev(torch, pos)
    n = len(pos)
    group = torch.full((max(n, 1),), -7, dtype=torch.int32, device="cuda")
    scope = torch.full((max(n, 1),), 9, dtype=torch.uint8, device="cuda")
    em = gi.find_earth_moon(ctx, d.data_ptr(), n, touch, bounds, group.data_ptr(),
                            scope.data_ptr())
    return em, group.cpu().numpy()[:n], scope.cpu().numpy()[:n]


def _check_against(em, g, sc, want_groups, orc, bounds):
    assert np.array_equal(g, want_groups)
    ref = orc.earth_moon_ref(want_groups, bounds)
    assert em.earth_label == ref["earth"] and em.moon_label == ref["moon"]
    assert em.n_earth == ref["n_earth"] and em.n_moon == ref["n_moon"]
    assert em.n_groups == ref["n_groups"]
    assert list(em.earth_counts) == ref["earth_counts"]
    assert list(em.moon_counts) == ref["moon_counts"]
    want_scope = np.where(want_groups == ref["earth"], 1, np.where(want_groups == ref["moon"], 2, 0))
    assert np.array_equal(sc, want_scope)


@pytest.mark.parametrize("case", ["clumps", "gas", "ties", "single"])
def test_groups_match_reference_loop(gi, orc, torch_cuda, case):
    torch = torch_cuda
    pos = {"clumps": lambda: clumps(1, [700, 300, 120, 5], debris=40),
           "gas": lambda: _gas(5, 2500, 23.0),
           "ties": lambda: clumps(2, [50, 50, 50]),
           "single": lambda: clumps(3, [1])}[case]()
    n = len(pos)
    bounds = [n // 5, 2 * n // 5, 3 * n // 5]
    ctx = gi.Context(0)
    em, g, sc = _groups(gi, torch, ctx, pos, bounds)
    _check_against(em, g, sc, orc.groups_ref(pos), orc, bounds)
    ctx.close()


def test_groups_repeat_on_percolating_gas(gi, orc, torch_cuda):
    """Gas near the percolation density gives long chains, where concurrent
    root walks meet most often: every repeat names every body's group as the
    reference loop does."""
    torch = torch_cuda
    ctx = gi.Context(0)
    for seed in range(20, 28):
        pos = _gas(seed, 4000, 27.0)
        n = len(pos)
        bounds = [n // 5, 2 * n // 5, 3 * n // 5]
        want = orc.groups_ref(pos)
        for _ in range(4):
            em, g, sc = _groups(gi, torch, ctx, pos, bounds)
            _check_against(em, g, sc, want, orc, bounds)
    ctx.close()


def _gas(seed, n, box):
    rng = np.random.default_rng(seed)
    pos = np.zeros((n, 4), np.float32)
    pos[:, :3] = rng.uniform(0, box, size=(n, 3))
    return pos


def test_groups_large_against_union_find(gi, orc, torch_cuda):
    """300k bodies: a dense Earth, a Moon, thousands of debris groups and far
    escapers (1e6 D), checked against the oracle's union-find."""
    torch = torch_cuda
    rng = np.random.default_rng(9)
    earth = clumps(7, [200000], spacing=1.1)
    moon = clumps(8, [20000], spacing=1.1)
    moon[:, 0] += 300.0
    gas = _gas(10, 79000, 160.0)
    gas[:, 1] += 200.0
    far = np.zeros((1000, 4), np.float32)
    far[:, :3] = rng.uniform(-1e6, 1e6, size=(1000, 3))
    pos = np.concatenate([earth, moon, gas, far])
    pos = pos[rng.permutation(len(pos))]
    n = len(pos)
    bounds = [n // 7, n // 3, n // 2]
    ctx = gi.Context(0)
    em, g, sc = _groups(gi, torch, ctx, pos, bounds)
    _check_against(em, g, sc, orc.groups_uf(pos), orc, bounds)
    assert em.n_earth == 200000 and em.n_moon == 20000
    # repeated calls give the same answer
    em2, g2, _ = _groups(gi, torch, ctx, pos, bounds)
    assert np.array_equal(g, g2) and em2.n_groups == em.n_groups
    ctx.close()


def test_groups_edge_cases(gi, torch_cuda):
    torch = torch_cuda
    ctx = gi.Context(0)
    em = gi.find_earth_moon(ctx, 0, 0, 1.5, [0, 0, 0])
    assert em.earth_label == -1 and em.moon_label == -1 and em.n_groups == 0
    buf = torch.zeros((8, 4), device="cuda")
    with pytest.raises(gi.GIError) as e:
        gi.find_earth_moon(ctx, buf.data_ptr(), 8, 0.0, [0, 0, 0])
    assert e.value.status == 1
    with pytest.raises(gi.GIError) as e:
        gi.find_earth_moon(ctx, buf.data_ptr() + 4, 7, 1.5, [0, 0, 0])
    assert e.value.status == 3
    ctx.close()


def test_disk_classification(gi, torch_cuda):
    """An Earth clump, a Moon clump and test bodies on circular orbits
    (disk), on radial infall (bound, inside) and escaping (unbound)."""
    torch = torch_cuda
    p = gi.params_from_material(1.0, 1.0, 1.0, 0.4, 5.0, 1.5, 0.02, 0.01, 0.002, 0.001)
    earth = clumps(11, [8000], spacing=1.2)[:, :3].astype(np.float64)
    earth -= earth.mean(0)
    moon = clumps(12, [500], spacing=1.2)[:, :3].astype(np.float64) + np.array([400.0, 0, 0])
    M = 8000 * 0.4  # all Si
    R = np.linalg.norm(earth, axis=1).max() + 0.5
    rng = np.random.default_rng(13)
    extra, kinds = [], []
    for kind, k in (("disk", 300), ("inside", 200), ("unbound", 100)):
        for _ in range(k):
            th, z = rng.uniform(0, 2 * np.pi), rng.uniform(-0.2, 0.2)
            r = rng.uniform(2.0, 6.0) * R
            x = np.array([r * np.cos(th), r * np.sin(th), z])
            vc = np.sqrt(M / r)
            if kind == "disk":
                v = vc * np.array([-np.sin(th), np.cos(th), 0.0])
            elif kind == "inside":
                v = -0.3 * vc * x / r
            else:
                v = 2.0 * vc * x / r
            extra.append((x, v))
            kinds.append(kind)
    n = len(earth) + len(moon) + len(extra)
    pos = np.zeros((n, 4), np.float32)
    vel = np.zeros((n, 4), np.float32)
    pos[:len(earth), :3] = earth
    pos[len(earth):len(earth) + len(moon), :3] = moon
    for k, (x, v) in enumerate(extra):
        pos[len(earth) + len(moon) + k, :3] = x
        vel[len(earth) + len(moon) + k, :3] = v
    vel[:, 3] = 0.4
    # keep the test bodies apart from one another (no accidental groups)
    ctx = gi.Context(0)
    dp, dv = _dev(torch, pos), _dev(torch, vel)
    scope = torch.zeros(n, dtype=torch.uint8, device="cuda")
    em = gi.find_earth_moon(ctx, dp.data_ptr(), n, 1.5, [0, 0, 0], None, scope.data_ptr())
    assert em.n_earth == 8000 and em.n_moon == 500
    run = gi.Run(0, n, 0, 0, 0, 0, 0, 0)
    d = gi.find_disk(ctx, dp.data_ptr(), dv.data_ptr(), run, p, scope.data_ptr())
    assert abs(d.earth_mass - M) < 1e-6 * M
    # FP64 classification of the same bodies
    sc = scope.cpu().numpy()
    c = ctx.diag(dp.data_ptr(), dv.data_ptr(), run, p, label=scope.data_ptr(), scope=2)
    com, vcom = np.array(c[1:4]), np.array(c[4:7])
    want = {"disk": 0, "inside": 0, "unbound": 0}
    for k in range(len(extra)):
        i = len(earth) + len(moon) + k
        if sc[i] in (1, 2):
            continue
        r = pos[i, :3].astype(np.float64) - com
        v = vel[i, :3].astype(np.float64) - vcom
        eps = 0.5 * v @ v - M / np.linalg.norm(r)
        req = np.sum(np.cross(r, v) ** 2) / M
        got = sc[i]
        if eps < 0 and req > d.earth_radius:
            want["disk"] += 1
            assert got == 3
        elif eps < 0:
            want["inside"] += 1
            assert got == 0
        else:
            want["unbound"] += 1
            assert got == 0
    assert (d.n_disk, d.n_bound_inside, d.n_unbound) == (want["disk"], want["inside"],
                                                        want["unbound"])
    assert d.n_disk > 250 and d.n_unbound > 80
    disk = ctx.diag(dp.data_ptr(), dv.data_ptr(), run, p, label=scope.data_ptr(), scope=4)
    assert disk[14] == d.n_disk and abs(disk[0] - float(np.float32(0.4)) * d.n_disk) < 1e-9
    ctx.close()


# ---------------------------------------------------------------- drivers --

SHORT_GENERATING = (SETUP_GENERATING.replace("DampTime = 2.0", "DampTime = 0.2")
                    .replace("DampRestTime = 1.0", "DampRestTime = 0.1")
                    .replace("SpinRestTime = 1.5", "SpinRestTime = 0.15")
                    .replace("TotalNumberOfElements = 1500", "TotalNumberOfElements = 1200"))

ADD_TIME = """* days to add
AdditionTime = 0.006;
* step
Dt = 0.003;
* screen refresh
DrawRate = 10;
* frames
RecordRate = 7;
* recentre
RecenterRate = 11;
"""


def _replay_generate(gi, torch, setup, plan, seed):
    """The body builder replayed with the public calls: damped steps, damped
    rest, force / spin / move, spin rest, drift removal."""
    b = plan.body
    pos, vel, _ = gi.raw_bodies(seed, b)
    fc, mc = gi.separate_consts_from_body_params(b, setup.dt)
    p = gi.params_from_separate_consts(fc)
    n1 = b.nfe1 + b.nsi1
    damped = [gi.Run(0, n1, b.nfe1, 0, mc.Dt, mc.DtOverMassFe, mc.DtOverMassSi, setup.damp1),
              gi.Run(n1, b.n - n1, b.nfe2, 0, mc.Dt, mc.DtOverMassFe, mc.DtOverMassSi,
                     setup.damp2)]
    rest = [gi.Run(r.offset, r.n, r.nfe, 0, r.dt, r.dt_over_mass_fe, r.dt_over_mass_si, 0.0)
            for r in damped]
    counts = fo.generate_phase_counts(setup.dt, plan.damp_time, plan.damp_rest_time,
                                      plan.spin_rest_time)
    ctx = gi.Context(0)
    dp, dv = _dev(torch, pos), _dev(torch, vel)
    force = torch.zeros_like(dp)
    if counts[0]:
        ctx.step(dp.data_ptr(), dv.data_ptr(), damped, p, counts[0])
    if counts[1]:
        ctx.step(dp.data_ptr(), dv.data_ptr(), rest, p, counts[1])
    if counts[2]:
        ctx.forces(dp.data_ptr(), dv.data_ptr(), force.data_ptr(), rest, p)
        hp, hv = dp.cpu().numpy(), dv.cpu().numpy()
        gi.spin_body(hp, hv, plan, 1, list(setup.spin1[:3]), plan.spin1_w)
        gi.spin_body(hp, hv, plan, 2, list(setup.spin2[:3]), plan.spin2_w)
        dp.copy_(torch.from_numpy(hp))
        dv.copy_(torch.from_numpy(hv))
        ctx.move(dp.data_ptr(), dv.data_ptr(), force.data_ptr(), rest)
        if counts[2] > 1:
            ctx.step(dp.data_ptr(), dv.data_ptr(), rest, p, counts[2] - 1)
    torch.cuda.synchronize()
    hp, hv = dp.cpu().numpy(), dv.cpu().numpy()
    gi.zero_drift(hp, hv, plan)
    ctx.close()
    return hp, hv, counts


def test_generate_target_impactor_matches_replay(gi, torch_cuda, tmp_path):
    torch = torch_cuda
    setup_path = tmp_path / "setupGeneratingTargetImpactor"
    setup_path.write_text(SHORT_GENERATING)
    info = tmp_path / "TargetImpactorInformation"
    info.mkdir()
    rep = gi.generate_target_impactor(str(setup_path), str(info), seed=17)
    setup = gi.read_setup_generating(str(setup_path))
    plan = gi.derive_units(setup)
    want_p, want_v, counts = _replay_generate(gi, torch, setup, plan, 17)
    assert [rep.damped_steps, rep.rest_steps, rep.spin_steps] == counts
    assert rep.steps == sum(counts) and counts[2] > 0
    pos, vel = gi.read_body_file(str(info / "targetImpactorInitialPosVel"))
    assert np.array_equal(pos, want_p) and np.array_equal(vel, want_v)
    b = gi.read_body_params(str(info / "targetImpactorParameters"))
    assert (b.n, b.nfe1, b.nsi1, b.nfe2, b.nsi2) == (plan.body.n, plan.body.nfe1, plan.body.nsi1,
                                                    plan.body.nfe2, plan.body.nsi2)
    assert (info / "targetImpactorStats").stat().st_size > 500
    # each body is centred and spinning about its own axis
    for body, axis in ((1, np.array(setup.spin1[:3])), (2, np.array(setup.spin2[:3]))):
        s, _, e = fo.body_ranges({k: getattr(b, k) for k in ("nfe1", "nsi1", "nfe2", "nsi2", "n")},
                                 body)
        m = vel[s:e, 3].astype(np.float64)
        r = pos[s:e, :3].astype(np.float64)
        v = vel[s:e, :3].astype(np.float64)
        L = (m[:, None] * np.cross(r, v)).sum(0)
        assert np.dot(L / np.linalg.norm(L), axis / np.linalg.norm(axis)) > 0.9


def test_impact_initialize_and_add_time(gi, orc, torch_cuda, tmp_path):
    torch = torch_cuda
    setup_path = tmp_path / "setupGeneratingTargetImpactor"
    setup_path.write_text(SHORT_GENERATING)
    info = tmp_path / "TargetImpactorInformation"
    info.mkdir()
    gi.generate_target_impactor(str(setup_path), str(info), seed=23)
    init_path = tmp_path / "setupImpactInitialization"
    # bodies about 48 D apart (several radii), closing at ~15 D per time unit
    init_path.write_text(SETUP_IMPACT_INIT)
    impact = tmp_path / "ImpactBin" / "run"
    (impact / "ImpactInformation").mkdir(parents=True)
    gi.impact_initialize(str(info), str(init_path), str(impact / "ImpactInformation"))
    b = gi.read_body_params(str(info / "targetImpactorParameters"))
    frames = str(impact / "ImpactInformation" / "impactPosVel")
    p0, v0 = gi.read_body_file(str(info / "targetImpactorInitialPosVel"))
    want_p, want_v = gi.impact_initial_conditions(b, gi.read_setup_impact_init(str(init_path)), p0, v0)
    t, pos, vel = gi.frames_read(frames, b.n, 0)
    assert t == 0.0 and np.array_equal(pos, want_p) and np.array_equal(vel, want_v)
    stats = gi.system_stats_host(pos, vel, b.nfe1 + b.nfe2, b.mass_fe, b.mass_si)
    view = gi.read_view_centering(str(impact / "ImpactInformation" / "viewCenteringInfo"))
    assert np.allclose(view, [float(f"{x:f}") for x in stats[1:7]], atol=1e-6)

    # add time: frames every 7 steps, recentre every 11, replayed below
    add = impact / "setupImpactAddTime"
    add.write_text(ADD_TIME)
    rep = gi.impact_add_time(str(info), str(add), str(impact))
    s = gi.read_setup_add_time(str(add))
    additional = s.additional_time_days * 86400.0 / b.unit_time
    events = fo.add_time_events(0.0, additional, s.dt, s.record_rate, s.recenter_rate)
    assert rep.steps == events[-1][0] and rep.end_time == events[-1][1]
    assert rep.frames_written == sum(e[2] for e in events)
    assert rep.recenters == sum(e[3] for e in events)
    assert gi.frames_count(frames, b.n) == 1 + rep.frames_written

    fc, mc = gi.collision_consts_from_body_params(b, s.dt)
    p = gi.params_from_collision_consts(fc)
    run = gi.Run(0, b.n, fc.NFe, 0, mc.Dt, mc.DtOverMassFe, mc.DtOverMassSi, 0.0)
    ctx = gi.Context(0)
    dp, dv = _dev(torch, want_p), _dev(torch, want_v)
    done, k_frame = 0, 1
    for k, t, rec, cen in events:
        ctx.step(dp.data_ptr(), dv.data_ptr(), [run], p, k - done)
        done = k
        if rec:
            ft, fp, fv = gi.frames_read(frames, b.n, k_frame)
            k_frame += 1
            assert ft == np.float32(t)
            assert np.array_equal(fp, dp.cpu().numpy()) and np.array_equal(fv, dv.cpu().numpy())
        if cen:
            d = ctx.diag(dp.data_ptr(), dv.data_ptr(), run, p)
            hp, hv = dp.cpu().numpy(), dv.cpu().numpy()
            vf = np.array(view, np.float32)
            hp[:, :3] += vf[:3] - np.array(d[1:4], np.float32)
            hv[:, :3] += vf[3:6] - np.array(d[4:7], np.float32)
            dp.copy_(torch.from_numpy(hp))
            dv.copy_(torch.from_numpy(hv))
    # final groups and statistics
    hp = dp.cpu().numpy()
    g = orc.groups_uf(hp, 1.5)
    ref = orc.earth_moon_ref(g, [b.nfe1, b.nfe1 + b.nfe2, b.nfe1 + b.nfe2 + b.nsi1])
    em = rep.earth_moon
    assert em.earth_label == ref["earth"] and em.n_earth == ref["n_earth"]
    assert em.n_moon == ref["n_moon"] and list(em.earth_counts) == ref["earth_counts"]
    assert rep.disk.earth_mass > 0 and rep.disk_stats[14] == rep.disk.n_disk
    text = (impact / "runStatsFile").read_text()
    assert "The mass of Earth" in text and "Angular momentum of the entire system" in text
    # a second call resumes from the last frame written
    rep2 = gi.impact_add_time(str(info), str(add), str(impact))
    last_t = gi.frames_read(frames, b.n, 1 + rep.frames_written - 1)[0]
    assert rep2.start_time == last_t
    assert gi.frames_count(frames, b.n) == 1 + rep.frames_written + rep2.frames_written
    ctx.close()
