"""Failure paths on the GPU, made on the host (no GPU fault, trap or hang):

  * the persistent force kernel's work queue and split tickets, overwritten
    between calls as a launch that was cut short would leave them: the next
    call must still be right, because every launch clears them first;
  * the Earth / Moon union-find given one attempt per link on a clump where
    thousands of links race for the same roots: the bounded loop runs out,
    the call reports GI_ERR_TIMEOUT, and the context stays usable;
  * a serving-loop request cancelled while live: the other runs keep their
    bits, and a new run reuses the freed range.

The reference has no counterpart to any of these: it stops the process on
the first CUDA error (commonFunctions.h:12-22) and groups on the host
(impactBasicFunctions.h:124-152)."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

GI_ERR_TIMEOUT = 5


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("pattern", [0x01010101, 0x7F7F7F7F])
@pytest.mark.parametrize("n", [3000, 20000, 140000])
def test_forces_right_after_counters_overwritten(gi, orc, torch_cuda, n, pattern):
    """Both byte patterns read as queue positions past the end of any table
    (so a kernel that trusted them would skip every work item) and as split
    tickets that never come round (so no i-block would be finished).  The
    call after the overwrite uses other bodies than the call before it, so
    left-over sums cannot pass for a result.  n = 140,000 takes the serial
    contact path (n^2 >= 2^34), the others the side-by-side one."""
    torch = torch_cuda
    import gi_workloads as wl
    p = wl.params(gi)
    s = torch.cuda.current_stream().cuda_stream
    ctx = gi.Context(0, accum=gi.GI_ACCUM_KAHAN)  # the one-sided kernel's queue
    ctx.set_tuning(2, 1024)  # split j-chunks: tickets and partial sums in use
    pa, va, nfe_a = gi.ic_lattice(11, n, spacing=0.999, jitter=0.004, vel_sigma=1.0)
    pb, vb, nfe_b = gi.ic_lattice(12, n, spacing=1.001, jitter=0.006, vel_sigma=0.7)
    da, dva = _dev(torch, pa), _dev(torch, va)
    df = torch.zeros_like(da)
    ctx.forces(da.data_ptr(), dva.data_ptr(), df.data_ptr(), [wl.run_desc(gi, 0, n, nfe_a)], p, s)
    torch.cuda.synchronize()
    ctx.fill_counters(pattern, s)
    db, dvb = _dev(torch, pb), _dev(torch, vb)
    df.fill_(float("nan"))
    run_b = wl.run_desc(gi, 0, n, nfe_b)
    ctx.forces(db.data_ptr(), dvb.data_ptr(), df.data_ptr(), [run_b], p, s)
    torch.cuda.synchronize()
    got = df.cpu().numpy()
    fresh = gi.Context(0, accum=gi.GI_ACCUM_KAHAN)
    fresh.set_tuning(2, 1024)
    dfr = torch.zeros_like(db)
    fresh.forces(db.data_ptr(), dvb.data_ptr(), dfr.data_ptr(), [run_b], p, s)
    torch.cuda.synchronize()
    want = dfr.cpu().numpy()
    assert np.array_equal(got[:, :3], want[:, :3])
    # and the fused step after another overwrite
    ctx.fill_counters(pattern, s)
    ctx.step(db.data_ptr(), dvb.data_ptr(), [run_b], p, 2, s)
    fp, fv = _dev(torch, pb), _dev(torch, vb)
    fresh.step(fp.data_ptr(), fv.data_ptr(), [run_b], p, 2, s)
    torch.cuda.synchronize()
    assert torch.equal(db, fp) and torch.equal(dvb, fv)
    idx = np.arange(0, n, max(1, n // 512)).astype(np.int32)
    f64, _ = orc.forces_fp64(pb, vb, [run_b], p, idx=idx)
    assert rel_l2(got[idx, :3], f64) < 1e-5
    ctx.close()
    fresh.close()


def _clump(seed, n, radius):
    """n points inside a ball of the given radius: every pair is closer than
    2 radius, so with radius < 0.75 every pair touches at 1.5."""
    rng = np.random.default_rng(seed)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r = radius * rng.uniform(0, 1, size=(n, 1)) ** (1 / 3)
    out = np.zeros((n, 4), np.float32)
    out[:, :3] = d * r
    return out


def test_union_find_tries_run_out_and_context_recovers(gi, orc, torch_cuda):
    """One attempt per link on 4,096 mutually touching bodies: the threads of
    a warp that link to the same body try to re-hang the same root in one
    instruction, all but one fail, and with no retry left the call must
    report GI_ERR_TIMEOUT instead of groups.  With the default limit the same
    context then groups the clump (and a two-clump case) as the reference
    loop does."""
    torch = torch_cuda
    pos = _clump(31, 4096, 0.7)
    n = len(pos)
    bounds = [n // 4, n // 2, 3 * n // 4]
    ctx = gi.Context(0, cluster_tries=1)
    d = _dev(torch, pos)
    with pytest.raises(gi.GIError) as e:
        gi.find_earth_moon(ctx, d.data_ptr(), n, 1.5, bounds)
    assert e.value.status == GI_ERR_TIMEOUT
    ctx.set_options(cluster_tries=0)
    em = gi.find_earth_moon(ctx, d.data_ptr(), n, 1.5, bounds)
    assert em.n_groups == 1 and em.n_earth == n and em.earth_label == 0
    two = np.concatenate([pos, _clump(32, 1000, 0.7) + np.float32([50.0, 0, 0, 0])])
    two = two[np.random.default_rng(3).permutation(len(two))]
    d2 = _dev(torch, two)
    group = torch.full((len(two),), -1, dtype=torch.int32, device="cuda")
    em2 = gi.find_earth_moon(ctx, d2.data_ptr(), len(two), 1.5, bounds, group.data_ptr())
    assert np.array_equal(group.cpu().numpy(), orc.groups_ref(two))
    assert (em2.n_earth, em2.n_moon, em2.n_groups) == (4096, 1000, 2)
    # the force path of the same context still works
    import gi_workloads as wl
    pw, vw, nfe = gi.ic_lattice(5, 2048, spacing=0.999, jitter=0.004, vel_sigma=1.0)
    run = wl.run_desc(gi, 0, 2048, nfe)
    dp, dv = _dev(torch, pw), _dev(torch, vw)
    df = torch.zeros_like(dp)
    ctx.forces(dp.data_ptr(), dv.data_ptr(), df.data_ptr(), [run], wl.params(gi))
    torch.cuda.synchronize()
    f64, _ = orc.forces_fp64(pw, vw, [run], wl.params(gi))
    assert rel_l2(df.cpu().numpy()[:, :3], f64) < 1e-5
    ctx.close()


def test_cancel_live_run_leaves_others_bit_identical(gi, torch_cuda):
    """Four runs live together; one is cancelled mid-way and a fifth is
    admitted into the freed range.  Every finished run equals the same run
    stepped alone, bit for bit."""
    torch = torch_cuda
    import gi_workloads as wl
    p = wl.params(gi)
    sizes, steps = [2500, 4000, 1200, 3300, 2400], [40, 30, 50, 40, 30]
    reqs = []
    for k, (n, ns) in enumerate(zip(sizes, steps)):
        pos, vel, nfe = gi.ic_lattice(90 + k, n, spacing=0.999, jitter=0.004, vel_sigma=1.0)
        reqs.append((pos, vel, wl.run_desc(gi, 0, n, nfe), ns))
    srv = gi.Server(p, device=0, budget_bytes=1 << 30, max_live_runs=4, steps_per_round=10)
    ids = [srv.submit(pos, vel, r, ns) for pos, vel, r, ns in reqs[:4]]
    srv.round()
    srv.round()
    assert srv.query(ids[1]).state == gi.REQ_LIVE
    srv.cancel(ids[1])
    ids.append(srv.submit(*reqs[4][:3], reqs[4][3]))
    for _ in range(20):
        if srv.stats().live == 0 and srv.stats().queued == 0:
            break
        srv.round()
    st = srv.stats()
    assert st.completed == 4 and st.cancelled == 1 and st.bytes_in_use == 0
    for k in (0, 2, 3, 4):
        pos, vel, r, ns = reqs[k]
        got_p, got_v = srv.fetch(ids[k], r.n)
        c = gi.Context(0)
        dp, dv = _dev(torch, pos), _dev(torch, vel)
        c.step(dp.data_ptr(), dv.data_ptr(), [r], p, ns)
        torch.cuda.synchronize()
        c.close()
        assert np.array_equal(got_p, dp.cpu().numpy()), k
        assert np.array_equal(got_v, dv.cpu().numpy()), k
    srv.close()
