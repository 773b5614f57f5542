"""Serving loop on the GPU: runs admitted at different times and stepped in
a changing mix give bit-identical results to each run stepped alone."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("policy", [0, 1])
def test_each_result_same_alone_and_in_the_mix(gi, torch_cuda, policy):
    torch = torch_cuda
    import gi_workloads as wl
    p = wl.params(gi)
    sizes = [3000, 900, 7000, 1500, 5000]
    steps = [30, 45, 20, 60, 25]
    reqs = []
    for k, (n, ns) in enumerate(zip(sizes, steps)):
        pos, vel, nfe = gi.ic_lattice(70 + k, n, spacing=0.999, jitter=0.004, vel_sigma=1.0)
        reqs.append((pos, vel, wl.run_desc(gi, 0, n, nfe), ns))
    # policy 1 with a small fill target leaves runs out of rounds, so their
    # state must move between the two pool buffers correctly
    srv = gi.Server(p, device=0, budget_bytes=1 << 30, max_live_runs=3, steps_per_round=10,
                    policy=policy, fill_interactions=2_000_000)
    ids = {}
    for k, (pos, vel, r, ns) in enumerate(reqs):
        ids[k] = srv.submit(pos, vel, r, ns)
        if k % 2 == 1:
            srv.round()  # arrivals interleaved with rounds: the mix keeps changing
    for _ in range(60):
        if srv.stats().completed == len(reqs):
            break
        srv.round()
    assert srv.stats().completed == len(reqs)
    for k, (pos, vel, r, ns) in enumerate(reqs):
        got_p, got_v = srv.fetch(ids[k], r.n)
        c = gi.Context(0)
        dp = torch.from_numpy(pos).cuda()
        dv = torch.from_numpy(vel).cuda()
        c.step(dp.data_ptr(), dv.data_ptr(), [r], p, ns)
        torch.cuda.synchronize()
        c.close()
        assert np.array_equal(got_p, dp.cpu().numpy()), k
        assert np.array_equal(got_v, dv.cpu().numpy()), k
    srv.close()
