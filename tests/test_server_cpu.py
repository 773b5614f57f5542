"""Scheduling logic of the serving loop, run without a GPU (dry-run server):
admission by HBM budget and slots, FIFO order, exact step counts across
rounds, pool reuse and accounting."""
from __future__ import annotations

import numpy as np
import pytest


def bodies(n, seed=0):
    rng = np.random.default_rng(seed)
    return rng.normal(size=(n, 4)).astype(np.float32), rng.normal(size=(n, 4)).astype(np.float32)


def run(gi, n, nfe=None):
    return gi.Run(0, n, n // 3 if nfe is None else nfe, 0, 1e-3, 1e-3, 2.5e-3, 0.0)


@pytest.fixture
def params(gi):
    return gi.params_from_material()


def test_budget_limits_live_runs_fifo(gi, params):
    n = 1000
    per_run = 2 * 2 * 16 * n  # two state buffers of pos + vel
    srv = gi.Server(params, device=gi.SERVER_DRY_RUN, budget_bytes=2 * per_run, max_live_runs=8,
                    steps_per_round=10)
    ids = [srv.submit(*bodies(n, k), run(gi, n), 25) for k in range(3)]
    assert srv.round() == 0
    st = srv.stats()
    assert (st.live, st.queued, st.bytes_in_use) == (2, 1, 2 * per_run)
    assert [srv.query(i).state for i in ids] == [gi.REQ_LIVE, gi.REQ_LIVE, gi.REQ_QUEUED]
    assert srv.round() == 0
    assert srv.round() == 2          # 25 steps = 10 + 10 + 5
    assert srv.query(ids[0]).steps_done == 25
    assert srv.query(ids[2]).state == gi.REQ_QUEUED  # admitted at the next round
    srv.round()
    assert srv.query(ids[2]).state == gi.REQ_LIVE
    for _ in range(3):
        srv.round()
    assert srv.query(ids[2]).state == gi.REQ_DONE
    st = srv.stats()
    assert st.completed == 3 and st.live == 0 and st.bytes_in_use == 0
    assert st.interactions == 3 * 25 * n * (n - 1)
    p, v = srv.fetch(ids[0], n)
    assert np.array_equal(p, bodies(n, 0)[0])  # dry run leaves the state as it was
    with pytest.raises(gi.GIError):
        srv.query(ids[0])  # fetched requests are forgotten


def test_slots_and_head_of_line(gi, params):
    srv = gi.Server(params, device=gi.SERVER_DRY_RUN, budget_bytes=10**9, max_live_runs=2,
                    steps_per_round=7)
    ids = [srv.submit(*bodies(100 + k), run(gi, 100 + k), 7) for k in range(5)]
    srv.round()
    assert srv.stats().completed == 2 and srv.stats().queued == 3
    big = gi.Server(params, device=gi.SERVER_DRY_RUN, budget_bytes=64 * 1000, max_live_runs=8,
                    steps_per_round=5)
    a = big.submit(*bodies(600), run(gi, 600), 10)   # 38,400 bytes
    b = big.submit(*bodies(500), run(gi, 500), 10)   # 32,000: does not fit beside a
    c = big.submit(*bodies(10), run(gi, 10), 10)     # would fit, but waits behind b (FIFO)
    big.round()
    assert [big.query(i).state for i in (a, b, c)] == [gi.REQ_LIVE, gi.REQ_QUEUED, gi.REQ_QUEUED]
    with pytest.raises(gi.GIError) as e:
        big.submit(*bodies(2000), run(gi, 2000), 1)  # more than the whole budget
    assert e.value.status == 11


def test_pool_reuse_and_zero_step_runs(gi, params):
    srv = gi.Server(params, device=gi.SERVER_DRY_RUN, budget_bytes=10**10, max_live_runs=4,
                    steps_per_round=3)
    for wave in range(5):
        ids = [srv.submit(*bodies(2000 + 37 * k), run(gi, 2000 + 37 * k), 3) for k in range(4)]
        srv.round()
        assert all(srv.query(i).state == gi.REQ_DONE for i in ids)
    assert srv.stats().pool_bodies <= 65536  # ranges are reused, the pool does not creep
    z = srv.submit(*bodies(5), run(gi, 5), 0)
    srv.round()
    assert srv.query(z).state == gi.REQ_DONE and srv.query(z).steps_done == 0


def test_bad_requests(gi, params):
    srv = gi.Server(params, device=gi.SERVER_DRY_RUN, budget_bytes=10**6)
    with pytest.raises(gi.GIError):
        srv.submit(*bodies(10), gi.Run(0, 10, 11, 0, 0, 0, 0, 0), 5)
    with pytest.raises(gi.GIError):
        srv.submit(*bodies(10), gi.Run(0, 10, 1, 3, 0, 0, 0, 0), 5)
    with pytest.raises(gi.GIError):
        srv.submit(*bodies(10), run(gi, 10), -1)


def test_shortest_remaining_work_first(gi, params):
    """GI_SERVE_SHORTEST steps the live runs with the least remaining work
    (steps left x N^2) until a step's pair count reaches the fill target;
    the others wait.  Every run still gets exactly its steps."""
    # fill at 1 interaction: one run per step, the cheapest first
    srv = gi.Server(params, device=gi.SERVER_DRY_RUN, budget_bytes=10**9, max_live_runs=8,
                    steps_per_round=10, policy=gi.SERVE_SHORTEST, fill_interactions=1)
    big = srv.submit(*bodies(3000), run(gi, 3000), 20)
    small = srv.submit(*bodies(300), run(gi, 300), 30)
    mid = srv.submit(*bodies(1000), run(gi, 1000), 20)
    srv.round()
    q = {k: srv.query(i) for k, i in (("big", big), ("small", small), ("mid", mid))}
    assert (q["small"].steps_done, q["mid"].steps_done, q["big"].steps_done) == (10, 0, 0)
    for _ in range(2):
        srv.round()
    assert srv.query(small).state == gi.REQ_DONE       # 30 steps in the first 3 rounds
    assert srv.query(mid).steps_done == 0 and srv.query(big).steps_done == 0
    for _ in range(2):
        srv.round()
    assert srv.query(mid).state == gi.REQ_DONE and srv.query(big).steps_done == 0
    for _ in range(2):
        srv.round()
    assert srv.query(big).state == gi.REQ_DONE
    st = srv.stats()
    assert st.interactions == 20 * 3000 * 2999 + 30 * 300 * 299 + 20 * 1000 * 999
    # a fill target of the two smaller runs' pair count steps both of them together
    srv2 = gi.Server(params, device=gi.SERVER_DRY_RUN, budget_bytes=10**9, max_live_runs=8,
                     steps_per_round=10, policy=gi.SERVE_SHORTEST,
                     fill_interactions=300 * 299 + 1000 * 999)
    ids = [srv2.submit(*bodies(n), run(gi, n), 10) for n in (3000, 300, 1000)]
    srv2.round()
    assert [srv2.query(i).steps_done for i in ids] == [0, 10, 10]
    with pytest.raises(gi.GIError):
        gi.Server(params, device=gi.SERVER_DRY_RUN, budget_bytes=10**9, policy=7)


def test_cancel_frees_slot_and_budget(gi, params):
    """A cancelled request gives its slot and budget back at once: a live
    run's range returns to the pool, a queued request leaves the queue, and
    the others keep their exact step counts."""
    n = 1000
    per_run = 2 * 2 * 16 * n
    srv = gi.Server(params, device=gi.SERVER_DRY_RUN, budget_bytes=2 * per_run, max_live_runs=2,
                    steps_per_round=10)
    a, b, c, d = (srv.submit(*bodies(n, k), run(gi, n), 30) for k in range(4))
    srv.round()
    assert [srv.query(i).state for i in (a, b, c, d)] == [gi.REQ_LIVE, gi.REQ_LIVE,
                                                          gi.REQ_QUEUED, gi.REQ_QUEUED]
    srv.cancel(a)                      # live: slot, range and budget come back now
    st = srv.stats()
    assert (st.live, st.queued, st.bytes_in_use, st.cancelled) == (1, 2, per_run, 1)
    with pytest.raises(gi.GIError):
        srv.query(a)                   # forgotten
    srv.cancel(d)                      # queued: leaves the queue
    assert srv.stats().queued == 1
    srv.round()                        # c takes a's slot
    assert srv.query(c).state == gi.REQ_LIVE
    assert srv.query(b).steps_done == 20 and srv.query(c).steps_done == 10
    while srv.stats().live:
        srv.round()
    assert srv.query(b).steps_done == 30 and srv.query(c).steps_done == 30
    st = srv.stats()
    assert (st.completed, st.cancelled, st.bytes_in_use) == (2, 2, 0)
    srv.cancel(b)                      # a finished result is discarded
    with pytest.raises(gi.GIError):
        srv.fetch(b, n)
    with pytest.raises(gi.GIError) as e:
        srv.cancel(12345)              # unknown id
    assert e.value.status == 1  # GI_ERR_INVALID_ARG
    # the pool ranges handed back are reused: a fresh pair fits where a and b were
    e1, e2 = (srv.submit(*bodies(n, 9 + k), run(gi, n), 5) for k in range(2))
    srv.round()
    assert srv.query(e1).state == gi.REQ_DONE and srv.query(e2).state == gi.REQ_DONE
    assert srv.stats().pool_bodies <= 65536
