"""The bench's multi-rank path on CPU: two gloo ranks launched like
torchrun (RANK / WORLD_SIZE / MASTER_* in the environment).  The timed
region is the slowest rank's, the whole-job value sums the replicas, and
the reference arm runs on rank 0 only (the other ranks exit at once)."""
from __future__ import annotations

import importlib.util
import os
import socket

import pytest
import torch.multiprocessing as mp

from conftest import ROOT


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _load_bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _rank(rank, world, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist
    bench = _load_bench()
    r, local, w = bench.dist_setup("gloo")
    got = {"rank": r, "world": w}
    # rank k took (k + 1) * 100 ms: the job is timed by the slowest
    got["max_ms"] = bench.max_over_ranks((r + 1) * 100.0)
    got["value"] = bench.replica_value(1000, 10, got["max_ms"], w)
    if r != 0:
        import sys
        saved = sys.argv
        sys.argv = ["bench.py", "--impl", "reference"]
        try:
            got["reference_arm"] = bench.run_reference(bench.args_parse())
        finally:
            sys.argv = saved
    dist.barrier()
    out[r] = got
    dist.destroy_process_group()


def test_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        port = _free_port()
        procs = [ctx.Process(target=_rank, args=(k, 2, port, out)) for k in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(timeout=120)
        codes = [p.exitcode for p in procs]
        res = dict(out)
    assert codes == [0, 0], codes
    for r in (0, 1):
        assert res[r]["world"] == 2 and res[r]["max_ms"] == 200.0
        assert res[r]["value"] == pytest.approx(2 * 1000 * 10 / 0.2)
    assert res[1]["reference_arm"] is None  # only rank 0 runs and prints the reference arm


def test_single_process_defaults():
    bench = _load_bench()
    assert bench.max_over_ranks(3.5) == 3.5
    assert bench.replica_value(4_355_934_000, 40, 72.5, 1) == pytest.approx(4_355_934_000 * 40 / 0.0725)
