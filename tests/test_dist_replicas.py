"""The N > 1 path of the benchmark is replicas: every rank runs its own copy of
the step, the job's time is the slowest rank's and its rate the sum.  The
rank plumbing (process group, barrier, max over ranks) is exercised here with
two gloo ranks on the CPU."""
from __future__ import annotations

import os
import socket

import pytest

torch = pytest.importorskip("torch")
mp = pytest.importorskip("torch.multiprocessing")


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    import bench
    d = bench.Dist()
    try:
        d.barrier()
        # rank r "took" 1 + r seconds: the job time is the slowest rank's
        t = d.max(1.0 + rank)
        out.put((rank, d.world, t, bench.whole_job_rate(1_000_000, 10, d.world, t)))
    finally:
        d.close()


def test_two_gloo_ranks_take_the_max_time_and_sum_the_work():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[0] for r in res] == [0, 1]
    for _, world, t, rate in res:
        assert world == 2
        assert t == 2.0
        assert rate == pytest.approx(1_000_000 * 10 * 2 / 2.0 / 1e6)


def test_single_process_needs_no_process_group():
    import bench
    for k in ("RANK", "WORLD_SIZE"):
        os.environ.pop(k, None)
    d = bench.Dist()
    assert d.world == 1 and d.rank == 0 and d.pg is None
    assert d.max(3.5) == 3.5
    assert bench.whole_job_rate(4194304, 5, 1, 0.1) == pytest.approx(4194304 * 5 / 0.1 / 1e6)
