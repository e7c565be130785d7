"""bench.py's replica bookkeeping over two gloo ranks on the CPU: the job's
timed interval is the slowest rank's on every rank, the rate counts every
rank's units, and the barrier and teardown complete on both ranks."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(r, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port),
                      WORLD_SIZE="2", RANK=str(r), LOCAL_RANK=str(r))
    sys.path.insert(0, ROOT)
    import bench
    ranks = bench.Ranks(backend="gloo")
    t = ranks.max(1.5 + r)  # rank 1 is the slower one
    ranks.barrier()
    rate = bench.job_rate(1000.0, ranks.world, t)
    ranks.close()
    out.put((r, ranks.world, t, rate))


def test_two_gloo_ranks_take_the_slowest_time():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=180)
    for p in procs:
        if p.is_alive():
            p.kill()
    assert [p.exitcode for p in procs] == [0, 0]
    got = sorted(q.get(timeout=10) for _ in range(2))
    for r, world, t, rate in got:
        assert world == 2
        assert t == 2.5
        assert rate == pytest.approx(1000.0 * 2 / 2.5)


def test_one_rank_needs_no_process_group(monkeypatch):
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    sys.path.insert(0, ROOT)
    import bench
    ranks = bench.Ranks()
    assert ranks.world == 1 and ranks.max(3.25) == 3.25
    ranks.barrier()
    ranks.close()
    assert bench.job_rate(10.0, 1, 2.0) == 5.0
