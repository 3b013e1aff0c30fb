"""Multi-GPU runs are replicas only: every rank evaluates its own copy of the
workload and bench.py reports the summed atom-steps over the slowest rank's
time.  The host side of that (rank discovery, barrier, max/sum over ranks)
runs here on CPU as two gloo ranks; no data-path collective exists to test.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank_main(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    d = bench.Dist("gloo")
    d.barrier()
    t_slowest = d.max(1.0 + rank)             # per-rank "step time"
    atoms = d.sum(100.0 * (rank + 1))         # per-rank units of work
    d.barrier()
    d.close()
    q.put((rank, t_slowest, atoms))


def test_two_gloo_ranks_reduce_like_bench():
    torch = pytest.importorskip("torch")
    import multiprocessing as mp
    import socket
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(60)
        assert p.exitcode == 0
    # max over ranks of the time, sum over ranks of the work
    assert out == [(0, 2.0, 300.0), (1, 2.0, 300.0)]
    assert torch is not None


def test_single_rank_defaults():
    sys.path.insert(0, ROOT)
    import bench
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        os.environ.pop(k, None)
    assert bench.dist_env() == (0, 1, 0)
    d = bench.Dist("gloo")
    assert d.max(3.5) == 3.5 and d.sum(2.0) == 2.0
    d.close()
