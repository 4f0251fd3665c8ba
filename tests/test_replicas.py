"""The multi-GPU path of bench.py is independent replicas (one scene has no
partition without halo exchanges every neighbour build and CG iteration):
each rank times its own steps and the job's time is the slowest rank's.
This checks that aggregation with world size 2 over gloo on the CPU."""
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, out):
    import torch.distributed as dist

    sys.path.insert(0, REPO)
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sec = 1.0 + rank  # rank 1 is the slow one
    t = bench.max_over_ranks(sec, dist)
    v = bench.replica_throughput(1000, 10, t, world)
    out.put((rank, t, v))
    dist.destroy_process_group()


def test_two_replica_ranks_report_the_slowest_time():
    mp = pytest.importorskip("torch.multiprocessing")
    import socket

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [2.0, 2.0]
    assert all(abs(r[2] - 2 * 1000 * 10 / 2.0) < 1e-9 for r in res)
