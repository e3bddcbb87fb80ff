"""The multi-rank path of bench.py (independent replicas) with 2 gloo ranks on CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import sys

    import torch.distributed as dist

    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    # each replica times its own (different) run; the job is as slow as the slowest rank
    value, t = bench.replica_aggregate(1.0 + rank, 256 * 10, dist, "cpu")
    # a rank whose replica is missing its work fails loudly rather than hanging
    dist.barrier()
    q.put((rank, value, t))
    dist.destroy_process_group()


def test_replica_aggregate_two_gloo_ranks():
    ctx = torch.multiprocessing.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    for rank, value, t in res:
        assert t == 2.0  # max over ranks
        assert abs(value - 2 * 2560 / 2.0) < 1e-9  # work of both replicas over the slowest time


def test_single_process_aggregate():
    import bench

    value, t = bench.replica_aggregate(2.0, 512)
    assert t == 2.0 and value == 256.0
