"""Replica aggregation of bench.py across ranks (world size 2, gloo, CPU):
the job's time is the slowest rank's and its value counts every rank's work."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch.distributed as tdist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    tdist.init_process_group("gloo", rank=rank, world_size=world)
    ms = 10.0 if rank == 0 else 25.0  # rank 1 is the slow replica
    value, ms_max = bench.aggregate(1000.0, ms, world)
    tdist.barrier()
    tdist.destroy_process_group()
    q.put((rank, value, ms_max))


def test_two_replicas_take_the_slowest_time():
    torch = pytest.importorskip("torch")
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    got = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, value, ms_max in got:
        assert ms_max == 25.0
        assert abs(value - 2 * 1000.0 / 0.025) < 1e-6


def test_single_process_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    value, ms = bench.aggregate(500.0, 5.0, 1)
    assert ms == 5.0 and abs(value - 100000.0) < 1e-9
