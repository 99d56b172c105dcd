"""Replica path of bench.py (one independent sweep per rank, max-over-ranks
timing) on two gloo ranks on the CPU."""
import os
import socket
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, REPO)
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        t = [2.0, 3.0][rank]                     # rank 1 is the slow replica
        q.put((rank, bench.max_over_ranks(t), bench.replica_throughput(722.0, t)))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_gloo_replicas():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    for rank, tmax, value in got:
        assert tmax == 3.0
        assert value == pytest.approx(722.0 * 2 / 3.0)
