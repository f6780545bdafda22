"""bench.py's multi-rank bookkeeping on CPU: two gloo ranks, each with its
own particle count and time, give the whole-job sum of particles and the
slowest rank's time on every rank (the figures the bench's value is made
of when torchrun launches one rank per GPU)."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    ws, r, local = bench.dist_env()
    sums, maxes = bench.aggregate_ranks([1000 + 7 * rank, 1.0], [0.5 + rank, -rank], device="cpu")
    q.put((rank, ws, r, local, sums, maxes))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_aggregation():
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(k, world, port, q)) for k in range(world)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ws, r, local, sums, maxes in out:
        assert ws == world and r == rank and local == rank
        assert sums == [1000.0 + 1007.0, 2.0]
        assert maxes == [1.5, 0.0]


def test_single_rank_passthrough():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.aggregate_ranks([3, 4], [5], device="cpu") == ([3.0, 4.0], [5.0])
