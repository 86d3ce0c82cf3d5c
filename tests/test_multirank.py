"""N > 1 replicas: the bench's max-over-ranks aggregation on 2 gloo ranks (CPU)."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    v = bench.reduce_max_over_ranks(1.5 + rank)  # rank 1 is the slowest replica
    q.put((rank, v))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_take_max():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = dict(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out == {0: 2.5, 1: 2.5}


def test_single_rank_identity():
    import bench
    assert bench.reduce_max_over_ranks(3.25) == 3.25
