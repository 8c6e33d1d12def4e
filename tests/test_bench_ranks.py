"""The multi-GPU path is replicas (queries shard by query, no collective on
the data path); its only cross-rank step is the timing reduction of
bench.py, checked here with two gloo ranks on CPU."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, q):
    import torch
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    t_dev, wall, n = bench.reduce_over_ranks(dist, torch, 1.0 + rank, 2.0 + 3 * rank,
                                             1000, "cpu")
    q.put((rank, t_dev, wall, n))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_timing_reduction_two_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in range(2))
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t_dev, wall, n in out:
        assert t_dev == 2.0 and wall == 5.0 and n == 2000
