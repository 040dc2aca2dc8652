"""Multi-GPU path on CPU: the residual/RK4 path does not shard, so N GPUs run N
independent replicas; bench.py combines their timings with a max over ranks and
their work with a sum. World-size-2 gloo ranks check that combination."""
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
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    t = bench.max_over_ranks(dist, 1.0 + rank)  # rank r reports 1 + r seconds
    bench.barrier(dist)
    q.put((rank, t))
    dist.destroy_process_group()


def test_replica_timing_is_max_over_ranks():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = dict(q.get(timeout=10) for _ in range(world))
    assert res == {0: 2.0, 1: 2.0}
