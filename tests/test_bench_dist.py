"""bench.py's multi-rank aggregation (replicas, max over ranks) on two gloo ranks on the CPU."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    import torch
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    def reduce_max(x):
        t = torch.tensor([x], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    # rank r took (r + 1) seconds for 3 frames of 1000 samples
    value, seconds = bench.aggregate(1000, 3, world, float(rank + 1), reduce_max)
    q.put((rank, value, seconds))
    dist.barrier()
    dist.destroy_process_group()


def test_aggregate_replicas_max_over_ranks():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, value, seconds in res:
        assert seconds == 2.0  # the slowest rank
        assert value == pytest.approx(1000 * 3 * world / 2.0)


def test_aggregate_single_rank():
    import bench
    assert bench.aggregate(100, 4, 1, 2.0) == (200.0, 2.0)
