"""Replica aggregation across ranks over gloo on CPU (world size 2)."""

import os
import socket

import torch.multiprocessing as mp


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def worker(rank, world, port, queue):
    import torch.distributed as dist

    from sand_atlas_dem_gb300.replicas import aggregate

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    out = aggregate(grain_steps=1000 * (rank + 1), seconds=0.5 + rank)
    queue.put((rank, out))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_aggregate_uses_slowest_rank():
    ctx = mp.get_context("spawn")
    queue = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=worker, args=(r, 2, port, queue)) for r in range(2)]
    for p in procs:
        p.start()
    results = dict(queue.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank in (0, 1):
        out = results[rank]
        assert out["ranks"] == 2
        assert out["grain_steps"] == 3000 and out["seconds"] == 1.5
        assert out["value"] == 2000
