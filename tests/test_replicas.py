"""Replica logic on CPU: disjoint view shards and max-over-ranks timing with
world_size 2 over gloo (no GPU)."""
import os

import pytest
import torch.multiprocessing as mp

from renderer_ray_marching_gb300.replicas import max_over_ranks, shard


def test_shard_is_disjoint_and_covering():
    items = list(range(257))
    for world in (1, 2, 3, 8):
        parts = [shard(items, r, world) for r in range(world)]
        flat = sorted(x for p in parts for x in p)
        assert flat == items
        assert max(len(p) for p in parts) - min(len(p) for p in parts) <= 1
    with pytest.raises(ValueError):
        shard(items, 2, 2)


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    views = list(range(10))
    mine = shard(views, rank, world)
    slowest = max_over_ranks(1.0 + rank)
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, mine, slowest))


def test_two_rank_gloo_max_over_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + (os.getpid() % 2000)
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out[0][1] == [0, 2, 4, 6, 8] and out[1][1] == [1, 3, 5, 7, 9]
    assert out[0][2] == 2.0 and out[1][2] == 2.0
