"""Replica sharding and the max-over-ranks timing, with gloo ranks on CPU."""
import os

import pytest
import torch.multiprocessing as mp

from j3d_gb300.multi import reduce_timing, shard


def test_shard_covers_everything_once():
    for n in (0, 1, 5, 32, 33):
        for world in (1, 2, 3, 8):
            parts = [shard(n, r, world) for r in range(world)]
            items = [i for p in parts for i in p]
            assert items == list(range(n))
            assert max(len(p) for p in parts) - min(len(p) for p in parts) <= 1
    with pytest.raises(ValueError):
        shard(4, 2, 2)


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    cams = list(shard(32, rank, world))
    ms = 10.0 + rank  # rank 1 is the slower one
    rays = 1000 * len(cams)
    q.put((rank, cams, reduce_timing(ms, rays)))
    dist.destroy_process_group()


def test_two_gloo_ranks_reduce_like_the_bench():
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
    (r0, c0, t0), (r1, c1, t1) = out
    assert c0 == list(range(16)) and c1 == list(range(16, 32))
    assert t0 == t1 == (11.0, 32000)


def test_single_process_is_identity():
    assert reduce_timing(3.5, 7) == (3.5, 7)
