"""Replicas across GPUs: each rank renders its own frames on its own copy of
the BVH (rays are independent; no collective on the data path).

shard() splits a list of work items (cameras, frames, requests) across ranks;
reduce_timing() combines per-rank step times and ray counts the way the
benchmark reports them (max time over ranks, sum of rays).
"""
from __future__ import annotations


def shard(n_items: int, rank: int, world: int) -> range:
    """Contiguous share of [0, n_items) for `rank` (sizes differ by at most 1)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"bad rank {rank} of {world}")
    base, extra = divmod(n_items, world)
    start = rank * base + min(rank, extra)
    return range(start, start + base + (1 if rank < extra else 0))


def reduce_timing(ms: float, rays: int) -> tuple[float, int]:
    """(max ms over ranks, total rays over ranks); identity without a process group."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return ms, rays
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([ms], dtype=torch.float64, device=dev)
    r = torch.tensor([rays], dtype=torch.int64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(r, op=dist.ReduceOp.SUM)
    return float(t.item()), int(r.item())
