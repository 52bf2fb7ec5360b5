"""Trajectory sharding across processes (one process per GPU).

Trajectories are independent, so an ensemble splits into contiguous shards with no
data-path collective; the only exchange is the host gather of (ts, us) -- the analogue
of the reference's `pmap` over batches and `vcat` of the results (src/solve.jl:109-160).
Each shard passes its first global index as `traj_offset`, so that noise streams (GPUEM)
and any per-trajectory derivation are identical whatever the shard count.
"""
from __future__ import annotations

import numpy as np


def shard_range(B: int, world: int, rank: int) -> range:
    """Contiguous shard of trajectory indices for `rank` (sizes differ by at most one)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad world/rank")
    base, extra = divmod(B, world)
    start = rank * base + min(rank, extra)
    return range(start, start + base + (1 if rank < extra else 0))


def gather_to_rank0(arrays, group=None):
    """Gather per-rank numpy arrays (first axis = trajectories, possibly ragged) on rank 0
    with torch.distributed (gloo or nccl); returns the concatenation on rank 0, None elsewhere."""
    import torch
    import torch.distributed as dist
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    n = torch.tensor([arrays.shape[0]], dtype=torch.int64)
    sizes = [torch.zeros(1, dtype=torch.int64) for _ in range(world)]
    dist.all_gather(sizes, n, group=group)
    maxn = int(max(s.item() for s in sizes))
    pad = np.zeros((maxn,) + arrays.shape[1:], dtype=arrays.dtype)
    pad[: arrays.shape[0]] = arrays
    t = torch.from_numpy(pad)
    out = [torch.zeros_like(t) for _ in range(world)] if rank == 0 else None
    dist.gather(t, out, dst=0, group=group)
    if rank != 0:
        return None
    return np.concatenate([o.numpy()[: int(s.item())] for o, s in zip(out, sizes)])
