"""Replica parallelism for droplet batches (multi-GPU without a data-path collective).

Droplets are independent (the reference itself is single-GPU, one process per parameter set), so
N GPUs run N independent batches: `shard` splits a sweep's droplet list across ranks (strong
scaling of a fixed sweep), or every rank runs the full list (weak scaling, as bench.py does). The
only collectives are host-side bookkeeping: a barrier around timed regions and the maximum of the
per-rank times. Works with the gloo (CPU) and nccl (GPU) backends.
"""
from __future__ import annotations

import os


def env_rank():
    """(rank, world_size, local_rank) from the torchrun environment (defaults: a single process)."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def shard(items, rank: int, world: int):
    """Round-robin share of `items` for `rank` (every item goes to exactly one rank)."""
    if world <= 0 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    return list(items)[rank::world]


def balanced_shard(sizes, rank: int, world: int):
    """Indices of droplets for `rank`, greedy by site count (largest first onto the least loaded rank)."""
    order = sorted(range(len(sizes)), key=lambda i: -sizes[i] ** 3)
    load = [0] * world
    owner = [0] * len(sizes)
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        owner[i] = r
        load[r] += sizes[i] ** 3
    return [i for i in range(len(sizes)) if owner[i] == rank]


def max_over_ranks(value: float, device=None) -> float:
    """Maximum of a per-rank float over the default process group (the value itself without one)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device or "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value: float, device=None) -> float:
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device or "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())
