"""Data-parallel replicas: independent solves split round-robin over ranks, one GPU each.

Energies × configurations × systems are independent and T is a scalar per solve, so there is no
exchange on the data path. Each rank solves its share on its own device, and the results meet on
the host at the end (the CLI gathers the same way over its configuration loop,
`crates/caroli-cli/src/run.rs:41-45`). Works with any `torch.distributed` backend (NCCL between
GPUs, gloo on CPUs).
"""
from __future__ import annotations


def shard(items, rank, world):
    """The items of `rank` (round-robin) and their positions in `items`."""
    idx = list(range(rank, len(items), world))
    return [items[i] for i in idx], idx


def gather(local, positions, total, group=None):
    """Every rank's `(positions, values)` merged into one list of length `total`, on every rank."""
    import torch.distributed as dist

    world = dist.get_world_size(group)
    parts = [None] * world
    dist.all_gather_object(parts, (list(positions), list(local)), group=group)
    out = [None] * total
    for pos, vals in parts:
        for p, v in zip(pos, vals):
            out[p] = v
    if any(v is None for v in out):
        raise RuntimeError("replicas.gather: a position was not computed by any rank")
    return out
