"""Independent tissue instances sharded over ranks (one GPU each).

The batched sweep has no exchange between instances, so a multi-GPU run gives
each rank a subset of the instances and runs them as one batch on its own GPU;
the only communication is the final gather of per-instance results and the
max-over-ranks timing.  One mesh over several ranks needs an interface halo
per assembly and per matrix-vector product: that is partition.py.
"""
from __future__ import annotations

import heapq

import numpy as np


def shard_instances(sizes, world):
    """Balanced, deterministic assignment of instances to ranks: largest first
    onto the least-loaded rank (ties: lowest rank).  Returns, per rank, the
    sorted list of instance indices."""
    if world < 1:
        raise ValueError("world size must be positive")
    order = sorted(range(len(sizes)), key=lambda i: (-int(sizes[i]), i))
    heap = [(0, r) for r in range(world)]
    out = [[] for _ in range(world)]
    for i in order:
        load, r = heapq.heappop(heap)
        out[r].append(i)
        heapq.heappush(heap, (load + int(sizes[i]), r))
    return [sorted(o) for o in out]


def gather_results(dist, rank, world, mine: dict):
    """Gather {instance index: result} dictionaries on rank 0 (None elsewhere).
    `dist` is torch.distributed with an initialised process group."""
    objs = [None] * world if rank == 0 else None
    dist.gather_object(mine, objs, dst=0)
    if rank != 0:
        return None
    merged = {}
    for part in objs:
        for k, v in part.items():
            if k in merged:
                raise RuntimeError(f"instance {k} was run on two ranks")
            merged[k] = v
    return merged


def max_over_ranks(dist, value: float) -> float:
    """The largest of one float over all ranks (for timing)."""
    import torch

    t = torch.tensor([float(value)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t[0])


def checksum(pos) -> float:
    """A size-independent fingerprint of a position vector."""
    p = np.asarray(pos, dtype=np.float64)
    return float(np.sum(p * np.cos(np.arange(p.size))))
