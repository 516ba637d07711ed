"""Sharding of batched instances across GPUs (one process per GPU).

Independent instances need no data exchange, so ranks split the instance list
and each advances its share with ``BatchedCahnHilliard``; there is no
collective on the data path.  The split balances the voxel count (greedy:
largest instance first, to the rank with the least work so far), which is what
one IMEX step's cost is proportional to.  Single grids do not shard (a slab FFT
would need an all-to-all); they run as independent replicas.
"""

from __future__ import annotations

import numpy as np


def partition_instances(shapes, world_size):
    """Instance indices per rank, balanced by sum(Nx*Ny*Nz); deterministic."""
    if world_size < 1:
        raise ValueError("world_size must be >= 1")
    cost = [int(np.prod(s)) for s in shapes]
    order = sorted(range(len(shapes)), key=lambda i: (-cost[i], i))
    load = [0] * world_size
    parts = [[] for _ in range(world_size)]
    for i in order:
        r = min(range(world_size), key=lambda k: (load[k], k))
        parts[r].append(i)
        load[r] += cost[i]
    return [sorted(p) for p in parts]


def my_instances(shapes, rank, world_size):
    return partition_instances(shapes, world_size)[rank]


def shard(shapes, rank, world_size, *per_instance):
    """This rank's share of a batch: ``(indices, shapes, *per_instance values)`` of the instances
    ``partition_instances(shapes, world_size)[rank]``.  ``per_instance`` are scalars (broadcast) or
    sequences with one value per instance (mobility, eps, fields, ...).  Every rank derives the same
    split from the same list, so no collective is needed to agree on it."""
    if not 0 <= rank < world_size:
        raise ValueError(f"rank {rank} outside world of {world_size}")
    idx = partition_instances(shapes, world_size)[rank]
    n = len(shapes)
    out = [idx, [tuple(shapes[i]) for i in idx]]
    for v in per_instance:
        if np.isscalar(v) or (isinstance(v, np.ndarray) and v.ndim == 0):
            out.append([v] * len(idx))
        else:
            if len(v) != n:
                raise ValueError(f"per-instance values: {len(v)} for {n} instances")
            out.append([v[i] for i in idx])
    return tuple(out)

