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
