"""Instance sharding across GPUs: one process per GPU, no exchange step.

The batched workloads are independent instances.  The reference propagates
them one at a time (``_correlation_2p_1t``, ``pyqed/oqs.py:717-791``, called
once per instance); here a batch is split across ranks, each rank propagates
its share on its own GPU with the single-GPU engine, and the results are
collected on the host.  Nothing crosses between GPUs on the data path.

Partition: greedy longest-processing-time-first on the per-instance cost
(the RK4 work per instance-step is proportional to N^3: 64 N^3 flops with
diagonal collapse operators, 64 (1 + K) N^3 with K dense ones).  Instances
are taken in decreasing cost (ties by index) and each goes to the rank with
the least load so far (ties to the lowest rank); each rank's list is then
sorted by index, so that a rank's sub-batch keeps the batch order and the
gather puts every result back in its original slot.
"""
from __future__ import annotations

import numpy as np

__all__ = ["instance_cost", "partition", "shard_indices", "resolve_shard", "take", "gather",
           "gather_to_rank0"]


def instance_cost(dims, n_cops=0, dense=False):
    """Relative cost of one instance-step: N^3, times (1 + K) with K dense
    collapse operators."""
    d = np.asarray(dims, dtype=np.float64)
    return d ** 3 * ((1 + n_cops) if dense else 1)


def partition(dims, world_size, cost=None):
    """Index lists (ascending) of the instances each of ``world_size`` ranks
    propagates.  ``cost`` overrides ``instance_cost(dims)``."""
    if world_size < 1:
        raise ValueError("world_size must be >= 1")
    dims = np.asarray(dims)
    w = instance_cost(dims) if cost is None else np.asarray(cost, dtype=np.float64)
    order = sorted(range(dims.size), key=lambda b: (-w[b], b))
    load = np.zeros(world_size)
    parts = [[] for _ in range(world_size)]
    for b in order:
        r = int(np.argmin(load))  # lowest rank among the least loaded
        parts[r].append(b)
        load[r] += w[b]
    return [np.array(sorted(p), dtype=np.int64) for p in parts]


def shard_indices(dims, rank, world_size, cost=None):
    """The instances of ``rank`` (ascending indices)."""
    if not 0 <= rank < world_size:
        raise ValueError("rank %d outside a world of %d" % (rank, world_size))
    return partition(dims, world_size, cost)[rank]


def resolve_shard(shard):
    """``shard`` as (rank, world_size): a pair, or ``"dist"`` for the ranks of
    the initialised ``torch.distributed`` process group."""
    if shard is None:
        return None
    if isinstance(shard, str):
        if shard != "dist":
            raise ValueError("shard must be (rank, world_size) or 'dist'")
        import torch.distributed as dist
        if not dist.is_initialized():
            raise RuntimeError("shard='dist' needs an initialised torch.distributed process group")
        return dist.get_rank(), dist.get_world_size()
    rank, world = (int(shard[0]), int(shard[1]))
    if not 0 <= rank < world:
        raise ValueError("rank %d outside a world of %d" % (rank, world))
    return rank, world


def take(seq, idx):
    """Elements ``idx`` of a per-instance list (None passes through)."""
    if seq is None:
        return None
    return [seq[int(b)] for b in idx]


def gather(parts, n_total):
    """Reassemble per-rank results: ``parts`` is a list of (indices, values)
    with values a sequence (or array) aligned with indices; returns a list of
    n_total entries in the original order.  Every index must appear once."""
    out = [None] * n_total
    seen = np.zeros(n_total, dtype=bool)
    for idx, vals in parts:
        if len(idx) != len(vals):
            raise ValueError("indices and values differ in length")
        for b, v in zip(idx, vals):
            if seen[b]:
                raise ValueError("instance %d returned twice" % b)
            seen[b] = True
            out[int(b)] = v
    if not seen.all():
        raise ValueError("instances missing from the gather: %s" % np.nonzero(~seen)[0][:8])
    return out


def gather_to_rank0(indices, values, n_total, group=None):
    """Host-side gather over ``torch.distributed`` (objects, any backend):
    rank 0 gets the full list in the original order, the other ranks None."""
    import torch.distributed as dist
    payload = (np.asarray(indices), list(values))
    objs = [None] * dist.get_world_size(group) if dist.get_rank(group) == 0 else None
    dist.gather_object(payload, objs, dst=0, group=group)
    if dist.get_rank(group) != 0:
        return None
    return gather(objs, n_total)
