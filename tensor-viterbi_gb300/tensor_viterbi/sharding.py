"""Sequences across GPUs: independent decodes shard with no collective on the
data path (one process per GPU).  A single sequence does not shard: its
recurrence needs the whole delta[t] at every step, so more GPUs only run
replicas.

Each rank takes a longest-processing-time share of the batch (sequences in
decreasing cost, each to the least-loaded rank; ties to the lower rank),
decodes it, and rank 0 gathers the results in input order (a host-side
object gather; it works over gloo and NCCL alike).
"""
from __future__ import annotations

import numpy as np


def lpt_shards(costs, world_size: int) -> list:
    """Indices of each rank's share, ascending; every index in exactly one
    share; a rank's load exceeds the lightest by at most one item's cost."""
    costs = np.asarray(costs, dtype=np.float64)
    order = np.argsort(-costs, kind="stable")
    loads = np.zeros(world_size)
    shards = [[] for _ in range(world_size)]
    for k in order:
        r = int(np.argmin(loads))
        loads[r] += costs[k]
        shards[r].append(int(k))
    return [sorted(s) for s in shards]


def my_shard(costs, world_size: int, rank: int) -> list:
    return lpt_shards(costs, world_size)[rank]


def decode_sharded(decode_fn, sequences, costs=None, group=None):
    """Decode this rank's share of `sequences` with decode_fn(seq) and gather
    everything on rank 0: returns the list of results in input order on rank
    0 and None on the others.  Without an initialised process group it
    decodes everything locally."""
    import torch.distributed as dist
    if costs is None:
        costs = [len(s) for s in sequences]
    if not (dist.is_available() and dist.is_initialized()):
        return [decode_fn(s) for s in sequences]
    ws, rank = dist.get_world_size(group), dist.get_rank(group)
    mine = my_shard(costs, ws, rank)
    local = [(k, decode_fn(sequences[k])) for k in mine]
    gathered = [None] * ws if rank == 0 else None
    dist.gather_object(local, gathered, dst=0, group=group)
    if rank != 0:
        return None
    out = [None] * len(sequences)
    for part in gathered:
        for k, res in part:
            out[k] = res
    return out
