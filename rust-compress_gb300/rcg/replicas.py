"""Replica execution across GPUs: the search path does not shard (a search is a sequential bisection over one
image), so N GPUs run N independent replicas, each on its own images, with no collective on the data path.

Host-side only: which images a rank takes, and the max-over-ranks timing the benchmark reports.
"""

import os


def env_rank():
    """(rank, world_size, local_rank) from the torchrun environment (1 process when absent)."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def shard(sizes, rank, world):
    """Indices of the items rank `rank` of `world` processes, balanced by cost (e.g. pixel count).

    Greedy longest-processing-time assignment: items sorted by cost (ties by index) go to the least loaded rank (ties
    by rank). Deterministic, so every rank computes the same partition without communicating; each item is assigned
    to exactly one rank."""
    if world <= 1:
        return list(range(len(sizes)))
    order = sorted(range(len(sizes)), key=lambda i: (-sizes[i], i))
    load = [0] * world
    owner = [0] * len(sizes)
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        owner[i] = r
        load[r] += sizes[i]
    return [i for i in range(len(sizes)) if owner[i] == rank]


def max_over_ranks(value, dist=None):
    """The maximum of a float over all ranks (the job's time is its slowest rank's)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    import torch

    t = torch.tensor([float(value)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value, dist=None):
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    import torch

    t = torch.tensor([float(value)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())
