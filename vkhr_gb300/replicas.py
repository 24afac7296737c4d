"""Multi-GPU plumbing of the path: one process per GPU, no data-path collective.

Hair styles are independent and a frame's pixels are independent, so the
path shards with no exchange: `shard()` splits a batch of styles across
ranks (each rank voxelizes and raymarches its own styles), and `bench.py
--gpus N` runs N replicas of the production frame.  The only collectives
are for measurement: a barrier around the timed region and the maximum of
the per-rank times.
"""
import os

import torch
import torch.distributed as dist


def world():
    """(rank, world_size, local_rank) from the launcher's environment."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def init(backend="nccl"):
    rank, size, local = world()
    if size > 1 and not dist.is_initialized():
        dist.init_process_group(backend)
    return rank, size, local


def barrier():
    if dist.is_initialized():
        dist.barrier()


def max_over_ranks(x, device="cpu"):
    """The largest value of x over all ranks (x on every rank)."""
    if not dist.is_initialized():
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def shard(costs, rank, size):
    """Indices of the jobs rank `rank` of `size` processes: greedy longest-
    processing-time assignment on the given per-job costs (deterministic, so
    every rank computes the same split without communicating)."""
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    load = [0.0] * size
    owner = [0] * len(costs)
    for i in order:
        r = min(range(size), key=lambda q: (load[q], q))
        owner[i] = r
        load[r] += costs[i]
    return [i for i in range(len(costs)) if owner[i] == rank]
