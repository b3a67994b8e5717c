"""Replicas across GPUs.

The assembly and continuity solve of one mesh have no exchange step on a
single rank: the reference's only data-path collective is the Tpetra
Export-ADD of shared rows in loadComplete (src/TpetraLinearSystem.C:1757-1778),
which a one-rank mesh does not need.  N GPUs therefore run N independent
replicas (one mesh per rank, weak scaling); the job time is the maximum over
ranks, measured between barriers, and the job throughput counts the units
of all ranks.  torch.distributed is used only for the barrier and the max.
"""
import os


def init_from_env(backend="gloo"):
    """(world_size, rank, local_rank, dist or None) from the torchrun environment."""
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        if not dist.is_initialized():
            dist.init_process_group(backend)
        return ws, rank, local, dist
    return 1, 0, 0, None


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, value):
    if dist is None:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(units_per_rank, steps, seconds_max, world_size):
    """Units processed by all ranks per second of the slowest rank."""
    return world_size * units_per_rank * steps / seconds_max
