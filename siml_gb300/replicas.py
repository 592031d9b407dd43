"""Replicas across the GPUs of one node.

The similarity path has no exchange step: each GPU holds its own copy of the
database and works on disjoint units (row blocks of the query set, job lists,
request streams), so N GPUs are N independent replicas.  The only
collectives are the ones a measurement needs: a barrier around the timed
region and the maximum of the per-rank times.  They run on NCCL for CUDA
ranks and on gloo for CPU ranks.
"""
from __future__ import annotations

import os


def env():
    """(rank, world_size, local_rank) from the launcher's environment."""
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


def init(backend, device=None):
    """Joins the process group when there is more than one rank."""
    rank, world, _ = env()
    if world <= 1:
        return False
    import torch.distributed as dist
    if not dist.is_initialized():
        if device is not None and backend == "nccl":
            dist.init_process_group(backend, device_id=device)
        else:
            dist.init_process_group(backend)
    return True


def block_of(step, world, rank, nblocks):
    """Row block of `step` on `rank`: round robin, so the ranks' blocks of one
    step are distinct whenever world <= nblocks."""
    return (step * world + rank) % nblocks


def jobs_of(njobs, world, rank):
    """Indices of the jobs a rank runs when a job list is split: every
    world-th job, starting at the rank."""
    return list(range(rank, njobs, world))


def barrier():
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        dist.barrier()


def max_over_ranks(value, device=None):
    """The largest of the ranks' values (each rank's own value when alone)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def finish():
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        dist.destroy_process_group()
