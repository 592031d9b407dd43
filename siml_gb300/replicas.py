"""Replicas across the GPUs of one node, and database shards.

The similarity path has no exchange step: each GPU holds its own copy of the
database and works on disjoint units (row blocks of the query set, job lists,
request streams), so N GPUs are N independent replicas.  The only
collectives are the ones a measurement needs: a barrier around the timed
region and the maximum of the per-rank times.  They run on NCCL for CUDA
ranks and on gloo for CPU ranks.

A database too large for one GPU is split instead into contiguous column
slabs (``shard_bounds``), one per GPU, each GPU searching its slab for all
rows.  The per-slab answers combine on the host with no device exchange:
full-matrix rows side by side, histograms summed, top-k lists merged by
(similarity descending, index ascending), and getNeighbors lists
concatenated with the reference's overflow rule applied across slabs
(``merge_neighbors``; slabs start on 128-column wave boundaries, so each
slab's waves are the full search's waves).
"""
from __future__ import annotations

import os

import numpy as np


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


WAVE = 128   # columns per getNeighbors wave (pysiml/kernels.py:433-474)


def shard_bounds(n_db, world, align=WAVE):
    """[begin, end) column slab of each of `world` shards: contiguous, in
    order, every non-empty slab beginning on a multiple of `align` (trailing
    slabs may be empty when the database is small)."""
    per = -(-max(int(n_db), 0) // max(int(world), 1))
    per = -(-per // align) * align
    return [(min(r * per, n_db), min((r + 1) * per, n_db)) for r in range(world)]


def merge_rows(parts):
    """Full-matrix blocks of consecutive slabs, side by side."""
    return np.concatenate([np.asarray(p) for p in parts], axis=1)


def merge_hist(parts):
    """Histograms of the slabs, summed."""
    out = np.asarray(parts[0]).astype(np.int64 if np.asarray(parts[0]).dtype.kind in "iu" else np.float64)
    for p in parts[1:]:
        out = out + np.asarray(p)
    return out


def merge_topk(parts, k):
    """Per-row top-k of the slabs (absolute indices, -1 / -1.0 padding) into
    the top-k of the whole database: similarity descending, ties to the
    lower index, padded like siml_topk."""
    idx = np.concatenate([np.asarray(p[0]) for p in parts], axis=1)
    sims = np.concatenate([np.asarray(p[1], dtype=np.float32) for p in parts], axis=1)
    rows = idx.shape[0]
    oi = np.full((rows, k), -1, np.int32)
    os_ = np.full((rows, k), -1.0, np.float32)
    for r in range(rows):
        keep = idx[r] >= 0
        ii, ss = idx[r][keep], sims[r][keep]
        order = np.lexsort((ii, -ss))[:k]
        oi[r, :len(order)] = ii[order]
        os_[r, :len(order)] = ss[order]
    return oi, os_


def merge_neighbors(parts, bounds, pitch):
    """getNeighbors answers of consecutive slabs -> the answer over all of
    them, as one search over the whole database gives it.

    parts[s] = (idx [rows, >= min(count, pitch + 128)] absolute indices,
    sims or None, counts [rows]) for slab bounds[s], each searched with a
    pitch of at least pitch + 128 (maxneighbors = pitch + 128).  A row's
    hits are listed in column order while they fit in the pitch; on overflow
    the count grows by whole waves of 128 columns and stops after the first
    wave that takes it above the pitch.  Slab starts are wave boundaries, so
    that wave lies in the first slab whose hits no longer fit, and the slab's
    extra 128 of room lists every hit through it.  Returns (idx [rows,
    pitch], sims [rows, pitch] or None, counts [rows]) with -1 / NaN past a
    row's listed hits."""
    for b, e in bounds:
        if b % WAVE and e > b:
            raise ValueError("slabs must start on %d-column boundaries" % WAVE)
    room = pitch + WAVE
    rows = np.asarray(parts[0][2]).shape[0]
    with_sims = parts[0][1] is not None
    oi = np.full((rows, pitch), -1, np.int32)
    os_ = np.full((rows, pitch), np.nan, np.float32) if with_sims else None
    oc = np.zeros(rows, np.int64)
    for r in range(rows):
        running, out_i, out_s = 0, [], []
        for (b, _), (pi, ps, pc) in zip(bounds, parts):
            c = int(pc[r])
            k = min(c, room)
            li = np.asarray(pi)[r, :k]
            if li.shape[0] < k:
                raise ValueError("a slab listed fewer hits than pitch + %d" % WAVE)
            ls = np.asarray(ps)[r, :k] if with_sims else None
            if running + c <= pitch:
                out_i.extend(li.tolist())
                if with_sims:
                    out_s.extend(ls.tolist())
                running += c
                continue
            need = pitch - running                        # hits of this slab that still fit
            w = (int(li[need]) - b) // WAVE               # the wave that takes the total past the pitch
            running += int(np.count_nonzero((li - b) // WAVE <= w))
            out_i.extend(li[:need].tolist())
            if with_sims:
                out_s.extend(ls[:need].tolist())
            break
        oc[r] = running
        n = min(len(out_i), pitch)
        oi[r, :n] = out_i[:n]
        if with_sims:
            os_[r, :n] = out_s[:n]
    return oi, os_, oc.astype(np.int32)
