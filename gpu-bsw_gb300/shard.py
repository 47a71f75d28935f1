"""Pair sharding across ranks (one process per GPU).

Replaces the reference's OpenMP splitter (driver.cpp:23-41, 59-70), which gives
every GPU an equal COUNT of pairs, with contiguous ranges balanced by forward
cells (|ref| * |query|), the unit the passes' time follows.  Pairs are
independent: every rank aligns its range and owns the matching slice of the
results, so the data path needs no collective; gathering the slices is the
caller's choice (``gather_results``).
"""
import numpy as np


def shard_ranges(cells, world):
    """Contiguous [start, end) ranges, one per rank, with near-equal cell sums."""
    cells = np.asarray(cells, dtype=np.int64)
    n = len(cells)
    if world <= 1 or n == 0:
        return [(0, n)] + [(n, n)] * max(0, world - 1)
    csum = np.concatenate([[0], np.cumsum(cells)])
    total = csum[-1]
    bounds = [0]
    for r in range(1, world):
        target = total * r / world
        k = int(np.searchsorted(csum, target, side="left"))
        k = min(max(k, bounds[-1]), n)
        bounds.append(k)
    bounds.append(n)
    return [(bounds[r], bounds[r + 1]) for r in range(world)]


def rank_slice(batch, rank, world):
    """(start, end, sub-batch) of this rank's pairs."""
    cells = batch.ref_lengths().astype(np.int64) * batch.query_lengths()
    a, b = shard_ranges(cells, world)[rank]
    return a, b, batch.subset(np.arange(a, b))


def gather_results(local, rank, world, group=None):
    """Concatenate per-rank (n_r, 5) result slices in rank order (torch.distributed)."""
    import torch.distributed as dist
    parts = [None] * world
    dist.all_gather_object(parts, np.asarray(local), group=group)
    return np.concatenate([p.reshape(-1, 5) for p in parts], axis=0)
