"""Pair sharding across ranks (one process per GPU).

Replaces the reference's OpenMP splitter (driver.cpp:23-41, 59-70), which gives
every GPU an equal COUNT of pairs, with contiguous ranges balanced by forward
cells (|ref| * |query|), the unit the passes' time follows.  The split itself is
libgbsw's ``gbsw_split_pairs``, the one the C++ drop-in uses to spread a call
over its devices (a host function: it runs without a GPU).  Pairs are
independent: every rank aligns its range and owns the matching slice of the
results, so the data path needs no collective; gathering the slices is the
caller's choice (``gather_results``).
"""
import numpy as np


def shard_ranges(cells, world):
    """Contiguous [start, end) ranges, one per rank, with near-equal cell sums."""
    from . import GbswError, load
    cells = np.ascontiguousarray(cells, dtype=np.int64)
    n = len(cells)
    world = max(1, int(world))
    bounds = np.zeros(world + 1, dtype=np.int64)
    rc = load().gbsw_split_pairs(cells.ctypes.data if n else None, n, world, bounds.ctypes.data)
    if rc != 0:
        raise GbswError(rc, "gbsw_split_pairs")
    return [(int(bounds[r]), int(bounds[r + 1])) for r in range(world)]


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
