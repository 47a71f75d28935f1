"""CPU tests of the multi-GPU split (gbsw_split_pairs, the C++ drop-in's and the
sharding helper's): contiguous ranges balanced by cells, checked against the
rule stated in gbsw.h and against a balance bound, for device counts a test
machine does not have."""
import ctypes
import importlib

import numpy as np
import pytest


def _split(lib, cells, parts):
    cells = np.ascontiguousarray(cells, dtype=np.int64)
    bounds = np.zeros(parts + 1, dtype=np.int64)
    rc = lib.gbsw_split_pairs(cells.ctypes.data if len(cells) else None, len(cells), parts, bounds.ctypes.data)
    return rc, bounds


def _rule(cells, parts):
    """Part r ends at the first pair whose running cell sum reaches r / parts of the total."""
    csum = np.concatenate([[0], np.cumsum(cells)])
    b = [0]
    for r in range(1, parts):
        k = int(np.searchsorted(csum, csum[-1] * r / parts, side="left"))
        b.append(min(max(k, b[-1]), len(cells)))
    return b + [len(cells)]


@pytest.mark.parametrize("parts", [1, 2, 3, 4, 7, 8, 16])
def test_split_follows_the_rule_and_balances(built, parts):
    lib = built.load()
    rng = np.random.default_rng(parts)
    for n in (0, 1, 5, 100, 10_000):
        cells = rng.integers(0, 400 * 1024, n) * rng.integers(1, 300, n)
        rc, bounds = _split(lib, cells, parts)
        assert rc == 0
        assert bounds.tolist() == _rule(cells, parts)
        assert bounds[0] == 0 and bounds[-1] == n and np.all(np.diff(bounds) >= 0)
        if n:
            sums = [int(cells[bounds[r]:bounds[r + 1]].sum()) for r in range(parts)]
            # a contiguous cut is within one pair of the even share
            assert max(sums) <= cells.sum() / parts + cells.max() + 1


def test_split_rejects_bad_arguments(built):
    lib = built.load()
    rc, _ = _split(lib, [1, -1, 2], 2)
    assert rc == -1
    assert lib.gbsw_split_pairs(None, 3, 2, None) == -1
    b = np.zeros(2, np.int64)
    assert lib.gbsw_split_pairs(None, 0, 0, b.ctypes.data) == -1


def test_sharding_helper_uses_the_library_split(built, workloads):
    shard = importlib.import_module("gpu-bsw_gb300.shard")
    batch = workloads.custom_dna(500, 5, 50, 900, 20, 300)
    cells = batch.ref_lengths().astype(np.int64) * batch.query_lengths()
    for world in (1, 2, 3, 8):
        _, bounds = _split(built.load(), cells, world)
        assert shard.shard_ranges(cells, world) == [(int(bounds[r]), int(bounds[r + 1])) for r in range(world)]
