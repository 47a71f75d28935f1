"""CPU check of the reverse pass's column bound (reverse_columns in
gpu-bsw_gb300/csrc/sw_common.cuh).

The reverse pass computes only the first nrows + (match * nrows - score) / P
reversed columns of the longer prefix, P = min(-mismatch, -open, -extend), when
the roles of the two sequences are the same forward and reverse.  The argument
(every alignment of the forward score inside the prefixes ends on the forward
end's row of the longer sequence, and each non-match position of it costs at
least P) says the begin always lies inside the bound.  This test checks that on
the oracle's begins for several shapes and scorings, and that the bound does cut
columns on most pairs of the DNA throughput shape."""
import importlib

import numpy as np
import pytest

import oracle

wl = importlib.import_module("gpu-bsw_gb300.workloads")


def _bound(a, b, na, nb, target, match, p):
    """Columns the reverse pass computes (the kernels' reverse_columns)."""
    ncols, nrows = max(na, nb), min(na, nb)
    if p <= 0 or match <= 0 or ((a < b) != (na < nb)):
        return ncols
    slack = match * nrows - target
    if slack < 0:
        return ncols
    return min(ncols, nrows + slack // p)


CASES = [
    ("dna_throughput", lambda: wl.dna_throughput(3000, seed=5), (3, -3, -6, -1)),
    ("plain_dna", lambda: wl.plain_dna(2000, seed=6), (3, -3, -6, -1)),
    ("custom_related", lambda: wl.custom_dna(2000, 7, 20, 700, 10, 400, related=0.6), (1, -3, -3, -1)),
    ("custom_weak_gaps", lambda: wl.custom_dna(2000, 8, 20, 700, 10, 400, related=0.6), (2, -1, -2, -2)),
]


@pytest.mark.parametrize("name,make,scores", CASES, ids=[c[0] for c in CASES])
def test_every_begin_inside_the_bound(name, make, scores):
    batch = make()
    match, mismatch, open_, ext = scores
    p = min(-mismatch, -open_, -ext) if (mismatch < 0 and open_ < 0 and ext < 0) else 0
    res = oracle.align(oracle.DNA, batch.ref, batch.ref_off, batch.query, batch.query_off, scores=scores)
    la, lb = batch.ref_lengths(), batch.query_lengths()
    cut = checked = 0
    for k in range(batch.n):
        s, rb, re_, qb, qe = (int(v) for v in res[k])
        if s <= 0:
            continue
        a, b = int(la[k]), int(lb[k])
        bound = _bound(a, b, re_, qe, s, match, p)
        # the begin as a reversed 1-based column of the longer prefix
        col = max(re_, qe) - (rb if re_ >= qe else qb)
        assert 1 <= col <= bound, (name, k, s, a, b, re_, qe, rb, qb, col, bound)
        checked += 1
        cut += bound < max(re_, qe)
    assert checked > batch.n // 2
    if name == "dna_throughput":
        assert cut > checked // 2  # the bound matters on the headline shape
