"""CPU checks of the reverse pass's band (reverse_band / band_first_row in
gpu-bsw_gb300/csrc/sw_common.cuh).

The reverse pass runs transposed: rows are the shorter reversed prefix, columns
the longer one.  Under the conditions of the column bound, every cell (r, c) of
an alignment reaching the forward score satisfies c <= r + band with
band = (match * rows - score) // P, P = min(-mismatch, -open, -extend), so each
strip starts at the band's first row and values outside the band may be computed
from zeros.  Two checks:

* every begin the oracle reports lies inside the band (several shapes and
  scorings, thousands of pairs);
* on small pairs, a plain reverse DP whose cells outside the band are forced to
  the zero state finds the same first cell reaching the score (smallest row,
  then smallest column) as the full DP -- the property the kernels rely on.
"""
import importlib

import numpy as np
import pytest

import oracle

wl = importlib.import_module("gpu-bsw_gb300.workloads")


def _band(a, b, na, nb, target, match, p):
    """The kernels' reverse_band: -1 when it does not apply."""
    nrows = min(na, nb)
    if p <= 0 or match <= 0 or ((a < b) != (na < nb)):
        return -1
    slack = match * nrows - target
    return -1 if slack < 0 else slack // p


def _penalty(scores):
    match, mismatch, open_, ext = scores
    return min(-mismatch, -open_, -ext) if (mismatch < 0 and open_ < 0 and ext < 0) else 0


CASES = [
    ("dna_throughput", lambda: wl.dna_throughput(3000, seed=5), (3, -3, -6, -1)),
    ("mixed_long", lambda: wl.custom_dna(300, 9, 1500, 3000, 1000, 1500, related=1.0), (3, -3, -6, -1)),
    ("custom_related", lambda: wl.custom_dna(2000, 7, 20, 700, 10, 400, related=0.6), (1, -3, -3, -1)),
    ("custom_weak_gaps", lambda: wl.custom_dna(2000, 8, 20, 700, 10, 400, related=0.6), (2, -1, -2, -2)),
]


@pytest.mark.parametrize("name,make,scores", CASES, ids=[c[0] for c in CASES])
def test_every_begin_inside_the_band(name, make, scores):
    batch = make()
    p = _penalty(scores)
    res = oracle.align(oracle.DNA, batch.ref, batch.ref_off, batch.query, batch.query_off, scores=scores)
    la, lb = batch.ref_lengths(), batch.query_lengths()
    checked = banded = 0
    for k in range(batch.n):
        s, rb, re_, qb, qe = (int(v) for v in res[k])
        if s <= 0:
            continue
        a, b = int(la[k]), int(lb[k])
        band = _band(a, b, re_, qe, s, scores[0], p)
        if band < 0:
            continue
        # the begin in the transposed reversed matrix: row of the shorter prefix,
        # column of the longer one (1-based)
        if re_ >= qe:
            col, row = re_ - rb, qe - qb
        else:
            col, row = qe - qb, re_ - rb
        assert 1 <= row and 1 <= col <= row + band, (name, k, s, a, b, re_, qe, rb, qb, row, col, band)
        checked += 1
        banded += band < max(re_, qe) - 1
    assert checked > batch.n // 2 and banded > checked // 2


def _reverse_first_hit(L, S, scores, target, band=None):
    """Transposed reverse DP over reversed prefixes: rows = S, columns = L.
    Cells outside the band (c > r + band) are held at the zero state.  Returns the
    first (row, col) whose H equals target, or None."""
    match, mismatch, open_, ext = scores
    n, m = len(S), len(L)
    H = np.zeros((n + 1, m + 1), np.int64)
    E = np.zeros((n + 1, m + 1), np.int64)
    F = np.zeros((n + 1, m + 1), np.int64)
    neg = -(1 << 40)
    E[:, 0] = neg
    F[0, :] = neg
    for r in range(1, n + 1):
        for c in range(1, m + 1):
            if band is not None and c > r + band:
                continue  # outside the band: zero state
            E[r, c] = max(E[r, c - 1] + ext, H[r, c - 1] + open_)
            F[r, c] = max(F[r - 1, c] + ext, H[r - 1, c] + open_)
            s = match if S[r - 1] == L[c - 1] else mismatch
            H[r, c] = max(0, H[r - 1, c - 1] + s, E[r, c], F[r, c])
        hits = np.nonzero(H[r, 1:] == target)[0]
        if len(hits):
            return r, int(hits[0]) + 1
    return None


def _band_first_row(first_col, band):
    """The kernels' band_first_row."""
    if band < 0:
        return 1
    r = first_col - band - 1
    return 1 if r <= 1 else r - ((r - 1) & 1)


def _strip_first_hit(L, S, scores, target, band, W):
    """The reverse pass as the kernels lay it out: columns up to the column bound,
    cut into W-column strips from column 1, the last one padded on the right
    (real columns past the bound, then score -128 past the prefix), each strip
    computed from its band_first_row down, every cell above that left at the zero
    state; the first row holding the score in any computed column, padding
    included, and its leftmost such column."""
    match, mismatch, open_, ext = scores
    n, m = len(S), len(L)
    run = min(m, n + band)
    nstrips = -(-run // W)
    width = nstrips * W
    first = [_band_first_row(s * W + 1, band) for s in range(nstrips)]
    H = np.zeros((n + 1, width + 1), np.int64)
    E = np.zeros((n + 1, width + 1), np.int64)
    F = np.zeros((n + 1, width + 1), np.int64)
    neg = -(1 << 40)
    E[:, 0] = neg
    F[0, :] = neg
    for r in range(1, n + 1):
        for c in range(1, width + 1):
            if r < first[(c - 1) // W]:
                continue
            E[r, c] = max(E[r, c - 1] + ext, H[r, c - 1] + open_)
            F[r, c] = max(F[r - 1, c] + ext, H[r - 1, c] + open_)
            if c <= m:
                s = match if S[r - 1] == L[c - 1] else mismatch
            else:
                s = -128
            H[r, c] = max(0, H[r - 1, c - 1] + s, E[r, c], F[r, c])
        hits = np.nonzero(H[r, 1:width + 1] == target)[0]
        if len(hits):
            return r, int(hits[0]) + 1
    return None


@pytest.mark.parametrize("scores", [(3, -3, -6, -1), (1, -3, -3, -1), (2, -1, -2, -2), (5, -4, -8, -2)])
def test_banded_reverse_dp_finds_the_same_begin(scores):
    batch = wl.custom_dna(150, 11 + scores[0], 20, 90, 10, 70, related=0.7)
    p = _penalty(scores)
    res = oracle.align(oracle.DNA, batch.ref, batch.ref_off, batch.query, batch.query_off, scores=scores)
    la, lb = batch.ref_lengths(), batch.query_lengths()
    cut = 0
    for k in range(batch.n):
        s, rb, re_, qb, qe = (int(v) for v in res[k])
        if s <= 0:
            continue
        a, b = int(la[k]), int(lb[k])
        band = _band(a, b, re_, qe, s, scores[0], p)
        ref, qry = batch.strings(k)
        # reversed prefixes; the shorter prefix gives the rows (the reference
        # counts the reference as the longer one on equal lengths)
        A, B = ref[:re_][::-1], qry[:qe][::-1]
        L, S = (A, B) if re_ >= qe else (B, A)
        full = _reverse_first_hit(L, S, scores, s)
        # the model reproduces the oracle's begin (row of the shorter prefix,
        # column of the longer, both reversed)
        assert full == ((qe - qb, re_ - rb) if re_ >= qe else (re_ - rb, qe - qb)), (k, full)
        if band < 0:
            continue
        assert _reverse_first_hit(L, S, scores, s, band) == full, (k, s, band)
        for W in (8, 16):
            assert _strip_first_hit(L, S, scores, s, band, W) == full, (k, s, band, W)
        cut += band + len(S) < len(L) or band < len(L) - 1
    assert cut > 10
