"""CPU check of the invariant behind the passes' padding rows.

The pass kernels (sw_pass.cuh, sw_dual.cu) run a row step for every lane on
every pipeline step.  A lane whose row lies before the pair's first row reads a
padding row code whose score is <= 0 in every column (0 or -1 for DNA, -128 for
protein).  The kernels rely on this: from the initial state (H = 0, E = F = 0),
such rows leave H, E and F exactly at that state whenever the gap values are
<= 0, so every lane enters its first real row in the boundary state.

This test runs the kernels' cell update (the clamped form with Ho = H + open,
T = max(Ho_diag + s, F' + open), E' = max(E + max(ext, open), T, 0)) over a
matrix with padding rows in front and checks that the real rows' H equal those
of the same matrix without them, for random scorings with gaps <= 0."""
import numpy as np
import pytest

import pyref


def _rows(scores, open_, ext, lead_pad):
    """H of every row of `scores` (rows x cols substitution scores), after
    `lead_pad` rows whose scores are drawn from {0, -1, -128}."""
    rng = np.random.default_rng(lead_pad * 7919 + scores.shape[1])
    rows, cols = scores.shape
    pad = rng.choice([0, -1, -128], size=(lead_pad, cols))
    ho = np.full(cols, open_, dtype=np.int64)   # H + open of the row above (H = 0)
    f = np.zeros(cols, dtype=np.int64)
    out = []
    for s_row in list(pad) + list(scores):
        e = 0                     # E entering column 0 (the left boundary)
        diag = open_              # Ho of the boundary column (H = 0)
        new_ho = np.empty_like(ho)
        for j in range(cols):
            fv = max(f[j] + ext, ho[j], 0)
            t = max(fv + open_, diag + s_row[j])
            hov = max(e + open_, t)
            e = max(e + max(ext, open_), t, 0)
            diag = ho[j]
            new_ho[j] = hov
            f[j] = fv
        ho = new_ho
        out.append(ho - open_)
    return np.array(out[lead_pad:])


@pytest.mark.parametrize("seed", range(6))
def test_padding_rows_leave_the_boundary_state(seed):
    rng = np.random.default_rng(seed)
    rows, cols = rng.integers(1, 25), rng.integers(1, 25)
    match, mismatch = int(rng.integers(1, 6)), int(rng.integers(-6, 3))
    open_, ext = int(rng.integers(-12, 1)), int(rng.integers(-4, 1))
    a = rng.integers(0, 4, size=cols)
    b = rng.integers(0, 4, size=rows)
    scores = np.where(b[:, None] == a[None, :], match, mismatch)
    plain = _rows(scores, open_, ext, 0)
    for lead in (1, 3, 31):
        np.testing.assert_array_equal(_rows(scores, open_, ext, lead), plain,
                                      err_msg="lead=%d open=%d ext=%d" % (lead, open_, ext))
    # and the kernels' form of the recurrence is the reference's (the Python
    # restatement of kernel.cpp's H matrix)
    H = pyref._matrix(list(b), list(a), lambda x, y: match if x == y else mismatch, open_, ext)
    np.testing.assert_array_equal(plain, np.array(H)[1:, 1:])


def test_a_positive_padding_score_would_leak():
    """The bound is needed: one padding row scoring +5 changes the real rows."""
    scores = np.where(np.eye(6, dtype=bool), 3, -1)
    plain = _rows(scores, -6, -1, 0)
    rows, cols = scores.shape
    ho = np.full(cols, -6, dtype=np.int64)
    f = np.zeros(cols, dtype=np.int64)
    out = []
    for s_row in [np.full(cols, 5)] + list(scores):
        e, diag, new_ho = 0, -6, np.empty_like(ho)
        for j in range(cols):
            fv = max(f[j] - 1, ho[j], 0)
            t = max(fv - 6, diag + s_row[j])
            new_ho[j] = max(e - 6, t)
            e = max(e - 1, t, 0)
            diag = ho[j]
            f[j] = fv
        ho = new_ho
        out.append(ho + 6)
    assert not np.array_equal(np.array(out[1:]), plain)
