"""A second, independent restatement of the reference's results for tiny pairs.

Pure Python, full matrices, used only to cross-check the C oracle.  Where the C
oracle simulates the reference's shuffle trees lane by lane, this module states
the same results as an explicit order on matrix cells:

* forward (kernel.cpp:198-394 with the trees of kernel.cpp:47-86/137-182): among
  cells with H == max, the smallest row i of the longer sequence; among those,
  the column j of the shorter sequence with the smallest
  ``bitrev5((j-1) >> 5) * 32 + bitrev5((j-1) & 31)`` -- the order in which the
  two-level shfl_down tree lets a left lane keep a full tie;
* reverse (kernel.cpp:397-604 with the trees of kernel.cpp:3-45/90-135): among
  cells of the reversed-prefix matrix with H == max, the smallest reversed
  column t, then the smallest reversed row.
"""

DNA = 0
AA = 1


def bitrev5(x):
    r = 0
    for _ in range(5):
        r = (r << 1) | (x & 1)
        x >>= 1
    return r


def tie_key(j):
    """Tree order of the 1-based column j among full (value, row) ties (runs of
    1,024 columns, beyond the reference's block limit, in increasing order)."""
    t = j - 1
    return ((t >> 10) << 10) + bitrev5((t >> 5) & 31) * 32 + bitrev5(t & 31)


def _matrix(L, S, score, open_, ext):
    nL, nS = len(L), len(S)
    H = [[0] * (nS + 1) for _ in range(nL + 1)]
    F = [[0] * (nS + 1) for _ in range(nL + 1)]
    E = [[0] * (nS + 1) for _ in range(nL + 1)]
    for i in range(1, nL + 1):
        for j in range(1, nS + 1):
            F[i][j] = max(F[i - 1][j] + ext, H[i - 1][j] + open_)
            E[i][j] = 0 if j == 1 else max(E[i][j - 1] + ext, H[i][j - 1] + open_)
            H[i][j] = max(H[i - 1][j - 1] + score(L[i - 1], S[j - 1]), E[i][j], F[i][j], 0)
    return H


def align_pair(kind, A, B, scores=None, matrix=None, encoding=None, gaps=None):
    """Returns (score, ref_begin, ref_end, query_begin, query_end); A = ref, B = query."""
    A = A.encode() if isinstance(A, str) else bytes(A)
    B = B.encode() if isinstance(B, str) else bytes(B)
    if kind == DNA:
        m, mm, open_, ext = scores

        def score(x, y):
            return m if x == y else mm
    else:
        open_, ext = gaps

        def score(x, y):
            return matrix[encoding[x] * 24 + encoding[y]]

    a, b = len(A), len(B)
    a_short = a < b
    S, L = (A, B) if a_short else (B, A)
    if len(S) == 0:
        return (0, -1, -1, -1, -1)
    H = _matrix(L, S, score, open_, ext)
    best = max(max(row) for row in H)
    if best <= 0:
        return (0, -1, -1, -1, -1)
    cells = [(i, j) for i in range(1, len(L) + 1) for j in range(1, len(S) + 1) if H[i][j] == best]
    i_star = min(i for i, _ in cells)
    j_star = min((j for i, j in cells if i == i_star), key=tie_key)
    if a_short:
        query_end, ref_end = i_star, j_star
    else:
        ref_end, query_end = i_star, j_star

    na, nb = ref_end, query_end
    a2_short = na < nb
    S2, L2 = (A[:na], B[:nb]) if a2_short else (B[:nb], A[:na])
    S2r, L2r = S2[::-1], L2[::-1]
    H2 = _matrix(L2r, S2r, score, open_, ext)
    best2 = max(max(row) for row in H2)
    cells2 = [(i, t) for i in range(1, len(L2r) + 1) for t in range(len(S2r)) if H2[i][t + 1] == best2]
    t_star = min(t for _, t in cells2)
    i2 = min(i for i, t in cells2 if t == t_star)
    begin_L = len(L2) - i2
    begin_S = len(S2) - t_star - 1
    if a2_short:
        query_begin, ref_begin = begin_L, begin_S
    else:
        ref_begin, query_begin = begin_L, begin_S
    return (best, ref_begin, ref_end, query_begin, query_end)


def traceback_pair(kind, A, B, result, scores=None, matrix=None, encoding=None, gaps=None):
    """The traceback's definition (see oracle/traceback.c) restated with full
    H/E/F matrices and a walk that re-derives each step from the values.
    Returns (ops as [(length, op char)], H(k, m))."""
    score, rb, re_, qb, qe = [int(x) for x in result]
    if score <= 0:
        return [], 0
    R, Q = A[rb:re_], B[qb:qe]
    m, k = len(R), len(Q)
    if kind == DNA:
        match, mismatch, open_, ext = scores
        sub = lambda r, q: match if r == q else mismatch  # noqa: E731
    else:
        open_, ext = gaps
        ref_longer = len(A) >= len(B)

        def sub(r, q):
            er, eq = encoding[r], encoding[q]
            return matrix[er * 24 + eq] if ref_longer else matrix[eq * 24 + er]
    NEG = -(1 << 30)
    gap = lambda n: max(open_ + (n - 1) * ext, NEG)  # noqa: E731
    H = [[0] * (m + 1) for _ in range(k + 1)]
    E = [[NEG] * (m + 1) for _ in range(k + 1)]
    F = [[NEG] * (m + 1) for _ in range(k + 1)]
    for j in range(1, m + 1):
        H[0][j] = gap(j)
    for i in range(1, k + 1):
        H[i][0] = gap(i)
        for j in range(1, m + 1):
            E[i][j] = max(E[i][j - 1] + ext, H[i][j - 1] + open_)
            F[i][j] = max(F[i - 1][j] + ext, H[i - 1][j] + open_)
            d = H[i - 1][j - 1] + sub(R[j - 1], Q[i - 1])
            H[i][j] = max(d, F[i][j], E[i][j])
    out = []

    def push(op):
        if out and out[-1][1] == op:
            out[-1][0] += 1
        else:
            out.append([1, op])
    i, j, state = k, m, "H"
    while i > 0 or j > 0:
        if i == 0:
            push("D")
            j -= 1
        elif j == 0:
            push("I")
            i -= 1
        elif state == "H":
            d = H[i - 1][j - 1] + sub(R[j - 1], Q[i - 1])
            if d >= F[i][j] and d >= E[i][j]:
                push("=" if R[j - 1] == Q[i - 1] else "X")
                i, j = i - 1, j - 1
            elif F[i][j] >= E[i][j]:
                state = "F"
            else:
                state = "E"
        elif state == "E":
            push("D")
            state = "E" if E[i][j - 1] + ext >= H[i][j - 1] + open_ else "H"
            j -= 1
        else:
            push("I")
            state = "F" if F[i - 1][j] + ext >= H[i - 1][j] + open_ else "H"
            i -= 1
    return [(n, op) for n, op in reversed(out)], H[k][m]


def path_score(kind, A, B, result, ops, scores=None, matrix=None, encoding=None, gaps=None):
    """Score of an alignment given as [(length, op char)] over the pair's segment."""
    score, rb, re_, qb, qe = [int(x) for x in result]
    if kind == DNA:
        match, mismatch, open_, ext = scores
    else:
        open_, ext = gaps
        ref_longer = len(A) >= len(B)
    i, j, total = qb, rb, 0
    for n, op in ops:
        if op in "=X":
            for _ in range(n):
                r, q = A[j], B[i]
                if kind == DNA:
                    total += match if r == q else mismatch
                else:
                    er, eq = encoding[r], encoding[q]
                    total += matrix[er * 24 + eq] if ref_longer else matrix[eq * 24 + er]
                i, j = i + 1, j + 1
        elif op == "D":
            total += open_ + (n - 1) * ext
            j += n
        else:
            total += open_ + (n - 1) * ext
            i += n
    assert i == qe and j == re_, (i, qe, j, re_)
    return total
