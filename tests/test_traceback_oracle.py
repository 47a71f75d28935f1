"""CPU tests of the traceback oracle (oracle/traceback.c): it agrees operation for
operation with the independent Python statement in tests/pyref.py, every path
runs from the pair's begin to its end, and rescoring a path from its operations
gives the pair's score (the forward pass's maximum)."""
import importlib

import numpy as np
import pytest

import oracle
import pyref

SCORINGS = [(3, -3, -6, -1), (1, -3, -3, -1), (2, -1, -2, -2), (1, 0, 0, 0), (5, -4, -10, -1)]


def _ops(packed):
    return [(int(v) >> 4, oracle.OPS[int(v) & 15]) for v in packed]


def _check_batch(kind, refs, qs, **sc):
    res = oracle.align_strings(kind, refs, qs, **sc)
    A = b"".join(r.encode() for r in refs)
    B = b"".join(q.encode() for q in qs)
    offA = np.cumsum([0] + [len(r) for r in refs])
    offB = np.cumsum([0] + [len(q) for q in qs])
    ops, off, pscore = oracle.traceback(kind, A, offA, B, offB, res, **sc)
    for k in range(len(refs)):
        got = _ops(ops[off[k]:off[k + 1]])
        exp, h = pyref.traceback_pair(kind, refs[k].encode(), qs[k].encode(), res[k], **sc)
        assert got == exp, (k, refs[k], qs[k], res[k], got, exp)
        assert pscore[k] == h
        if res[k][0] > 0:
            assert pscore[k] == res[k][0], (k, res[k], pscore[k])
            gaps = sc.get("gaps") or sc["scores"][2:]
            if gaps[0] <= gaps[1]:  # open <= extend: runs of one gap type are single gaps
                assert pyref.path_score(kind, refs[k].encode(), qs[k].encode(), res[k], got, **sc) == res[k][0]
        else:
            assert got == []
    return res


@pytest.mark.parametrize("scores", SCORINGS)
def test_dna_random_and_related(scores):
    rng = np.random.default_rng(91)
    refs, qs = [], []
    for _ in range(120):
        r = "".join(rng.choice(list("ACGT"), rng.integers(1, 90)))
        if rng.random() < 0.6 and len(r) > 4:
            a = rng.integers(0, len(r) - 2)
            q = list(r[a:a + rng.integers(2, 60)])
            for t in range(len(q)):
                if rng.random() < 0.1:
                    q[t] = rng.choice(list("ACGT"))
            if rng.random() < 0.5 and len(q) > 3:
                del q[rng.integers(0, len(q) - 1)]
            q = "".join(q)
        else:
            q = "".join(rng.choice(list("ACGT"), rng.integers(1, 60)))
        refs.append(r)
        qs.append(q)
    _check_batch(oracle.DNA, refs, qs, scores=scores)


def test_tie_heavy_repeats_and_edges():
    refs = ["ACACACACAC", "AAAA", "A", "", "ACGT", "GGGGCCCC", "ACGTNNacgt", "AC" * 30]
    qs = ["CACA", "AAAAAAAA", "A", "ACGT", "", "CCCCGGGG", "ACGTNNACGT", "CA" * 20 + "AC" * 5]
    for scores in SCORINGS:
        _check_batch(oracle.DNA, refs, qs, scores=scores)


def test_protein():
    sc = importlib.import_module("gpu-bsw_gb300.scoring")
    rng = np.random.default_rng(92)
    alpha = list("ARNDCQEGHILKMFPSTWYVBZX*")
    refs = ["".join(rng.choice(alpha, rng.integers(1, 70))) for _ in range(60)]
    qs = [r[rng.integers(0, max(1, len(r) // 3)):] if rng.random() < 0.5 else
          "".join(rng.choice(alpha, rng.integers(1, 70))) for r in refs]
    for gaps in [(-6, -1), (-11, -1)]:
        _check_batch(oracle.AA, refs, qs, matrix=sc.BLOSUM62, encoding=sc.ENCODING, gaps=gaps)


def test_cigar_string():
    assert oracle.cigar(np.array([(3 << 4) | 7, (1 << 4) | 8, (2 << 4) | 1, (4 << 4) | 2], np.uint32)) == "3=1X2I4D"
