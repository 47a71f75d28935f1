"""CPU tests of the oracle: against the reference's own outputs (golden fixtures)
and against an independent pure-Python restatement."""
import importlib
import os
import random
import sys

import numpy as np
import pytest

import oracle
import pyref
from helpers import GOLDEN

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
import make_golden  # noqa: E402

sc = importlib.import_module("gpu-bsw_gb300.scoring")


def _rs(rng, n, alpha):
    return "".join(rng.choice(alpha) for _ in range(n))


def _cases(seed, count, maxlen):
    rng = random.Random(seed)
    refs, qs = [], []
    for _ in range(count):
        alpha = rng.choice(["ACGT", "AC", "A", "ACGTN"])
        a = rng.randint(0, maxlen)
        r = _rs(rng, a, alpha)
        if rng.random() < 0.5 and a > 3:
            s0 = rng.randint(0, a - 2)
            q = r[s0:s0 + rng.randint(1, a - s0)]
            q = "".join(c if rng.random() > 0.1 else rng.choice(alpha) for c in q)
        else:
            q = _rs(rng, rng.randint(0, maxlen), alpha)
        refs.append(r)
        qs.append(q)
    return refs, qs


@pytest.mark.parametrize("scores", [(3, -3, -6, -1), (1, -3, -3, -1), (2, -1, -2, -2), (1, 0, 0, 0),
                                    (5, -4, -10, -1)])
def test_oracle_matches_python_restatement_dna(scores):
    refs, qs = _cases(hash(scores) & 0xffff, 250, 70)
    got = oracle.align_strings(oracle.DNA, refs, qs, scores=scores)
    for k in range(len(refs)):
        assert tuple(got[k]) == pyref.align_pair(pyref.DNA, refs[k], qs[k], scores=scores), (refs[k], qs[k])


def test_oracle_matches_python_restatement_multiwarp_ties():
    # columns beyond 32 and 64 exercise the warp level of the reference's argmax tree
    rng = random.Random(7)
    refs, qs = [], []
    for _ in range(30):
        unit = _rs(rng, rng.randint(1, 4), rng.choice(["A", "AC", "ACGT"]))
        refs.append((unit * 400)[: rng.randint(100, 300)])
        qs.append((unit * 400)[rng.randint(0, 3):][: rng.randint(33, 200)])
    got = oracle.align_strings(oracle.DNA, refs, qs, scores=(1, -1, -1, -1))
    for k in range(len(refs)):
        assert tuple(got[k]) == pyref.align_pair(pyref.DNA, refs[k], qs[k], scores=(1, -1, -1, -1))


def test_oracle_matches_python_restatement_protein():
    rng = random.Random(3)
    alpha = sc.AA_ORDER + "JOU"
    refs = [_rs(rng, rng.randint(0, 50), alpha) for _ in range(150)]
    qs = [_rs(rng, rng.randint(0, 50), alpha) for _ in range(150)]
    for gaps in [(-6, -1), (-11, -1)]:
        got = oracle.align_strings(oracle.AA, refs, qs, matrix=sc.BLOSUM62, encoding=sc.ENCODING, gaps=gaps)
        for k in range(len(refs)):
            exp = pyref.align_pair(pyref.AA, refs[k], qs[k], matrix=sc.BLOSUM62, encoding=sc.ENCODING, gaps=gaps)
            assert tuple(got[k]) == exp


def test_tie_key_is_the_tree_order():
    # the bit-reversed key must pick the same column as a lane-by-lane simulation
    # of the reference's shfl_down tree on full (value, row) ties
    def tree(cands):
        cur = list(cands)
        off = 16
        while off:
            nxt = []
            for lane in range(32):
                me, other = cur[lane], cur[lane + off] if lane + off < 32 else cur[lane]
                if other[0] > me[0] or (other[0] == me[0] and other[1] < me[1]):
                    me = other
                nxt.append(me)
            cur = nxt
            off //= 2
        return cur[0]
    rng = random.Random(5)
    for _ in range(500):
        cols = rng.sample(range(32), rng.randint(1, 8))
        cands = [(0, 0, 0)] * 32
        for c in cols:
            cands[c] = (5, 2, c + 1)
        assert tree(cands)[2] == min((c + 1 for c in cols), key=pyref.tie_key)


def test_empty_and_zero_score_convention():
    got = oracle.align_strings(oracle.DNA, ["", "ACGT", "AAAA", ""], ["ACGT", "", "CCCC", ""],
                               scores=(3, -3, -6, -1))
    assert got.tolist() == [[0, -1, -1, -1, -1]] * 4


def test_protein_symbol_outside_table_is_rejected():
    with pytest.raises(ValueError):
        oracle.align_strings(oracle.AA, ["ACDa"], ["ACD"], matrix=sc.BLOSUM62, encoding=sc.ENCODING,
                             gaps=(-6, -1))


@pytest.mark.skipif(not GOLDEN, reason="golden fixtures not generated")
@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
def test_oracle_reproduces_reference_outputs(path):
    kind, params, refs, qs, exp = make_golden.load_fixture(path)
    got = make_golden.oracle_results(kind, params, refs, qs)
    bad = np.nonzero(np.any(got != exp, axis=1))[0]
    assert len(bad) == 0, [(int(k), got[k].tolist(), exp[k].tolist()) for k in bad[:5]]


def test_scoring_tables():
    m = np.array(sc.BLOSUM62).reshape(24, 24)
    assert (m == m.T).all()
    assert sc.ENCODING[ord("A")] == 0 and sc.ENCODING[ord("*")] == 23
    assert sc.ENCODING[ord("J")] == sc.ENCODING[ord("O")] == sc.ENCODING[ord("U")] == 0
    assert len(sc.ENCODING) == 91


def test_oracle_beyond_1024_columns_matches_python_restatement():
    # the shorter sequence above 1,024 (beyond the reference's block limit):
    # runs of 1,024 columns in increasing order, same order inside each run
    refs = ["AC" * 560, "A" * 1100 + "C" * 8]
    qs = ["AC" * 540, "A" * 1060]
    got = oracle.align_strings(oracle.DNA, refs, qs, scores=(1, -1, -1, -1))
    for k in range(len(refs)):
        assert tuple(got[k]) == pyref.align_pair(pyref.DNA, refs[k], qs[k], scores=(1, -1, -1, -1))
