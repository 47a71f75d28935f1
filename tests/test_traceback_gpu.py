"""GPU tests of gbsw_traceback_host: one optimal path per aligned pair.

The kernel must reproduce the traceback oracle (oracle/traceback.c) operation
for operation -- the path definition and its tie rules are this library's own,
as the reference declares a traceback but never implements one -- and every
path must run from the pair's begin to its end with the pair's score."""
import importlib

import numpy as np
import pytest

import oracle
from helpers import oracle_batch

pytestmark = pytest.mark.gpu

DNA_BENCH = (3, -3, -6, -1)
AA_GAPS = (-6, -1)


def _oracle_trace(batch, kind, res, scores=None, gaps=None):
    sc = importlib.import_module("gpu-bsw_gb300.scoring")
    if kind == 0:
        return oracle.traceback(oracle.DNA, batch.ref, batch.ref_off, batch.query, batch.query_off, res,
                                scores=scores)
    return oracle.traceback(oracle.AA, batch.ref, batch.ref_off, batch.query, batch.query_off, res,
                            matrix=sc.BLOSUM62, encoding=sc.ENCODING, gaps=gaps)


def _check(aligner, batch, sc, kind, scores=None, gaps=None):
    res = np.ascontiguousarray(aligner.align_batch(batch, sc))
    ops, off = aligner.traceback_batch(batch, sc, res)
    eops, eoff, epscore = _oracle_trace(batch, kind, res, scores=scores, gaps=gaps)
    np.testing.assert_array_equal(off, eoff)
    np.testing.assert_array_equal(ops, eops)
    np.testing.assert_array_equal(epscore, np.where(res[:, 0] > 0, res[:, 0], 0))
    return res, ops, off


def _consumed(ops):
    """(reference symbols, query symbols) a path covers."""
    r = q = 0
    for v in ops:
        n, op = int(v) >> 4, int(v) & 15
        r += n if op in (2, 7, 8) else 0
        q += n if op in (1, 7, 8) else 0
    return r, q


def test_dna_against_oracle(built, workloads, aligner):
    gbsw = built
    b = workloads.PairBatch.concat([workloads.dna_throughput(3000, seed=101), workloads.mixed_dna(40, seed=102),
                                    workloads.PairBatch.from_strings(0, ["", "AAAA", "ACGTNNacgt" * 30, "A"],
                                                                     ["ACGT", "CCCC", "ACGTNNACGT" * 20, "A"])])
    res, ops, off = _check(aligner, b, gbsw.make_scoring(gbsw.DNA, scores=DNA_BENCH), 0, scores=DNA_BENCH)
    for k in range(b.n):
        seg = ops[off[k]:off[k + 1]]
        if res[k, 0] > 0:
            assert _consumed(seg) == (res[k, 2] - res[k, 1], res[k, 4] - res[k, 3])
        else:
            assert len(seg) == 0
    assert gbsw.cigar(ops[off[0]:off[1]])


@pytest.mark.parametrize("scores", [(1, -3, -3, -1), (1, 0, 0, 0), (2, 1, -3, -1), (5, -4, -10, -1)])
def test_dna_other_scorings(built, workloads, aligner, scores):
    gbsw = built
    b = workloads.custom_dna(800, 103, 20, 700, 10, 400, related=0.6)
    _check(aligner, b, gbsw.make_scoring(gbsw.DNA, scores=scores), 0, scores=scores)


def test_protein_against_oracle(built, workloads, aligner):
    gbsw = built
    b = workloads.protein(1500, seed=104)
    _check(aligner, b, gbsw.make_scoring(gbsw.PROTEIN, matrix=gbsw.scoring.BLOSUM62, gaps=AA_GAPS), 1,
           gaps=AA_GAPS)


def test_full_size_batch_in_several_launches(built, workloads, aligner):
    """100,000 pairs need more direction memory than one launch holds."""
    gbsw = built
    b = workloads.dna_throughput(100_000, seed=105)
    sc = gbsw.make_scoring(gbsw.DNA, scores=DNA_BENCH)
    res = np.ascontiguousarray(aligner.align_batch(b, sc))
    ops, off = aligner.traceback_batch(b, sc, res)
    idx = np.arange(0, b.n, 41)
    sub = b.subset(idx)
    eops, eoff, _ = _oracle_trace(sub, 0, res[idx], scores=DNA_BENCH)
    for t, k in enumerate(idx):
        np.testing.assert_array_equal(ops[off[k]:off[k + 1]], eops[eoff[t]:eoff[t + 1]], err_msg="pair %d" % k)
    assert int(off[-1]) == len(ops)


def test_bad_results_refused(built, workloads, aligner):
    gbsw = built
    b = workloads.dna_throughput(200, seed=106)
    sc = gbsw.make_scoring(gbsw.DNA, scores=DNA_BENCH)
    res = np.array(aligner.align_batch(b, sc))
    bad = res.copy()
    k = int(np.argmax(res[:, 0] > 0))
    bad[k, 2] = b.ref_lengths()[k] + 5  # end past the sequence
    with pytest.raises(gbsw.GbswError) as ei:
        aligner.traceback_batch(b, sc, bad)
    assert ei.value.status == -1
    # results of another scoring: the paths miss their scores
    other = gbsw.make_scoring(gbsw.DNA, scores=(1, -3, -3, -1))
    with pytest.raises(gbsw.GbswError):
        aligner.traceback_batch(b, other, res)
    # the context stays usable
    ops, off = aligner.traceback_batch(b, sc, res)
    assert len(off) == b.n + 1
