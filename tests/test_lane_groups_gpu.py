"""GPU parity of every lane-group width of the int32 passes (4, 8, 16 and 32 lanes
per pair), forced through gbsw_options.lane_group, and of the width the library
picks by itself from the batch size.

Width 4 with DNA includes the dual-pair int16x2 kernel; the wider groups run
small batches.  Every width must give the reference's results bit for bit: the
golden fixtures (outputs of the reference's own kernels) and the oracle on each
scoring mode (A/C/G/T profile, raw DNA bytes, protein int8 profile, protein
scores outside int8).
"""
import importlib
import os
import sys

import numpy as np
import pytest

import oracle
from helpers import GOLDEN, first_mismatches, oracle_batch

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
import make_golden  # noqa: E402

pytestmark = pytest.mark.gpu

WIDTHS = [4, 8, 16, 32, 128]
DNA_BENCH = (3, -3, -6, -1)
AA_GAPS = (-6, -1)


@pytest.fixture(scope="module")
def aligners(built):
    al = {w: built.Aligner(0, lane_group=w) for w in WIDTHS}
    yield al
    for a in al.values():
        a.close()


def _check(got, exp):
    bad, count = first_mismatches(got, exp)
    assert count == 0, "%d mismatching pairs, first: %s" % (count, bad)


def _scoring(gbsw, kind, params):
    if kind in ("dna", 0):
        return gbsw.make_scoring(gbsw.DNA, scores=params)
    return gbsw.make_scoring(gbsw.PROTEIN, matrix=gbsw.scoring.BLOSUM62, gaps=params)


@pytest.mark.skipif(not GOLDEN, reason="golden fixtures not generated")
@pytest.mark.parametrize("width", WIDTHS)
def test_golden_fixtures_every_width(built, aligners, width):
    wl = importlib.import_module("gpu-bsw_gb300.workloads")
    for path in GOLDEN:
        kind, params, refs, qs, exp = make_golden.load_fixture(path)
        got = aligners[width].align_batch(wl.PairBatch.from_strings(0, refs, qs), _scoring(built, kind, params))
        bad, count = first_mismatches(got, exp)
        assert count == 0, (os.path.basename(path), count, bad)


@pytest.mark.parametrize("width", WIDTHS)
def test_dna_modes_every_width(built, workloads, aligners, width):
    al = aligners[width]
    sc = _scoring(built, 0, DNA_BENCH)
    # A/C/G/T pairs (profile kernels; dual-pair at width 4)
    b = workloads.dna_throughput(1500, seed=61)
    _check(al.align_batch(b, sc), oracle_batch(b, 0, scores=DNA_BENCH))
    # raw bytes and pairs longer than one strip of every width, shorter sequences above 1,024
    raw = workloads.PairBatch.from_strings(0, ["ACGTNNACGTacgt" * 40, "NNNNACGT" * 60, "A" * 900, "ACGT" * 700],
                                           ["CGTNNACG" * 30, "ACGTNNNN" * 40, "A" * 700, "ACGA" * 400])
    mixed = workloads.PairBatch.concat([raw, workloads.mixed_dna(40, seed=62)])
    _check(al.align_batch(mixed, sc), oracle_batch(mixed, 0, scores=DNA_BENCH))
    # other scorings, including zero gap penalties and a positive mismatch
    for scores in [(1, -3, -3, -1), (1, 0, 0, 0), (2, 1, -3, -1)]:
        c = workloads.custom_dna(300, 63, 20, 700, 10, 400, related=0.6)
        _check(al.align_batch(c, _scoring(built, 0, scores)), oracle_batch(c, 0, scores=scores))


@pytest.mark.parametrize("width", WIDTHS)
def test_protein_modes_every_width(built, workloads, aligners, width):
    al = aligners[width]
    sc = importlib.import_module("gpu-bsw_gb300.scoring")
    b = workloads.protein(600, seed=64)
    _check(al.align_batch(b, _scoring(built, 1, AA_GAPS)), oracle_batch(b, 1, gaps=AA_GAPS))
    # scores outside int8: the shared-memory matrix variant
    big = (np.asarray(sc.BLOSUM62, dtype=np.int16) * 20).astype(np.int16)
    gaps = (-60, -10)
    scb = built.make_scoring(built.PROTEIN, matrix=big, gaps=gaps)
    c = workloads.protein(300, seed=65)
    exp = oracle.align(oracle.AA, c.ref, c.ref_off, c.query, c.query_off, matrix=big, encoding=sc.ENCODING,
                       gaps=gaps)
    _check(al.align_batch(c, scb), exp)


def test_automatic_width_matches_forced(built, workloads, aligners, aligner):
    """The default (width from the batch size) gives the same results as every
    forced width, on batch sizes that select each of them."""
    sc = _scoring(built, 0, DNA_BENCH)
    for n in (1, 700, 3000, 9000, 20_000):
        b = workloads.dna_throughput(n, seed=66)
        auto = aligner.align_batch(b, sc)
        for w in (4, 8, 16, 32):
            np.testing.assert_array_equal(aligners[w].align_batch(b, sc), auto, err_msg="n=%d width=%d" % (n, w))
    idx = np.arange(0, b.n, 97)
    _check(auto[idx], oracle_batch(b.subset(idx), 0, scores=DNA_BENCH))


def test_lane_group_option_validation(built):
    a = built.Aligner(0)
    with pytest.raises(built.GbswError):
        a.set_options(lane_group=12)
    a.set_options(lane_group=16)
    a.set_options(lane_group=0)
    a.close()


def _bucket(gbsw, count):
    for q, edge in enumerate(gbsw.BUCKET_EDGES):
        if count <= edge:
            return q
    return len(gbsw.BUCKET_EDGES)


def _check_plan(gbsw, table, kind, batch, st, rtable=None):
    rtable = rtable or {}
    """The plan each length bin ran is the tuning table's entry for its pair count
    (forward and reverse)."""
    short = np.minimum(batch.ref_lengths(), batch.query_lengths()) < 512
    for b, count in ((0, int(short.sum())), (1, int((~short).sum()))):
        # -1: not read back (every bucket the batch size allows holds the same plan)
        assert st["bin_pairs"][b] in (count, -1), (b, st)
        if count == 0:
            continue
        dual, lanes = table[(kind, b, _bucket(gbsw, count))]
        assert (st["bin_dual"][b], st["bin_lanes"][b], st["bin_tuned"][b]) == (dual, lanes, 1), (b, count, st)
        rdual, rlanes = rtable.get((kind, b, _bucket(gbsw, count)), (dual, lanes))
        assert (st["rev_dual"][b], st["rev_lanes"][b]) == (rdual, rlanes), (b, count, st)


def test_automatic_plan_follows_the_tuning_table(built, workloads, aligners, aligner):
    """With no forced width each length bin runs the tuning table's plan for its
    pair count; the results agree with every forced width and with the oracle,
    and the call reports the plan it ran."""
    table, rtable = aligner.get_tuning(), aligner.get_tuning(reverse=True)
    sc = _scoring(built, 1, AA_GAPS)
    for n in (1000, 30_000):
        b = workloads.protein(n, seed=67)
        auto = aligner.align_batch(b, sc)
        _check_plan(built, table, 1, b, aligner.stats(), rtable)
        for w in (16, 32):
            np.testing.assert_array_equal(aligners[w].align_batch(b, sc), auto, err_msg="n=%d width=%d" % (n, w))
            assert aligners[w].stats()["dual"] == 1
        idx = np.arange(0, b.n, max(1, b.n // 300))
        _check(auto[idx], oracle_batch(b.subset(idx), 1, gaps=AA_GAPS))
    d = _scoring(built, 0, DNA_BENCH)
    for n in (5000, 20_000, 60_000, 100_000):
        b = workloads.dna_throughput(n, seed=68)
        aligner.align_batch(b, d)
        _check_plan(built, table, 0, b, aligner.stats(), rtable)


def test_long_pairs_wide_dual_class(built, workloads, aligners):
    """Large-batch plan (4 lanes): A/C/G/T pairs whose shorter sequence is >= 512
    run two per 16-lane group (the wide dual class), the rest two per 4-lane
    group; both against the oracle, forward and reverse."""
    b = workloads.PairBatch.concat([workloads.mixed_dna(600, seed=69),
                                    workloads.custom_dna(200, 70, 500, 1400, 480, 900, related=0.7)])
    assert (np.minimum(b.ref_lengths(), b.query_lengths()) >= 512).sum() > 100
    sc = _scoring(built, 0, DNA_BENCH)
    _check(aligners[4].align_batch(b, sc), oracle_batch(b, 0, scores=DNA_BENCH))
    assert aligners[4].stats()["dual"] == 1
