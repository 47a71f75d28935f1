"""GPU tests of the int16x2 overflow detection: pairs run two per group in the
dual-pair int16x2 passes, and a pair whose best score exceeds 32767 - m (m = the
largest single-cell score) may have wrapped there, so the forward pass queues it
for the int32 pass instead.  Every result must equal the CPU oracle's (int32
throughout), and the rerun count must be exactly the pairs whose true score
exceeds that limit: pairs below it stay in int16x2, however long they are."""
import importlib

import numpy as np
import pytest

import oracle
from helpers import first_mismatches

pytestmark = pytest.mark.gpu


def _rng_seq(rng, alphabet, n):
    return bytes(rng.choice(np.frombuffer(alphabet, np.uint8), n))


def _mutate(rng, s, alphabet, rate):
    b = bytearray(s)
    for k in range(len(b)):
        if rng.random() < rate:
            b[k] = alphabet[rng.integers(len(alphabet))]
    return bytes(b)


def _dna_pairs(rng):
    refs, qs = [], []
    for k in range(60):
        r = _rng_seq(rng, b"ACGT", int(rng.integers(250, 520)))
        if k % 3 == 0:    # identical: 100 x length > 32667 from 327 columns on
            q = r[10:10 + int(rng.integers(300, 420))]
        elif k % 3 == 1:  # close to the limit from both sides
            q = _mutate(rng, r[:int(rng.integers(280, 380))], b"ACGT", 0.02)
        else:             # unrelated
            q = _rng_seq(rng, b"ACGT", int(rng.integers(100, 400)))
        refs.append(r)
        qs.append(q)
    return refs, qs


def _check(got, exp):
    bad, count = first_mismatches(got, exp)
    assert count == 0, "%d mismatching pairs, first: %s" % (count, bad)


def test_dna_overflow_pairs_rerun_in_int32(built, workloads):
    rng = np.random.default_rng(11)
    refs, qs = _dna_pairs(rng)
    wl = workloads
    batch = wl.PairBatch.concat([wl.PairBatch.from_strings(0, refs, qs), wl.dna_throughput(3000, seed=12)])
    scores = (100, -100, -150, -50)  # int8 profile scores; limit 32767 - 100
    exp = oracle.align(oracle.DNA, batch.ref, batch.ref_off, batch.query, batch.query_off, scores=scores)
    over = int(np.count_nonzero(exp[:, 0] > 32767 - 100))
    assert 10 < over < batch.n  # the batch holds both kinds
    sc = built.make_scoring(built.DNA, scores=scores)
    for width in (4, 16):
        a = built.Aligner(0, lane_group=width)
        _check(a.align_batch(batch, sc), exp)
        st = a.stats()
        assert st["dual"] == 1 and st["reruns"] == over, (width, st)
        # the int16 results truncate like the reference's short arrays
        r16 = a.align_batch(batch, sc, int16=True)
        assert np.array_equal(r16, exp.astype(np.int16))
        a.close()


def test_long_dna_pairs_below_the_limit_stay_in_int16(built, workloads):
    # 6 kb pairs at +3 score up to 18,000: beyond the old static bound of
    # 3 x length < 16,384, inside int16, so no rerun
    rng = np.random.default_rng(13)
    refs, qs = [], []
    for k in range(6):
        r = _rng_seq(rng, b"ACGT", 6000 + 37 * k)
        refs.append(r)
        qs.append(r[k:k + 5800] if k % 2 == 0 else _mutate(rng, r[:5900], b"ACGT", 0.01))
    batch = workloads.PairBatch.from_strings(0, refs, qs)
    scores = (3, -3, -6, -1)
    exp = oracle.align(oracle.DNA, batch.ref, batch.ref_off, batch.query, batch.query_off, scores=scores)
    assert exp[:, 0].max() > 16384
    a = built.Aligner(0, lane_group=4)
    _check(a.align_batch(batch, built.make_scoring(built.DNA, scores=scores)), exp)
    st = a.stats()
    assert st["dual"] == 1 and st["reruns"] == 0, st
    a.close()


def test_protein_overflow_pairs_rerun_in_int32(built, workloads):
    sc_mod = importlib.import_module("gpu-bsw_gb300.scoring")
    matrix = (np.asarray(sc_mod.BLOSUM62, dtype=np.int16) * 10)  # entries -40 .. 110: still int8
    gaps = (-60, -10)
    rng = np.random.default_rng(17)
    aa = b"ARNDCQEGHILKMFPSTWYV"
    refs, qs = [], []
    for k in range(40):
        r = _rng_seq(rng, aa, int(rng.integers(400, 1000)))
        q = r[:int(rng.integers(len(r) // 2, len(r)))] if k % 2 == 0 else _rng_seq(rng, aa, int(rng.integers(100, 700)))
        refs.append(r)
        qs.append(q)
    batch = workloads.PairBatch.concat([workloads.PairBatch.from_strings(1, refs, qs),
                                        workloads.protein(800, seed=18)])
    exp = oracle.align(oracle.AA, batch.ref, batch.ref_off, batch.query, batch.query_off, matrix=matrix,
                       encoding=sc_mod.ENCODING, gaps=gaps)
    over = int(np.count_nonzero(exp[:, 0] > 32767 - int(matrix.max())))
    assert over >= 5
    sc = built.make_scoring(built.PROTEIN, matrix=matrix, gaps=gaps)
    a = built.Aligner(0, lane_group=16)
    _check(a.align_batch(batch, sc), exp)
    st = a.stats()
    assert st["dual"] == 1 and st["reruns"] == over, st
    a.close()
