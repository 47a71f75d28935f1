"""GPU tests of the serving loop (gbsw_server_*): continuous batching of jobs.

The central property: every job's results are the same whether it ran alone or
merged into launches with other jobs, submitted from several threads at once,
with batches overlapping on the device -- and they equal the oracle's.  All
results are integers, so "the same" means bit for bit.
"""
import threading

import numpy as np
import pytest

from helpers import first_mismatches, oracle_batch

pytestmark = pytest.mark.gpu

DNA_SCORES = (3, -3, -6, -1)
GAPS = (-6, -1)


def _scorings(gbsw):
    return {0: gbsw.make_scoring(gbsw.DNA, scores=DNA_SCORES),
            1: gbsw.make_scoring(gbsw.PROTEIN, matrix=gbsw.scoring.BLOSUM62, gaps=GAPS)}


def _jobs(wl):
    jobs = wl.serving_jobs(20, seed=11, max_pairs=1200)
    # edge jobs: one pair, raw-byte DNA (not A/C/G/T: other kernel classes), a
    # pair with an empty sequence, and a no-hit pair
    jobs.append((0, wl.dna_throughput(1, seed=12)))
    jobs.append((0, wl.PairBatch.from_strings(0, ["ACGTNNACGTacgt" * 20, "", "AAAA", "NNNNACGT" * 30],
                                              ["CGTNNACG" * 9, "ACGT", "CCCC", "ACGTNNNN" * 12])))
    jobs.append((1, wl.protein(3, seed=13)))
    return jobs


def test_results_alone_equal_results_in_the_mix(built, workloads):
    gbsw = built
    sc = _scorings(gbsw)
    jobs = _jobs(workloads)

    with gbsw.Server(0, slots=1) as srv:
        alone = [srv.submit_batch(b, sc[kind]).wait().copy() for kind, b in jobs]
        st = srv.stats()
    assert st["jobs"] == len(jobs) and st["peak_running"] == 1

    # three submitting threads, four slots, launches capped so that both merged
    # and unmerged batches occur
    mixed = [None] * len(jobs)
    with gbsw.Server(0, slots=4, max_batch_pairs=3000) as srv:
        def submit(part):
            handles = [(k, srv.submit_batch(jobs[k][1], sc[jobs[k][0]])) for k in part]
            for k, h in handles:
                mixed[k] = h.wait().copy()

        threads = [threading.Thread(target=submit, args=(list(range(t, len(jobs), 3)),)) for t in range(3)]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        st = srv.stats()
    assert st["jobs"] == len(jobs) and st["hbm_in_use"] == 0 and st["queued"] == 0

    for k, (kind, b) in enumerate(jobs):
        assert mixed[k].shape == (b.n, 5)
        np.testing.assert_array_equal(mixed[k], alone[k], err_msg="job %d" % k)
        exp = oracle_batch(b, kind, scores=DNA_SCORES if kind == 0 else None, gaps=GAPS)
        bad, count = first_mismatches(alone[k], exp)
        assert count == 0, (k, bad)


def test_jobs_that_arrive_during_a_batch_are_merged(built, workloads):
    """One slot: a large job occupies the device while small jobs queue; the queued
    jobs of one scoring must leave in fewer launches than jobs."""
    gbsw = built
    sc = _scorings(gbsw)
    big = workloads.dna_throughput(100_000, seed=21)
    small = [workloads.dna_throughput(50, seed=30 + k) for k in range(24)]
    with gbsw.Server(0, slots=1, max_batch_pairs=200_000) as srv:
        hb = srv.submit_batch(big, sc[0])
        hs = [srv.submit_batch(b, sc[0]) for b in small]
        outs = [h.wait().copy() for h in hs]
        hb.wait()
        st = srv.stats()
    assert st["jobs"] == 25
    assert st["batches"] < 25, st
    for b, got in zip(small, outs):
        bad, count = first_mismatches(got, oracle_batch(b, 0, scores=DNA_SCORES))
        assert count == 0, bad


def test_batches_overlap_and_budget_limits_admission(built, workloads):
    gbsw = built
    sc = _scorings(gbsw)
    jobs = [workloads.dna_throughput(20_000, seed=40 + k) for k in range(8)]
    footprint = int(jobs[0].ref.size + jobs[0].query.size + 65 * jobs[0].n)
    # room for every job: several batches run at once
    with gbsw.Server(0, slots=4, max_batch_pairs=20_000) as srv:
        outs = [h.wait().copy() for h in [srv.submit_batch(b, sc[0]) for b in jobs]]
        st = srv.stats()
    assert st["peak_running"] >= 2, st
    # room for one job only: batches never overlap, and each job runs alone
    with gbsw.Server(0, slots=4, hbm_budget=int(footprint * 1.5), max_batch_pairs=1_000_000) as srv:
        outs2 = [h.wait().copy() for h in [srv.submit_batch(b, sc[0]) for b in jobs]]
        st2 = srv.stats()
    assert st2["peak_running"] == 1 and st2["batches"] == len(jobs), st2
    # a job larger than the whole budget still runs, alone
    with gbsw.Server(0, slots=2, hbm_budget=1 << 20) as srv:
        outs3 = [h.wait().copy() for h in [srv.submit_batch(b, sc[0]) for b in jobs[:2]]]
        assert srv.stats()["peak_running"] == 1
    for a, b, c in zip(outs, outs2, outs3):
        np.testing.assert_array_equal(a, b)
    for a, c in zip(outs[:2], outs3):
        np.testing.assert_array_equal(a, c)


def test_server_input_errors(built, workloads):
    gbsw = built
    sc = _scorings(gbsw)
    with gbsw.Server(0, slots=2) as srv:
        good = srv.submit_batch(workloads.protein(100, seed=50), sc[1])
        bad = workloads.PairBatch.from_strings(1, ["ARND", "ARNDz"], ["ARN", "RND"])
        with pytest.raises(gbsw.GbswError) as ei:
            srv.submit_batch(bad, sc[1])
        assert ei.value.status == -2
        with pytest.raises(gbsw.GbswError) as ei:
            srv.submit_batch(workloads.protein(2, seed=51), gbsw.make_scoring(gbsw.PROTEIN,
                                                                              matrix=gbsw.scoring.BLOSUM62,
                                                                              gaps=(1, -1)))
        assert ei.value.status == -1
        empty = srv.submit(sc[0], np.zeros(0, np.uint8), np.zeros(1, np.int64), np.zeros(0, np.uint8),
                           np.zeros(1, np.int64))
        assert empty.wait().shape == (0, 5)
        got = good.wait()
        exp = oracle_batch(workloads.protein(100, seed=50), 1, gaps=GAPS)
        np.testing.assert_array_equal(got, exp)
        # each job is waited for once; an unknown id is an error
        rc = srv.lib.gbsw_server_wait(srv.handle, 10**9, 0.0, None)
        assert rc == -1
        # a job still running when the timeout expires stays known
        big = srv.submit_batch(workloads.dna_throughput(100_000, seed=52), sc[0])
        with pytest.raises(TimeoutError):
            big.wait(timeout=0.0)
        assert big.wait().shape == (100_000, 5)


def test_packed_jobs_equal_raw_jobs(built, workloads):
    """Jobs submitted as packed streams (they stay packed through admission and in
    HBM, and are unpacked by the gather) give the same rows as the same jobs
    submitted raw, merged into the same launches or not; escapes included."""
    gbsw = built
    sc = _scorings(gbsw)
    jobs = _jobs(workloads)
    with gbsw.Server(0, slots=3, max_batch_pairs=4000) as srv:
        handles = []
        for kind, b in jobs:
            pr, pq = gbsw.pack(kind, b.ref), gbsw.pack(kind, b.query)
            handles.append((srv.submit_packed(sc[kind], pr, b.ref_off, pq, b.query_off),
                            srv.submit_batch(b, sc[kind])))
        for (hp, hr), (kind, b) in zip(handles, jobs):
            np.testing.assert_array_equal(hp.wait(), hr.wait())
        # the raw-byte DNA job travels with escape runs
        assert gbsw.pack(0, jobs[-2][1].ref).nruns > 0
        # errors: offsets that do not start at 0, a stream shorter than its
        # offsets, a protein escape outside the encoding table
        b = workloads.plain_dna(5, seed=70)
        pr, pq = gbsw.pack(0, b.ref), gbsw.pack(0, b.query)
        with pytest.raises(gbsw.GbswError) as ei:
            srv.submit_packed(sc[0], pr, b.ref_off + 1, pq, b.query_off)
        assert ei.value.status == -1
        short = gbsw.PackedStream(0, pr.words, pr.nsym - 1, pr.run_at, pr.run_off, pr.run_bytes)
        with pytest.raises(gbsw.GbswError) as ei:
            srv.submit_packed(sc[0], short, b.ref_off, pq, b.query_off)
        assert ei.value.status == -1
        bad = workloads.PairBatch.from_strings(1, ["ARNDz"], ["ARN"])
        with pytest.raises(gbsw.GbswError) as ei:
            srv.submit_packed(sc[1], gbsw.pack(1, bad.ref), bad.ref_off, gbsw.pack(1, bad.query), bad.query_off)
        assert ei.value.status == -2
        st = srv.stats()
    assert st["hbm_in_use"] == 0 and st["queued"] == 0
