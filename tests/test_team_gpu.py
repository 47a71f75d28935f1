"""GPU tests of the block-per-pair passes (lane_group 128: the four warps of a
block share one pair, a column strip each, handing strip edges on through
bounded waits): bit-exact against the oracle and the default plan on long
pairs, on shapes that leave warps idle or give them many strips, on raw DNA
bytes and protein, and on reverse passes that stop early."""
import numpy as np
import pytest

from helpers import first_mismatches, oracle_batch

pytestmark = pytest.mark.gpu

DNA_BENCH = (3, -3, -6, -1)
AA_GAPS = (-6, -1)


@pytest.fixture(scope="module")
def team(built):
    a = built.Aligner(0, lane_group=128)
    yield a
    a.close()


def _dna(gbsw):
    return gbsw.make_scoring(gbsw.DNA, scores=DNA_BENCH)


def _check(got, exp):
    bad, count = first_mismatches(got, exp)
    assert count == 0, "%d mismatching pairs, first: %s" % (count, bad)


def test_team_long_dna(built, workloads, team):
    b = workloads.custom_dna(240, 80, 2000, 9000, 1500, 6000, related=0.7)
    got = team.align_batch(b, _dna(built))
    st = team.stats()
    assert (st["lane_group"], st["dual"]) == (128, 0), st
    _check(got, oracle_batch(b, 0, scores=DNA_BENCH))


def test_team_strip_counts_and_edges(built, workloads, team, aligner):
    """Shorter sides around the 256-column strip of a warp: one strip (three
    warps idle), exactly one, one plus a column, four, five (a warp takes two),
    many; empty sequences; and raw bytes (N, lower case)."""
    rng = np.random.default_rng(81)
    refs, qs = [], []
    for short in (1, 100, 255, 256, 257, 511, 1024, 1025, 1280, 1300, 3000):
        for _ in range(6):
            a = "".join(rng.choice(list("ACGT"), short))
            long_ = list(a * 2)[: short + int(rng.integers(0, 900))]
            for k in rng.integers(0, len(long_), len(long_) // 20):
                long_[k] = rng.choice(list("ACGT"))
            r, q = "".join(long_), a
            if rng.random() < 0.5:
                r, q = q, r
            refs.append(r)
            qs.append(q)
    refs += ["", "ACGT", "ACGTNNNNACGTacgt" * 40]
    qs += ["ACGT", "", "ACGTNACGTACGTacg" * 30]
    b = workloads.PairBatch.from_strings(0, refs, qs)
    got = team.align_batch(b, _dna(built))
    _check(got, oracle_batch(b, 0, scores=DNA_BENCH))
    np.testing.assert_array_equal(got, aligner.align_batch(b, _dna(built)))


def test_team_protein(built, workloads, team):
    b = workloads.custom_protein(150, 82, 600, 3000)
    sc = built.make_scoring(built.PROTEIN, matrix=built.scoring.BLOSUM62, gaps=AA_GAPS)
    _check(team.align_batch(b, sc), oracle_batch(b, 1, gaps=AA_GAPS))


def test_team_reverse_early_stops(built, workloads, team):
    """Identical and near-identical long pairs end their reverse pass in the
    first rows (the team's shared best stops the later strips); unrelated pairs
    search far; repeats tie often."""
    rng = np.random.default_rng(83)
    unit = "".join(rng.choice(list("ACGT"), 37))
    refs, qs = [], []
    for n in (700, 2600, 5000):
        s = "".join(rng.choice(list("ACGT"), n))
        refs += [s, s[: n // 2] + "T" + s[n // 2:], unit * (n // 37), "".join(rng.choice(list("ACGT"), n))]
        qs += [s, s, unit * (n // 50), "".join(rng.choice(list("ACGT"), n // 2 + 300))]
    b = workloads.PairBatch.from_strings(0, refs, qs)
    _check(team.align_batch(b, _dna(built)), oracle_batch(b, 0, scores=DNA_BENCH))


def test_team_matches_default_plan_on_mixed(built, workloads, team, aligner):
    b = workloads.mixed_dna(6000, seed=84)
    np.testing.assert_array_equal(team.align_batch(b, _dna(built)), aligner.align_batch(b, _dna(built)))
