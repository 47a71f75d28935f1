"""GPU tests of the schedule's per-pair checks (forward_keys reads each pair's
bytes in 16-byte words): a single byte outside A/C/G/T -- at any position and
any alignment of the sequence in memory -- sends its pair to the raw-byte class,
and a single protein byte outside the encoding table is reported."""
import numpy as np
import pytest

from helpers import first_mismatches, oracle_batch

pytestmark = pytest.mark.gpu

DNA = (3, -3, -6, -1)


def test_one_non_acgt_byte_at_every_position(built, workloads, aligner):
    # 'N' in the reference against 'G' in the query: a mismatch as raw bytes, a
    # match if the pair were scored through the A/C/G/T profile (N reads as G)
    rng = np.random.default_rng(91)
    refs, qs = [], []
    for lead in range(17):              # shifts the sequence's start against 16-byte words
        refs.append("".join(rng.choice(list("ACGT"), lead + 3)))
        qs.append("".join(rng.choice(list("ACGT"), 5)))
        for pos in range(0, 70, 3):
            base = list("".join(rng.choice(list("ACGT"), 70)))
            q = base.copy()
            base[pos] = "N"
            q[pos] = "G"
            refs.append("".join(base))
            qs.append("".join(q))
    b = workloads.PairBatch.from_strings(0, refs, qs)
    got = aligner.align_batch(b, built.make_scoring(built.DNA, scores=DNA))
    bad, count = first_mismatches(got, oracle_batch(b, 0, scores=DNA))
    assert count == 0, bad


@pytest.mark.parametrize("lead", [0, 5, 15, 16, 31])
def test_protein_byte_outside_the_table_anywhere(built, workloads, aligner, lead):
    sc = built.make_scoring(built.PROTEIN, matrix=built.scoring.BLOSUM62, gaps=(-6, -1))
    for pos in (0, 7, 16, 33, 64):
        s = list("ARNDCQEGHILKMFPSTWYV" * 4)
        s[pos] = "z"
        b = workloads.PairBatch.from_strings(1, ["A" * lead, "".join(s)], ["ARND", "ARNDCQ"])
        with pytest.raises(built.GbswError) as ei:
            aligner.align_batch(b, sc)
        assert ei.value.status == -2, (lead, pos)
