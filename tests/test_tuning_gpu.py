"""GPU tests of the per-length-bin plans and the autotuner (gbsw_tune_device,
gbsw_get_tuning / gbsw_set_tuning): the tuner's report is consistent (every
candidate timed per bin, the choice is the fastest), its choices land in the
table at the bins' pair-count buckets and the next call runs them, and every
variant the table can name -- per bin, dual int16x2 or int32, any lane count --
gives results bit-identical to the CPU oracle."""
import numpy as np
import pytest

from helpers import first_mismatches, oracle_batch

pytestmark = pytest.mark.gpu

DNA = (3, -3, -6, -1)
AA_GAPS = (-6, -1)
EDGES = (1000, 3000, 10000, 30000, 100000)


def _bucket(pairs):
    return sum(pairs > e for e in EDGES)


def _check(got, exp):
    bad, count = first_mismatches(got, exp)
    assert count == 0, "%d mismatching pairs, first: %s" % (count, bad)


def _device(torch, batch):
    d = [torch.from_numpy(x).to("cuda:0") for x in (batch.ref, batch.ref_off, batch.query, batch.query_off)]
    ml = int(max(batch.ref_lengths().max(), batch.query_lengths().max()))
    return d, ml


def _mixed(workloads):
    # both bins: shorter sides 150-300 (short bin) and 600-900 (long bin)
    return workloads.PairBatch.concat([workloads.dna_throughput(2500, seed=31),
                                       workloads.custom_dna(300, 32, 900, 2000, 600, 900, related=0.8)])


def test_tuner_report_and_table(built, workloads):
    torch = pytest.importorskip("torch")
    batch = _mixed(workloads)
    sc = built.make_scoring(built.DNA, scores=DNA)
    a = built.Aligner(0)
    d, ml = _device(torch, batch)
    rep = a.tune_device(sc, d[0].data_ptr(), d[1].data_ptr(), d[2].data_ptr(), d[3].data_ptr(), batch.n, ml, reps=1)
    cands = rep["candidates"]
    assert (1, 4) in cands and (0, 32) in cands and (0, 128) in cands and len(cands) == 8, cands
    short = np.minimum(batch.ref_lengths(), batch.query_lengths())
    assert [b["pairs"] for b in rep["bins"]] == [int((short < 512).sum()), int((short >= 512).sum())]
    table = a.get_tuning()
    rtable = a.get_tuning(reverse=True)
    for b, info in enumerate(rep["bins"]):
        assert all(t > 0 for t in info["ms_forward"] + info["ms_reverse"]), info
        assert info["chosen"] == cands[int(np.argmin(info["ms_forward"]))]
        assert info["chosen_reverse"] == cands[int(np.argmin(info["ms_reverse"]))]
        assert info["bucket"] == _bucket(info["pairs"])
        assert table[(0, b, info["bucket"])] == info["chosen"]
        assert rtable[(0, b, info["bucket"])] == info["chosen_reverse"]
    # the next call on the same batch runs the tuned plan of each bin
    got = a.align_batch(batch, sc)
    st = a.stats()
    # bin_pairs -1: not read back, as every bucket the batch size allows holds the same plan
    assert st["bin_tuned"] == [1, 1] and st["bin_pairs"] in ([b["pairs"] for b in rep["bins"]], [-1, -1]), st
    assert [(st["bin_dual"][b], st["bin_lanes"][b]) for b in range(2)] == [b["chosen"] for b in rep["bins"]]
    assert [(st["rev_dual"][b], st["rev_lanes"][b]) for b in range(2)] == [b["chosen_reverse"] for b in rep["bins"]]
    _check(got, oracle_batch(batch, 0, scores=DNA))
    a.close()


@pytest.mark.parametrize("kind", [0, 1])
def test_every_variant_per_bin_is_exact(built, workloads, kind):
    if kind == 0:
        batch = _mixed(workloads)
        sc = built.make_scoring(built.DNA, scores=DNA)
        exp = oracle_batch(batch, 0, scores=DNA)
        variants = [(1, 4), (1, 8), (1, 16), (0, 4), (0, 8), (0, 16), (0, 32), (0, 128)]
    else:
        batch = workloads.PairBatch.concat([workloads.protein(1200, seed=33),
                                            workloads.custom_protein(150, 34, 520, 900)])
        sc = built.make_scoring(built.PROTEIN, matrix=built.scoring.BLOSUM62, gaps=AA_GAPS)
        exp = oracle_batch(batch, 1, gaps=AA_GAPS)
        variants = [(1, 16), (1, 32), (0, 4), (0, 8), (0, 16), (0, 32), (0, 128)]
    short = np.minimum(batch.ref_lengths(), batch.query_lengths())
    buckets = [_bucket(int((short < 512).sum())), _bucket(int((short >= 512).sum()))]
    a = built.Aligner(0)
    # each variant in the short bin, paired with another in the long bin, and
    # other variants again in the reverse pass
    for k, v in enumerate(variants):
        w = variants[(k + 3) % len(variants)]
        rv, rw = variants[(k + 1) % len(variants)], variants[(k + 5) % len(variants)]
        a.set_tuning({(kind, 0, buckets[0]): v, (kind, 1, buckets[1]): w},
                     {(kind, 0, buckets[0]): rv, (kind, 1, buckets[1]): rw})
        _check(a.align_batch(batch, sc), exp)
        st = a.stats()
        assert st["bin_tuned"] == [1, 1], (v, w, st)
        assert (st["bin_dual"][0], st["bin_lanes"][0]) == v and (st["bin_dual"][1], st["bin_lanes"][1]) == w
        assert (st["rev_dual"][0], st["rev_lanes"][0]) == rv and (st["rev_dual"][1], st["rev_lanes"][1]) == rw
    a.close()


def test_dual_reverse_after_int32_forward_above_int16(built, workloads):
    """An int32 forward pass followed by a dual-pair reverse pass: pairs whose
    score exceeds what the int16x2 kernels hold (identical 12 kb strings at +3
    score 36,000) take the int32 class in the reverse pass and keep exact
    begins; the others run dual."""
    rng = np.random.default_rng(35)
    big = ["".join(rng.choice(list("ACGT"), 12_000)) for _ in range(3)]
    b = workloads.PairBatch.concat([workloads.PairBatch.from_strings(0, big, big),
                                    workloads.custom_dna(200, 36, 900, 2000, 600, 900, related=0.8)])
    sc = built.make_scoring(built.DNA, scores=DNA)
    a = built.Aligner(0)
    entries = {(0, 1, q): (0, 32) for q in range(6)}
    entries.update({(0, 0, q): (0, 32) for q in range(6)})
    a.set_tuning(entries, {(0, 1, q): (1, 16) for q in range(6)})
    got = a.align_batch(b, sc)
    assert (got[:3, 0] == 36_000).all()
    _check(got, oracle_batch(b, 0, scores=DNA))
    assert a.stats()["rev_dual"][1] == 1
    a.close()


def test_set_tuning_rejects_variants_without_a_kernel(built):
    a = built.Aligner(0)
    with pytest.raises(built.GbswError):
        a.set_tuning({(0, 0, 0): (1, 32)})  # no 32-lane DNA dual kernel
    with pytest.raises(built.GbswError):
        a.set_tuning({(1, 1, 2): (0, 12)})
    with pytest.raises(built.GbswError):
        a.set_tuning({(1, 1, 2): (2, 16)})
    with pytest.raises(built.GbswError):
        a.set_tuning({}, {(0, 0, 0): (1, 32)})  # the reverse table is checked too
    a.set_tuning({})  # an empty table: every bin falls back to the size rule
    assert a.get_tuning() == {} and a.get_tuning(reverse=True) == {}
    a.close()
