"""GPU parity tests: the CUDA path (through the C ABI) against the reference's own
outputs (golden fixtures) and against the CPU oracle, bit-exact."""
import importlib
import os
import subprocess
import sys

import numpy as np
import pytest

from helpers import GOLDEN, first_mismatches, oracle_batch

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
import make_golden  # noqa: E402

pytestmark = pytest.mark.gpu

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DNA_BENCH = (3, -3, -6, -1)
AA_GAPS = (-6, -1)


def _scoring(gbsw, kind, params):
    if kind in ("dna", 0):
        return gbsw.make_scoring(gbsw.DNA, scores=params)
    return gbsw.make_scoring(gbsw.PROTEIN, matrix=gbsw.scoring.BLOSUM62, gaps=params)


def _check(got, exp):
    bad, count = first_mismatches(got, exp)
    assert count == 0, "%d mismatching pairs, first: %s" % (count, bad)


@pytest.mark.skipif(not GOLDEN, reason="golden fixtures not generated")
@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
def test_reference_outputs_bit_exact(aligner, built, path):
    kind, params, refs, qs, exp = make_golden.load_fixture(path)
    wl = importlib.import_module("gpu-bsw_gb300.workloads")
    batch = wl.PairBatch.from_strings(0, refs, qs)
    got = aligner.align_batch(batch, _scoring(built, kind, params))
    _check(got, exp)


@pytest.mark.parametrize("use_dpx", [True, False])
def test_plain_dna_1000_pairs(built, workloads, use_dpx):
    a = built.Aligner(0, use_dpx=use_dpx)
    b = workloads.plain_dna(1000, seed=1)
    _check(a.align_batch(b, _scoring(built, 0, DNA_BENCH)), oracle_batch(b, 0, scores=DNA_BENCH))
    a.close()


def test_dna_throughput_subset(aligner, built, workloads):
    b = workloads.dna_throughput(6000, seed=2)
    _check(aligner.align_batch(b, _scoring(built, 0, DNA_BENCH)), oracle_batch(b, 0, scores=DNA_BENCH))


def test_protein_subset(aligner, built, workloads):
    b = workloads.protein(1500, seed=3)
    _check(aligner.align_batch(b, _scoring(built, 1, AA_GAPS)), oracle_batch(b, 1, gaps=AA_GAPS))


def test_mixed_with_long_pairs(aligner, built, workloads):
    # includes pairs beyond the reference's 1,024 limit (oracle-only parity)
    b = workloads.mixed_dna(400, seed=4)
    assert (b.query_lengths() > 1024).any()
    _check(aligner.align_batch(b, _scoring(built, 0, DNA_BENCH)), oracle_batch(b, 0, scores=DNA_BENCH))


@pytest.mark.parametrize("scores", [(1, -3, -3, -1), (2, -1, -2, -2), (1, 0, 0, 0), (5, -4, -10, -1),
                                    (2, 1, -3, -1)])
def test_other_dna_scorings(aligner, built, workloads, scores):
    b = workloads.custom_dna(600, 31, 20, 700, 10, 400, related=0.6)
    _check(aligner.align_batch(b, _scoring(built, 0, scores)), oracle_batch(b, 0, scores=scores))


def test_edge_cases(aligner, built, workloads):
    wl = workloads
    refs = ["", "A", "A", "ACGT", "AAAA", "ACGTACGT", "N", "acgtNN", "G" * 3000, "ACGT" * 900,
            "T", "CCCCCCCCCC"]
    qs = ["ACGT", "", "A", "ACGT", "CCCC", "CGTA", "N", "ACGTnn", "G" * 2500, "ACGA" * 300,
          "T" * 1500, "C"]
    b = wl.PairBatch.from_strings(0, refs, qs)
    got = aligner.align_batch(b, _scoring(built, 0, DNA_BENCH))
    _check(got, oracle_batch(b, 0, scores=DNA_BENCH))
    assert got[0].tolist() == [0, -1, -1, -1, -1]   # empty reference
    assert got[4].tolist() == [0, -1, -1, -1, -1]   # no positive cell


def test_single_pair_batches(aligner, built, workloads):
    b = workloads.plain_dna(5, seed=8)
    exp = oracle_batch(b, 0, scores=DNA_BENCH)
    for k in range(5):
        sub = b.subset([k])
        _check(aligner.align_batch(sub, _scoring(built, 0, DNA_BENCH)), exp[k:k + 1])


def test_int16_results_match_int32(aligner, built, workloads):
    b = workloads.plain_dna(300, seed=9)
    sc = _scoring(built, 0, DNA_BENCH)
    r32 = aligner.align_batch(b, sc)
    r16 = aligner.align_batch(b, sc, int16=True)
    assert np.array_equal(r16.astype(np.int32), r32)


def test_input_errors(aligner, built, workloads):
    b = workloads.PairBatch.from_strings(1, ["ACDE"], ["ACDa"])
    with pytest.raises(built.GbswError) as e:
        aligner.align_batch(b, _scoring(built, 1, AA_GAPS))
    assert e.value.status == -2
    with pytest.raises(built.GbswError) as e:
        aligner.align_batch(b, built.make_scoring(built.DNA, scores=(3, -3, 1, -1)))
    assert e.value.status == -1
    long_ = workloads.PairBatch.from_strings(0, ["A" * 70000], ["A"])
    with pytest.raises(built.GbswError) as e:
        aligner.align_batch(long_, _scoring(built, 0, DNA_BENCH))
    assert e.value.status == -3
    # the context stays usable after errors
    ok = workloads.plain_dna(10, seed=1)
    _check(aligner.align_batch(ok, _scoring(built, 0, DNA_BENCH)), oracle_batch(ok, 0, scores=DNA_BENCH))


def test_python_driver_mirror(built):
    wl = importlib.import_module("gpu-bsw_gb300.workloads")
    b = wl.plain_dna(50, seed=12)
    contigs = [b.strings(k)[0].decode() for k in range(b.n)]
    reads = [b.strings(k)[1].decode() for k in range(b.n)]
    r = built.kernel_driver_dna(reads, contigs, [3, -3, -6, -1])
    exp = oracle_batch(b, 0, scores=DNA_BENCH)
    got = np.stack([r.top_scores, r.ref_begin, r.ref_end, r.query_begin, r.query_end], axis=1)
    _check(got.astype(np.int32), exp)
    pb = wl.protein(40, seed=13)
    contigs = [pb.strings(k)[0].decode() for k in range(pb.n)]
    reads = [pb.strings(k)[1].decode() for k in range(pb.n)]
    r = built.kernel_driver_aa(reads, contigs, list(built.scoring.BLOSUM62), -6, -1)
    got = np.stack([r.top_scores, r.ref_begin, r.ref_end, r.query_begin, r.query_end], axis=1)
    _check(got.astype(np.int32), oracle_batch(pb, 1, gaps=AA_GAPS))
    assert built.get_tot_gpu_mem(0) > 100 * 2**30


def test_device_entry_matches_host_entry(aligner, built, workloads):
    torch = pytest.importorskip("torch")
    b = workloads.dna_throughput(3000, seed=21)
    sc = _scoring(built, 0, DNA_BENCH)
    host = aligner.align_batch(b, sc)
    dev = torch.device("cuda", 0)
    ref = torch.from_numpy(b.ref).to(dev)
    qry = torch.from_numpy(b.query).to(dev)
    ro = torch.from_numpy(b.ref_off).to(dev)
    qo = torch.from_numpy(b.query_off).to(dev)
    out = torch.full((5, b.n), -7, dtype=torch.int32, device=dev)
    s = torch.cuda.current_stream(dev)
    max_len = int(max(b.ref_lengths().max(), b.query_lengths().max()))
    aligner.align_device(sc, ref.data_ptr(), ro.data_ptr(), qry.data_ptr(), qo.data_ptr(), b.n, max_len,
                         out[0].data_ptr(), out[1].data_ptr(), out[2].data_ptr(), out[3].data_ptr(),
                         out[4].data_ptr(), s.cuda_stream)
    aligner.check(s.cuda_stream)
    assert np.array_equal(out.cpu().numpy().T, host)


@pytest.mark.parametrize("shift", [1, 3])
def test_device_entry_unaligned_buffers_dual_path(aligner, built, workloads, shift):
    """Sequence buffers that start at an odd byte, on a batch large enough for the
    dual-pair kernel (its forward pass reads row symbols as aligned words), with an
    odd pair count so that the last unit holds one pair."""
    torch = pytest.importorskip("torch")
    b = workloads.dna_throughput(30_001, seed=22)
    sc = _scoring(built, 0, DNA_BENCH)
    host = aligner.align_batch(b, sc)
    assert aligner.stats()["dual"] == 1
    dev = torch.device("cuda", 0)
    ref_buf = torch.zeros(len(b.ref) + 8, dtype=torch.uint8, device=dev)
    qry_buf = torch.zeros(len(b.query) + 8, dtype=torch.uint8, device=dev)
    ref_buf[shift:shift + len(b.ref)] = torch.from_numpy(b.ref).to(dev)
    qry_buf[shift:shift + len(b.query)] = torch.from_numpy(b.query).to(dev)
    ro = torch.from_numpy(b.ref_off).to(dev)
    qo = torch.from_numpy(b.query_off).to(dev)
    out = torch.full((5, b.n), -7, dtype=torch.int32, device=dev)
    s = torch.cuda.current_stream(dev)
    max_len = int(max(b.ref_lengths().max(), b.query_lengths().max()))
    aligner.align_device(sc, ref_buf.data_ptr() + shift, ro.data_ptr(), qry_buf.data_ptr() + shift, qo.data_ptr(),
                         b.n, max_len, out[0].data_ptr(), out[1].data_ptr(), out[2].data_ptr(), out[3].data_ptr(),
                         out[4].data_ptr(), s.cuda_stream)
    aligner.check(s.cuda_stream)
    assert aligner.stats()["dual"] == 1
    assert np.array_equal(out.cpu().numpy().T, host)
    idx = np.arange(0, b.n, 97)
    assert np.array_equal(host[idx], oracle_batch(b.subset(idx), 0, scores=DNA_BENCH))


def test_full_size_dna_throughput_properties(aligner, built, workloads):
    """The whole 100,000-pair DNA batch: deterministic, sane, and sampled pairs equal the oracle."""
    b = workloads.dna_throughput(100_000, seed=2)
    sc = _scoring(built, 0, DNA_BENCH)
    r1 = aligner.align_batch(b, sc)
    r2 = aligner.align_batch(b, sc)
    assert np.array_equal(r1, r2)
    score, rb, re_, qb, qe = r1.T
    pos = score > 0
    assert pos.all()
    assert (rb[pos] >= 0).all() and (rb[pos] < re_[pos]).all() and (re_[pos] <= b.ref_lengths()[pos]).all()
    assert (qb[pos] >= 0).all() and (qb[pos] < qe[pos]).all() and (qe[pos] <= b.query_lengths()[pos]).all()
    rng = np.random.default_rng(0)
    idx = rng.choice(b.n, 400, replace=False)
    sub = b.subset(idx)
    _check(r1[idx], oracle_batch(sub, 0, scores=DNA_BENCH))
    # re-aligning the reported segments gives back the same score
    segs_r, segs_q = [], []
    for k in idx[:200]:
        r, q = b.strings(k)
        segs_r.append(r[rb[k]:re_[k]])
        segs_q.append(q[qb[k]:qe[k]])
    seg = workloads.PairBatch.from_strings(0, segs_r, segs_q)
    again = aligner.align_batch(seg, sc)
    assert np.array_equal(again[:, 0], score[idx[:200]])


@pytest.mark.parametrize("devices", [None, "0,0,0"])
def test_cpp_dropin_program(built, tmp_path, devices):
    """A C++ caller written against the reference's API, linked to libgbsw.so.
    With GBSW_DEVICES listing device 0 three times, the drop-in splits the call
    into three cell-balanced ranges run by three host threads, each with its own
    context: the multi-GPU path, exercised on one GPU."""
    src = tmp_path / "caller.cpp"
    src.write_text(r'''
#include <cstdio>
#include <string>
#include <vector>
#include "gpu_bsw/driver.hpp"
#include "gpu_bsw/utils.hpp"
int main() {
    std::vector<std::string> contigs = {"ACGTACGTTTGACCA", "GGGGACGTAC", "TTTT"};
    std::vector<std::string> reads = {"ACGTTTGA", "ACGT", "GGGG"};
    gpu_bsw_driver::alignment_results res;
    short scores[4] = {3, -3, -6, -1};
    gpu_bsw_driver::kernel_driver_dna(reads, contigs, &res, scores, 0.5);
    for (size_t k = 0; k < contigs.size(); ++k)
        std::printf("%d %d %d %d %d\n", res.top_scores[k], res.ref_begin[k], res.ref_end[k],
                    res.query_begin[k], res.query_end[k]);
    free_alignments(&res);
    return 0;
}
''')
    exe = tmp_path / "caller"
    libdir = os.path.dirname(built.lib_path())
    subprocess.check_call(["g++", "-std=c++17", str(src), "-I", os.path.join(REPO, "include"),
                           "-L", libdir, "-lgbsw", "-Wl,-rpath," + libdir,
                           "-o", str(exe)])
    env = dict(os.environ)
    env.pop("GBSW_DEVICES", None)
    if devices:
        env["GBSW_DEVICES"] = devices
        env["GBSW_VERBOSE"] = "1"
    out = subprocess.run([str(exe)], stdout=subprocess.PIPE, text=True, check=True, env=env).stdout
    if devices:  # one phase line per listed device, each with its own range of pairs
        assert sum(ln.startswith("Device 0: pairs") for ln in out.splitlines()) == 3, out
    out = "\n".join(ln for ln in out.splitlines() if ln[:1].isdigit() or ln[:1] == "-")
    got = np.array([[int(x) for x in ln.split()] for ln in out.strip().splitlines()], dtype=np.int32)
    wl = importlib.import_module("gpu-bsw_gb300.workloads")
    b = wl.PairBatch.from_strings(0, ["ACGTACGTTTGACCA", "GGGGACGTAC", "TTTT"], ["ACGTTTGA", "ACGT", "GGGG"])
    _check(got, oracle_batch(b, 0, scores=DNA_BENCH))


def test_scores_beyond_int16(aligner, built, workloads):
    """Identical 11-12 kb DNA strings at +3 and a 7,000-residue protein against
    itself score above 32,767 (oracle-only: the reference keeps shorts).  The
    int32 results equal the oracle's; the int16 form keeps the low 16 bits, as
    the reference's short arrays would."""
    rng = np.random.default_rng(81)
    dna = ["".join(rng.choice(list("ACGT"), n)) for n in (11_000, 12_000)]
    b = workloads.PairBatch.from_strings(0, dna + ["ACGT" * 10], dna + ["ACGA" * 10])
    sc = _scoring(built, 0, DNA_BENCH)
    r32 = aligner.align_batch(b, sc)
    _check(r32, oracle_batch(b, 0, scores=DNA_BENCH))
    assert r32[0, 0] == 33_000 and r32[1, 0] == 36_000
    r16 = aligner.align_batch(b, sc, int16=True)
    np.testing.assert_array_equal(r16, r32.astype(np.int16))
    aa = "".join(rng.choice(list("ARNDCQEGHILKMFPSTWYV"), 7000))
    p = workloads.PairBatch.from_strings(1, [aa, aa[:300]], [aa, aa[100:400]])
    r = aligner.align_batch(p, _scoring(built, 1, AA_GAPS))
    _check(r, oracle_batch(p, 1, gaps=AA_GAPS))
    assert r[0, 0] > 32_767


def test_dropin_pipelined_chunks(built, workloads, tmp_path):
    """A drop-in call of 300,000 pairs runs as three pipeline chunks (the next
    chunk packed and copied in while the current one is aligned, staging from
    the shared pinned pool): its results equal the C ABI's on the same pairs."""
    import json
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import ref_cuda
    b = workloads.custom_dna(300_000, 91, 60, 240, 30, 120, related=0.8)
    exe = ref_cuda.build_ours(built.lib_path())
    pairs = tmp_path / "pairs.tsv"
    ref_cuda.write_pairs(b, str(pairs))
    out = tmp_path / "out.tsv"
    env = dict(os.environ, GBSW_VERBOSE="1", GBSW_DEVICES="0")
    r = subprocess.run([exe, "dna", str(pairs), str(out), "3", "-3", "-6", "-1"], stdout=subprocess.PIPE,
                       stderr=subprocess.PIPE, text=True, env=env, check=True)
    assert "in 2 chunks" in r.stdout or "in 3 chunks" in r.stdout, r.stdout
    got = np.loadtxt(str(out), dtype=np.int32).reshape(-1, 5)
    a = built.Aligner(0)
    exp = a.align_batch(b, _scoring(built, 0, DNA_BENCH), int16=True).astype(np.int32)
    a.close()
    _check(got, exp)
    assert json.loads(r.stderr.strip().splitlines()[-1])["pairs"] == b.n


@pytest.mark.parametrize("lane_group", [0, 128])
def test_maximum_length_pairs(built, workloads, lane_group):
    """Sequences of exactly GBSW_MAX_SEQ_LEN (65,535) symbols: a related query
    inside one (the score passes the int16 range, so a dual plan reruns it in
    int32), an unrelated pair of the same reference, a long pair against a
    short one; through the default plan and block per pair; one more symbol is
    a length error."""
    rng = np.random.default_rng(121)
    big = "".join(rng.choice(list("ACGT"), 65535))
    q = list(big[20000:32000])  # 12,000 symbols: about 35,000 at +3
    for k in rng.integers(0, len(q), 60):
        q[k] = rng.choice(list("ACGT"))
    refs = [big, big, big[:40], "".join(rng.choice(list("ACGT"), 3000))]
    qs = ["".join(q), "".join(rng.choice(list("ACGT"), 2500)), big[:70], big]
    b = workloads.PairBatch.from_strings(0, refs, qs)
    a = built.Aligner(0, lane_group=lane_group)
    sc = _scoring(built, 0, DNA_BENCH)
    got = a.align_batch(b, sc)
    _check(got, oracle_batch(b, 0, scores=DNA_BENCH))
    assert got[0, 0] > 32767
    too_long = workloads.PairBatch.from_strings(0, [big + "A"], ["ACGT"])
    with pytest.raises(built.GbswError) as e:
        a.align_batch(too_long, sc)
    assert e.value.status == -3
    a.close()
