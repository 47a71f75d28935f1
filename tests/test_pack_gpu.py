"""GPU tests of the packed input path: the device unpack against the raw bytes,
and the packed host entry bit-exact against the reference's outputs (golden
fixtures, including the escape-heavy ``dna_bytes`` batch) and against the raw
host entry on full-size batches."""
import importlib
import os
import sys

import numpy as np
import pytest

from helpers import GOLDEN, first_mismatches, oracle_batch
from test_pack import unpack_np

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
import make_golden  # noqa: E402

pytestmark = pytest.mark.gpu

DNA_BENCH = (3, -3, -6, -1)
AA_GAPS = (-6, -1)


def _scoring(gbsw, kind, params):
    if kind in ("dna", 0):
        return gbsw.make_scoring(gbsw.DNA, scores=params)
    return gbsw.make_scoring(gbsw.PROTEIN, matrix=gbsw.scoring.BLOSUM62, gaps=params)


def _packed(gbsw, batch, kind):
    return gbsw.pack(kind, batch.ref), gbsw.pack(kind, batch.query)


@pytest.mark.skipif(not GOLDEN, reason="golden fixtures not generated")
@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
def test_reference_outputs_through_packed_entry(aligner, built, path):
    kind, params, refs, qs, exp = make_golden.load_fixture(path)
    k = 0 if kind in ("dna", 0) else 1
    wl = importlib.import_module("gpu-bsw_gb300.workloads")
    batch = wl.PairBatch.from_strings(k, refs, qs)
    pr, pq = _packed(built, batch, k)
    if os.path.basename(path).startswith("dna_bytes"):
        assert pr.nruns + pq.nruns > 0  # the fixture's N and lower-case bytes travel as escapes
    got = aligner.align_packed(_scoring(built, kind, params), pr, batch.ref_off, pq, batch.query_off)
    bad, count = first_mismatches(got, exp)
    assert count == 0, (count, bad)


@pytest.mark.parametrize("kind", [0, 1])
@pytest.mark.parametrize("offset", [0, 1, 5])
def test_unpack_device_matches_raw(built, kind, offset):
    torch = pytest.importorskip("torch")
    import ctypes
    rng = np.random.default_rng(10 + kind + offset)
    n = 100_003
    alpha = np.frombuffer(b"ACGT" if kind == 0 else b"ARNDCQEGHILKMFPSTWYVBZX", np.uint8)
    raw = rng.choice(alpha, n)
    hit = rng.random(n) < 0.003
    raw[hit] = rng.choice(np.frombuffer(b"Nnx*-", np.uint8), int(hit.sum()))
    raw[:3] = ord("n")          # a run at the start
    raw[-2:] = ord("-")         # and at the end
    p = built.pack(kind, raw)
    dev = torch.device("cuda", 0)
    words = torch.from_numpy(p.words.view(np.int32)).to(dev)
    at = torch.from_numpy(p.run_at).to(dev)
    off = torch.from_numpy(p.run_off).to(dev)
    by = torch.from_numpy(p.run_bytes).to(dev)
    out = torch.full((n + 32,), 7, dtype=torch.uint8, device=dev)
    dp = built._Packed()
    dp.words, dp.nsym, dp.nruns = words.data_ptr(), n, p.nruns
    dp.run_at, dp.run_off, dp.run_bytes = at.data_ptr(), off.data_ptr(), by.data_ptr()
    s = torch.cuda.current_stream(dev)
    rc = built.load().gbsw_unpack_device(kind, ctypes.byref(dp), out.data_ptr() + offset, s.cuda_stream)
    assert rc == 0
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    assert np.array_equal(got[offset:offset + n], raw)
    assert (got[:offset] == 7).all() and (got[offset + n:] == 7).all()  # nothing written outside
    assert np.array_equal(unpack_np(p), raw)


def test_packed_entry_full_size_dna(aligner, built, workloads):
    """100,000 DNA throughput pairs: packed entry == raw entry on every pair, in
    the int16 result form of the reference's arrays."""
    b = workloads.dna_throughput(100_000, seed=1)
    sc = _scoring(built, 0, DNA_BENCH)
    pr, pq = _packed(built, b, 0)
    assert pr.nbytes + pq.nbytes <= (b.ref.size + b.query.size) // 4 + 8
    raw = aligner.align_batch(b, sc, int16=True).copy()
    got = aligner.align_packed(sc, pr, b.ref_off, pq, b.query_off, int16=True)
    assert np.array_equal(got, raw)


def test_packed_entry_protein_and_mixed(aligner, built, workloads):
    b = workloads.protein(20_000, seed=4)
    sc = _scoring(built, 1, AA_GAPS)
    pr, pq = _packed(built, b, 1)
    got = aligner.align_packed(sc, pr, b.ref_off, pq, b.query_off)
    assert np.array_equal(got, aligner.align_batch(b, sc))
    sub = b.subset(np.arange(0, 20_000, 40))
    bad, count = first_mismatches(got[::40], oracle_batch(sub, 1, gaps=AA_GAPS))
    assert count == 0, bad
    m = workloads.mixed_dna(20_000, seed=5)
    sc = _scoring(built, 0, DNA_BENCH)
    pr, pq = _packed(built, m, 0)
    assert np.array_equal(aligner.align_packed(sc, pr, m.ref_off, pq, m.query_off), aligner.align_batch(m, sc))


def test_packed_entry_errors(aligner, built, workloads):
    b = workloads.plain_dna(50, seed=6)
    sc = _scoring(built, 0, DNA_BENCH)
    pr, pq = _packed(built, b, 0)
    short = built.PackedStream(0, pr.words, pr.nsym - 1, pr.run_at, pr.run_off, pr.run_bytes)
    with pytest.raises(built.GbswError) as ei:
        aligner.align_packed(sc, short, b.ref_off, pq, b.query_off)
    assert ei.value.status == -1
    bad_runs = built.PackedStream(0, pr.words, pr.nsym, np.array([4, 2], np.int64), np.array([0, 3, 4], np.int64),
                                  np.frombuffer(b"NNNN", np.uint8).copy())
    with pytest.raises(built.GbswError) as ei:
        aligner.align_packed(sc, bad_runs, b.ref_off, pq, b.query_off)
    assert ei.value.status == -1
    # offsets that decrease: found while the copies run, reported all the same,
    # and the context stays usable
    dec = b.ref_off.copy()
    dec[10], dec[11] = dec[11], dec[10]
    with pytest.raises(built.GbswError) as ei:
        aligner.align_packed(sc, pr, dec, pq, b.query_off)
    assert ei.value.status == -1
    np.testing.assert_array_equal(aligner.align_packed(sc, pr, b.ref_off, pq, b.query_off),
                                  aligner.align_batch(b, sc))
    # a protein byte outside the encoding table travels as an escape and is
    # reported by the passes, as with raw input
    wl = importlib.import_module("gpu-bsw_gb300.workloads")
    pb = wl.PairBatch.from_strings(1, ["ARNDz", "ARND"], ["ARN", "RND"])
    pr, pq = _packed(built, pb, 1)
    assert pr.nruns == 1
    with pytest.raises(built.GbswError) as ei:
        aligner.align_packed(_scoring(built, 1, AA_GAPS), pr, pb.ref_off, pq, pb.query_off)
    assert ei.value.status == -2
    # an empty call
    e = built.pack(0, np.zeros(0, np.uint8))
    assert aligner.align_packed(sc, e, np.zeros(1, np.int64), e, np.zeros(1, np.int64)).shape == (0, 5)


@pytest.mark.parametrize("kind", [0, 1])
def test_dropin_packed_ingest(built, workloads, tmp_path, kind):
    """The C++ drop-in packs its staging (2-bit / 5-bit words, escape runs for
    other bytes) and unpacks on the device; its results equal the raw-copy
    ingest (GBSW_DROPIN_PACK=0) and the C ABI on pairs with escaped bytes."""
    import json
    import subprocess
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(__file__)), "oracle"))
    import ref_cuda
    rng = np.random.default_rng(90 + kind)
    if kind == 0:
        b = workloads.dna_throughput(30_000, seed=91)
        esc = np.frombuffer(b"Nnacgt", np.uint8)
    else:
        b = workloads.protein(20_000, seed=92)
        esc = np.frombuffer(b"*", np.uint8)
    for buf in (b.ref, b.query):
        hit = rng.random(buf.size) < 0.001
        buf[hit] = rng.choice(esc, int(hit.sum()))
    exe = ref_cuda.build_ours(built.lib_path())
    pairs = tmp_path / "pairs.tsv"
    ref_cuda.write_pairs(b, str(pairs))
    sc = _scoring(built, kind, DNA_BENCH if kind == 0 else AA_GAPS)
    outs = {}
    for mode in ("1", "0"):
        out = tmp_path / ("out%s.tsv" % mode)
        if kind == 0:
            cmd = [exe, "dna", str(pairs), str(out), "3", "-3", "-6", "-1"]
        else:
            mat = tmp_path / "matrix.txt"
            mat.write_text(" ".join(str(int(v)) for v in built.scoring.BLOSUM62))
            cmd = [exe, "aa", str(pairs), str(out), str(mat), "-6", "-1"]
        env = dict(os.environ, GBSW_DROPIN_PACK=mode, GBSW_DEVICES="0")
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, env=env, check=True)
        assert json.loads(r.stderr.strip().splitlines()[-1])["pairs"] == b.n
        outs[mode] = np.loadtxt(str(out), dtype=np.int32).reshape(-1, 5)
    a = built.Aligner(0)
    exp = a.align_batch(b, sc, int16=True).astype(np.int32)
    a.close()
    np.testing.assert_array_equal(outs["1"], exp)
    np.testing.assert_array_equal(outs["0"], exp)
