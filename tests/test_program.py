"""program_gpu, the command-line front end with the reference program's I/O
conventions (main.cpp:13-248 of ADEPT / GPU-BSW): one sequence per non-'>' line,
five tab-separated columns per pair with 0-based inclusive ends, "Total Cells:N"
on stdout.

CPU tests cover the argument handling, which exits before any GPU work.  GPU
tests replay the golden fixtures whose scoring is the reference program's
(DNA {1,-3,-3,-1}; protein BLOSUM62 -6/-1) and compare with the reference's own
outputs, bit for bit, and check the other conventions against the oracle."""
import importlib
import os
import subprocess
import sys

import numpy as np
import pytest

from helpers import GOLDEN, oracle_batch

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
import make_golden  # noqa: E402


def _program(built):
    build = importlib.import_module("gpu-bsw_gb300.build")
    build.build_all()
    return build.PROGRAM


def _write_fasta(path, seqs, header=True):
    with open(path, "w") as f:
        for k, s in enumerate(seqs):
            if header:
                f.write(">seq%d\n" % k)
            f.write(s + "\n")


def _run(prog, *args):
    return subprocess.run([prog] + [str(a) for a in args], stdout=subprocess.PIPE, stderr=subprocess.PIPE,
                          text=True, timeout=600)


def _read_tsv(path):
    rows = [ln.split("\t") for ln in open(path).read().splitlines()]
    return np.array([[int(x) for x in r] for r in rows], dtype=np.int32).reshape(-1, 5)


def _as_program_columns(res):
    """(n, 5) library results -> the program's columns (ends minus one)."""
    out = res.copy()
    out[:, 2] -= 1
    out[:, 4] -= 1
    return out


def test_argument_errors_without_gpu(built, tmp_path):
    prog = _program(built)
    assert _run(prog).returncode == 2
    assert _run(prog, "rna", "a", "b", "c").returncode == 2
    ref, qry = tmp_path / "r.fa", tmp_path / "q.fa"
    _write_fasta(ref, ["ACGT", "ACGT"])
    _write_fasta(qry, ["ACGT"])
    r = _run(prog, "dna", ref, qry, tmp_path / "o.tsv")
    assert r.returncode == 2 and "2 reference sequences but 1 query" in r.stderr
    assert _run(prog, "dna", ref, tmp_path / "missing.fa", tmp_path / "o.tsv").returncode == 2
    assert _run(prog, "dna", ref, ref, tmp_path / "o.tsv", "--scores", "1,2").returncode == 2
    assert _run(prog, "dna", ref, ref, tmp_path / "o.tsv", "--frobnicate").returncode == 2


@pytest.mark.gpu
@pytest.mark.skipif(not GOLDEN, reason="golden fixtures not generated")
def test_reference_program_fixtures(built, tmp_path):
    """The fixtures made with the reference program's scoring, replayed through
    program_gpu: identical to the reference's results."""
    prog = _program(built)
    replayed = 0
    for path in GOLDEN:
        kind, params, refs, qs, exp = make_golden.load_fixture(path)
        if kind == "dna" and params == (1, -3, -3, -1):
            mode = "dna"
        elif kind != "dna" and params == (-6, -1):
            mode = "aa"
        else:
            continue
        name = os.path.basename(path).split(".")[0]
        ref, qry, out = tmp_path / (name + ".ref.fa"), tmp_path / (name + ".qry.fa"), tmp_path / (name + ".tsv")
        _write_fasta(ref, refs)
        _write_fasta(qry, qs)
        r = _run(prog, mode, ref, qry, out)
        assert r.returncode == 0, r.stderr
        cells = sum(len(a) * len(b) for a, b in zip(refs, qs))
        assert r.stdout.strip().splitlines()[-1] == "Total Cells:%d" % cells
        np.testing.assert_array_equal(_read_tsv(out), _as_program_columns(exp), err_msg=name)
        replayed += 1
    assert replayed >= 2


@pytest.mark.gpu
def test_program_conventions_against_oracle(built, workloads, tmp_path):
    """Options, FASTA without headers, empty lines (empty sequences), pairs with no
    positive score (printed as 0 -1 -2 -1 -2) and a batch larger than one chunk."""
    prog = _program(built)
    b = workloads.PairBatch.concat([workloads.plain_dna(3000, seed=71),
                                    workloads.PairBatch.from_strings(0, ["", "AAAA", "ACGT"], ["ACGT", "CCCC", ""])])
    refs = [b.strings(k)[0].decode() for k in range(b.n)]
    qs = [b.strings(k)[1].decode() for k in range(b.n)]
    ref, qry, out = tmp_path / "r.fa", tmp_path / "q.fa", tmp_path / "o.tsv"
    _write_fasta(ref, refs, header=False)
    _write_fasta(qry, qs, header=True)
    r = _run(prog, "dna", ref, qry, out, "--scores", "3,-3,-6,-1", "--factor", "0.25")
    assert r.returncode == 0, r.stderr
    got = _read_tsv(out)
    exp = _as_program_columns(oracle_batch(b, 0, scores=(3, -3, -6, -1)))
    np.testing.assert_array_equal(got, exp)
    assert got[-3:].tolist() == [[0, -1, -2, -1, -2]] * 3
    # protein with other gaps
    p = workloads.protein(500, seed=72)
    _write_fasta(ref, [p.strings(k)[0].decode() for k in range(p.n)])
    _write_fasta(qry, [p.strings(k)[1].decode() for k in range(p.n)])
    r = _run(prog, "aa", ref, qry, out, "--gaps", "-11,-1")
    assert r.returncode == 0, r.stderr
    np.testing.assert_array_equal(_read_tsv(out), _as_program_columns(oracle_batch(p, 1, gaps=(-11, -1))))
