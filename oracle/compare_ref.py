"""Times the reference's own CUDA kernels and this library on the same GPU and
workloads, and diffs their results pair by pair.

TEST INFRASTRUCTURE ONLY.  Needs the reference harness built first
(``bash oracle/build_ref.sh``, from the reference's sources) and a GPU:

    python oracle/compare_ref.py [--reps 3] [--out results.jsonl]

For each workload it writes the pairs to a TSV file and runs
``oracle/_ref/ref_harness`` (the reference's ``kernel_driver_dna`` /
``kernel_driver_aa``, fastest of ``--reps`` calls after CUDA context creation).
It runs the same harness source built against this library's source-compatible
``gpu_bsw/driver.hpp`` (``oracle/_ref/ours_harness``: identical scope, from
``std::vector<std::string>`` in to the pinned result arrays out), then
``gbsw_align_host16`` on packed host buffers and the device-resident passes.  It
prints one JSON line per workload with the timings and the number of pairs whose
five results differ from the reference's.

Every workload stays inside the reference's limits: at least two pairs,
min(longest query, longest reference) <= 1024, and no pair without a shared
symbol (such a pair scores 0 and the reference's reverse pass then writes
shared memory with a length of (unsigned)-1, kernel.cpp:429-438).
"""
import argparse
import importlib
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
sys.path.insert(0, REPO)

gbsw = importlib.import_module("gpu-bsw_gb300")
wl = importlib.import_module("gpu-bsw_gb300.workloads")

WORKLOADS = [
    ("plain_dna_1k", lambda: wl.plain_dna(1000, 1), "dna"),
    ("dna_throughput_100k", lambda: wl.dna_throughput(100_000, 2), "dna"),
    ("protein_30k", lambda: wl.protein(30_000, 3), "aa"),
    ("mixed_dna_short_bin_140k", lambda: wl.mixed_dna_short(140_000, 4), "dna"),
]


def reference_safe(batch):
    for k in range(batch.n):
        r, q = batch.strings(k)
        if not set(r) & set(q):
            return False
    return min(batch.ref_lengths().max(), batch.query_lengths().max()) <= 1024 and batch.n >= 2


def build_ours_harness():
    """ref_harness.cpp compiled against include/gpu_bsw and libgbsw.so."""
    exe = os.path.join(HERE, "_ref", "ours_harness")
    src = os.path.join(HERE, "ref_harness.cpp")
    lib = gbsw.lib_path()
    if os.path.exists(exe) and os.path.getmtime(exe) > max(os.path.getmtime(src), os.path.getmtime(lib)):
        return exe
    libdir = os.path.dirname(lib)
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-I" + os.path.join(REPO, "include", "gpu_bsw"),
                           "-I" + os.path.join(cuda, "include"), src, "-o", exe, "-L" + libdir, "-lgbsw",
                           "-Wl,-rpath," + libdir, "-L" + os.path.join(cuda, "lib64"), "-lcudart"])
    return exe


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--out", default=None)
    args = ap.parse_args()
    exe = os.path.join(HERE, "_ref", "ref_harness")
    if not os.path.exists(exe):
        raise SystemExit("build the reference harness first: bash oracle/build_ref.sh")
    ours = build_ours_harness()
    tmp = tempfile.mkdtemp()
    mat = os.path.join(tmp, "blosum62.txt")
    with open(mat, "w") as f:
        f.write(" ".join(map(str, gbsw.scoring.BLOSUM62)))
    al = gbsw.Aligner(0)
    lines = []
    for name, make, kind in WORKLOADS:
        b = make()
        assert reference_safe(b), name
        tsv = os.path.join(tmp, name + ".tsv")
        with open(tsv, "w") as f:
            for k in range(b.n):
                r, q = b.strings(k)
                f.write(r.decode() + "\t" + q.decode() + "\n")
        out = os.path.join(tmp, name + ".ref.tsv")
        env = dict(os.environ, GBSW_REF_REPS=str(args.reps))
        if kind == "dna":
            cmd = [exe, "dna", tsv, out, "3", "-3", "-6", "-1"]
            sc = gbsw.make_scoring(gbsw.DNA, scores=(3, -3, -6, -1))
        else:
            cmd = [exe, "aa", tsv, out, mat, "-6", "-1"]
            sc = gbsw.make_scoring(gbsw.PROTEIN, matrix=gbsw.scoring.BLOSUM62, gaps=(-6, -1))
        r = subprocess.run(cmd, stdout=subprocess.DEVNULL, stderr=subprocess.PIPE, text=True, env=env)
        if r.returncode != 0:
            raise SystemExit("reference failed on %s: %s" % (name, r.stderr[-2000:]))
        ref_s = json.loads(r.stderr.strip().splitlines()[-1])["seconds"]
        ref_res = np.loadtxt(out, dtype=np.int32).reshape(-1, 5)
        ours_out = out + ".ours"
        r = subprocess.run([ours] + cmd[1:3] + [ours_out] + cmd[4:], stdout=subprocess.DEVNULL,
                           stderr=subprocess.PIPE, text=True, env=env)
        if r.returncode != 0:
            raise SystemExit("drop-in harness failed on %s: %s" % (name, r.stderr[-2000:]))
        dropin_s = json.loads(r.stderr.strip().splitlines()[-1])["seconds"]
        dropin_bad = int(np.count_nonzero(np.any(np.loadtxt(ours_out, dtype=np.int32).reshape(-1, 5) != ref_res,
                                                 axis=1)))
        best, kern = 1e30, 1e30
        got = None
        for _ in range(args.reps + 1):
            t = time.perf_counter()
            got = al.align_batch(b, sc, int16=True).astype(np.int32)
            best = min(best, time.perf_counter() - t)
            st = al.stats()
            kern = min(kern, (st["forward_ms"] + st["reverse_ms"]) / 1e3)
        bad = int(np.count_nonzero(np.any(got != ref_res, axis=1)))
        cells = b.cells()
        line = {"workload": name, "pairs": b.n, "cells": cells,
                "reference_s": ref_s, "reference_gcups": round(cells / ref_s / 1e9, 2),
                "ours_dropin_s": round(dropin_s, 6), "ours_dropin_gcups": round(cells / dropin_s / 1e9, 2),
                "speedup_dropin_vs_reference": round(ref_s / dropin_s, 2),
                "dropin_pairs_differing_from_reference": dropin_bad,
                "ours_host_s": round(best, 6), "ours_host_gcups": round(cells / best / 1e9, 2),
                "ours_passes_gcups": round(cells / kern / 1e9, 2),
                "speedup_host_vs_reference": round(ref_s / best, 2),
                "pairs_differing_from_reference": bad}
        print(json.dumps(line), flush=True)
        lines.append(line)
    al.close()
    if args.out:
        with open(args.out, "w") as f:
            for ln in lines:
                f.write(json.dumps(ln) + "\n")


if __name__ == "__main__":
    main()
