"""Times the reference's own CUDA kernels and this library on the same GPU and
workloads, and diffs their results pair by pair.

TEST INFRASTRUCTURE ONLY.  Needs the reference harness built first
(``bash oracle/build_ref.sh``, from the reference's sources) and a GPU:

    python oracle/compare_ref.py [--reps 3] [--out results.jsonl]

For each workload ``oracle/ref_cuda.py`` runs ``oracle/_ref/ref_harness`` (the
reference's ``kernel_driver_dna`` / ``kernel_driver_aa``, fastest of ``--reps``
calls after CUDA context creation, with the kernel time of its own launches) and
the same harness source built against this library's source-compatible
``gpu_bsw/driver.hpp`` (identical scope, from ``std::vector<std::string>`` in to
the pinned result arrays out).  Then ``gbsw_align_host16`` on packed host
buffers and the device-resident passes.  It prints one JSON line per workload
with the timings and the number of pairs whose five results differ from the
reference's.  Every workload stays inside the reference's limits
(``ref_cuda.reference_safe``).
"""
import argparse
import importlib
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
sys.path.insert(0, REPO)
sys.path.insert(0, HERE)

import ref_cuda  # noqa: E402

gbsw = importlib.import_module("gpu-bsw_gb300")
wl = importlib.import_module("gpu-bsw_gb300.workloads")

WORKLOADS = [
    ("plain_dna_1k", lambda: wl.plain_dna(1000, 1), "dna"),
    ("dna_throughput_100k", lambda: wl.dna_throughput(100_000, 2), "dna"),
    ("protein_30k", lambda: wl.protein(30_000, 3), "aa"),
    ("mixed_dna_short_bin_140k", lambda: wl.mixed_dna_short(140_000, 4), "dna"),
]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--out", default=None)
    args = ap.parse_args()
    if not os.path.exists(ref_cuda.HARNESS):
        raise SystemExit("build the reference harness first: bash oracle/build_ref.sh")
    al = gbsw.Aligner(0)
    lines = []
    for name, make, kind in WORKLOADS:
        b = make()
        assert ref_cuda.reference_safe(b), name
        if kind == "dna":
            sc = gbsw.make_scoring(gbsw.DNA, scores=(3, -3, -6, -1))
        else:
            sc = gbsw.make_scoring(gbsw.PROTEIN, matrix=gbsw.scoring.BLOSUM62, gaps=(-6, -1))
        runs = ref_cuda.run_pair(b, kind, reps=args.reps, matrix=gbsw.scoring.BLOSUM62, lib_path=gbsw.lib_path())
        ref, dropin = runs["reference"], runs["dropin"]
        ref_res = ref["results"]
        best, kern = 1e30, 1e30
        got = None
        for _ in range(args.reps + 1):
            t = time.perf_counter()
            got = al.align_batch(b, sc, int16=True).astype(np.int32)
            best = min(best, time.perf_counter() - t)
            st = al.stats()
            kern = min(kern, (st["forward_ms"] + st["reverse_ms"]) / 1e3)
        bad = int(np.count_nonzero(np.any(got != ref_res, axis=1)))
        dropin_bad = int(np.count_nonzero(np.any(dropin["results"] != ref_res, axis=1)))
        cells = b.cells()
        line = {"workload": name, "pairs": b.n, "cells": cells,
                "reference_s": ref["seconds"], "reference_gcups": round(cells / ref["seconds"] / 1e9, 2),
                "reference_kernel_s": ref["kernel_seconds"], "reference_launches": ref["launches"],
                "reference_kernel_gcups": round(cells / ref["kernel_seconds"] / 1e9, 2),
                "ours_dropin_s": round(dropin["seconds"], 6),
                "ours_dropin_gcups": round(cells / dropin["seconds"] / 1e9, 2),
                "speedup_dropin_vs_reference": round(ref["seconds"] / dropin["seconds"], 2),
                "dropin_pairs_differing_from_reference": dropin_bad,
                "ours_host_s": round(best, 6), "ours_host_gcups": round(cells / best / 1e9, 2),
                "ours_passes_s": round(kern, 6), "ours_passes_gcups": round(cells / kern / 1e9, 2),
                "speedup_host_vs_reference": round(ref["seconds"] / best, 2),
                "speedup_passes_vs_reference_kernels": round(ref["kernel_seconds"] / kern, 2),
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
