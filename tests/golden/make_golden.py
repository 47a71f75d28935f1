"""Builds the golden fixtures of tests/golden/ from the reference's own kernels.

Three steps (the middle one needs a GPU and the reference binary):

1. ``python tests/golden/make_golden.py inputs DIR``
       writes seeded input sets DIR/<set>.pairs.tsv and DIR/manifest.json.  Every
       pair is checked with the CPU oracle first and pairs whose best score is 0
       are dropped: the reference cannot finish such a pair (its reverse pass
       sizes shared memory from an end of -1, kernel.cpp:426-438).  Every set keeps
       min(longest query, longest reference) <= 1024, the reference's block limit.
2. ``bash oracle/build_ref.sh && python tests/golden/make_golden.py run-ref DIR``
       runs oracle/_ref/ref_harness (the reference's driver and kernels rebuilt for
       sm_103a) on each set, writing DIR/<set>.ref.tsv.
3. ``python tests/golden/make_golden.py collect DIR``
       joins inputs and reference outputs into tests/golden/<set>.tsv.gz.

Fixture format (gzip'd text): '#'-comment header lines ``kind``, ``scores`` (DNA:
match mismatch open extend) or ``gaps`` (protein, BLOSUM62), then one pair per
line: ``ref  query  score  ref_begin  ref_end  query_begin  query_end`` (tab
separated; the reference's raw arrays: ends 1-based, begins 0-based).
"""
import gzip
import importlib
import json
import os
import random
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "oracle"))

import oracle  # noqa: E402

gbsw = importlib.import_module("gpu-bsw_gb300")
workloads = importlib.import_module("gpu-bsw_gb300.workloads")
scoring = gbsw.scoring

DNA_BENCH = (3, -3, -6, -1)
DNA_CLI = (1, -3, -3, -1)


def _repeats(rng, n, lo, hi, alphabet="ACGT"):
    refs, qs = [], []
    for _ in range(n):
        unit = "".join(rng.choice(alphabet) for _ in range(rng.randint(1, 5)))
        r = (unit * (hi // len(unit) + 2))[: rng.randint(lo, hi)]
        start = rng.randint(0, max(0, len(r) - lo // 2))
        q = r[start: start + rng.randint(max(1, lo // 2), hi)]
        q = "".join(c if rng.random() > 0.04 else rng.choice("ACGT") for c in q) or "A"
        if rng.random() < 0.5:
            refs.append(r)
            qs.append(q)
        else:
            refs.append(q)
            qs.append(r)
    return refs, qs


def _random(rng, n, alpha, lo, hi):
    def rs(k):
        return "".join(rng.choice(alpha) for _ in range(k))
    return [rs(rng.randint(lo, hi)) for _ in range(n)], [rs(rng.randint(lo, hi)) for _ in range(n)]


def _batch_strings(b):
    refs, qs = [], []
    for k in range(b.n):
        r, q = b.strings(k)
        refs.append(r.decode())
        qs.append(q.decode())
    return refs, qs


def make_sets():
    """name -> (kind, params, refs, queries)."""
    sets = {}
    sets["dna_plain"] = ("dna", DNA_BENCH) + tuple(_batch_strings(workloads.plain_dna(300, seed=11)))
    sets["dna_throughput"] = ("dna", DNA_BENCH) + tuple(_batch_strings(workloads.dna_throughput(300, seed=12)))
    b = workloads.custom_dna(300, 13, 20, 300, 20, 300, related=0.0)
    sets["dna_unrelated"] = ("dna", DNA_BENCH) + tuple(_batch_strings(b))
    sets["dna_repeats"] = ("dna", DNA_BENCH) + tuple(_repeats(random.Random(14), 300, 30, 400))
    sets["dna_cli_scoring"] = ("dna", DNA_CLI) + tuple(_batch_strings(workloads.plain_dna(300, seed=15)))
    rng = random.Random(16)
    refs, qs = _random(rng, 400, "ACGT", 1, 64)
    sets["dna_roles"] = ("dna", DNA_BENCH, refs, qs)
    refs, qs = _random(random.Random(17), 200, "ACGTNacgtn", 10, 200)
    sets["dna_bytes"] = ("dna", (2, -1, -3, -1), refs, qs)
    refs, qs = _repeats(random.Random(18), 24, 600, 1000, "ACGT")
    sets["dna_long_repeats"] = ("dna", DNA_BENCH, refs, qs)
    pb = workloads.protein(600, seed=19)
    keep = [k for k in range(pb.n) if pb.ref_lengths()[k] <= 400 and pb.query_lengths()[k] <= 400][:200]
    sets["aa_homologs"] = ("aa", (-6, -1)) + tuple(_batch_strings(pb.subset(keep)))
    refs, qs = _random(random.Random(20), 300, "ARNDCQEGHILKMFPSTWYVBZX*JOU", 5, 80)
    sets["aa_short"] = ("aa", (-6, -1), refs, qs)
    refs, qs = _random(random.Random(21), 200, "ARNDCQEGHILKMFPSTWYV", 5, 300)
    sets["aa_gaps_11_1"] = ("aa", (-11, -1), refs, qs)
    return sets


def oracle_results(kind, params, refs, qs):
    if kind == "dna":
        return oracle.align_strings(oracle.DNA, refs, qs, scores=params)
    return oracle.align_strings(oracle.AA, refs, qs, matrix=scoring.BLOSUM62,
                                encoding=scoring.ENCODING, gaps=params)


def cmd_inputs(d):
    os.makedirs(d, exist_ok=True)
    manifest = {}
    for name, (kind, params, refs, qs) in make_sets().items():
        res = oracle_results(kind, params, refs, qs)
        keep = [k for k in range(len(refs)) if res[k, 0] > 0]
        refs = [refs[k] for k in keep]
        qs = [qs[k] for k in keep]
        assert len(refs) >= 2
        assert min(max(map(len, refs)), max(map(len, qs))) <= 1024
        with open(os.path.join(d, name + ".pairs.tsv"), "w") as f:
            for r, q in zip(refs, qs):
                f.write("%s\t%s\n" % (r, q))
        manifest[name] = {"kind": kind, "params": list(params), "pairs": len(refs)}
    with open(os.path.join(d, "blosum62.txt"), "w") as f:
        f.write(" ".join(str(v) for v in scoring.BLOSUM62) + "\n")
    with open(os.path.join(d, "manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1)
    print(json.dumps(manifest))


def cmd_run_ref(d):
    exe = os.path.join(REPO, "oracle", "_ref", "ref_harness")
    manifest = json.load(open(os.path.join(d, "manifest.json")))
    for name, m in manifest.items():
        src = os.path.join(d, name + ".pairs.tsv")
        dst = os.path.join(d, name + ".ref.tsv")
        if m["kind"] == "dna":
            args = [exe, "dna", src, dst] + [str(v) for v in m["params"]]
        else:
            args = [exe, "aa", src, dst, os.path.join(d, "blosum62.txt")] + [str(v) for v in m["params"]]
        r = subprocess.run(args, stdout=subprocess.DEVNULL, stderr=subprocess.PIPE, text=True)
        if r.returncode != 0:
            raise SystemExit("reference failed on %s: %s" % (name, r.stderr))
        print(name, r.stderr.strip().splitlines()[-1])


def cmd_collect(d):
    manifest = json.load(open(os.path.join(d, "manifest.json")))
    for name, m in manifest.items():
        pairs = [ln.rstrip("\n").split("\t") for ln in open(os.path.join(d, name + ".pairs.tsv"))]
        outs = [ln.split() for ln in open(os.path.join(d, name + ".ref.tsv"))]
        assert len(pairs) == len(outs) == m["pairs"], name
        with gzip.open(os.path.join(HERE, name + ".tsv.gz"), "wt", compresslevel=9) as f:
            f.write("# set: %s\n# kind: %s\n" % (name, m["kind"]))
            key = "scores" if m["kind"] == "dna" else "gaps"
            f.write("# %s: %s\n" % (key, " ".join(str(v) for v in m["params"])))
            for (r, q), o in zip(pairs, outs):
                f.write("\t".join([r, q] + o) + "\n")
        print("wrote", name)


def load_fixture(path):
    """-> (kind, params, refs, queries, expected (n,5) int32)."""
    kind, params = None, None
    refs, qs, exp = [], [], []
    with gzip.open(path, "rt") as f:
        for ln in f:
            if ln.startswith("#"):
                k, _, v = ln[1:].partition(":")
                k = k.strip()
                if k == "kind":
                    kind = v.strip()
                elif k in ("scores", "gaps"):
                    params = tuple(int(x) for x in v.split())
                continue
            parts = ln.rstrip("\n").split("\t")
            refs.append(parts[0])
            qs.append(parts[1])
            exp.append([int(x) for x in parts[2:7]])
    return kind, params, refs, qs, np.array(exp, dtype=np.int32).reshape(-1, 5)


if __name__ == "__main__":
    cmd, d = sys.argv[1], sys.argv[2]
    {"inputs": cmd_inputs, "run-ref": cmd_run_ref, "collect": cmd_collect}[cmd](d)
