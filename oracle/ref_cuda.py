"""Runs the reference's own CUDA build (oracle/_ref/ref_harness, from
oracle/build_ref.sh) and the same harness built against this library's
source-compatible ``gpu_bsw/driver.hpp`` on one batch of pairs.

TEST INFRASTRUCTURE ONLY: the reference side of the GPU-vs-reference timing
(``bench.py``'s reference legs, ``oracle/compare_ref.py``) and of the golden
fixtures.  The product never imports it.

Inputs must stay inside the reference's limits (``reference_safe``): at least
two pairs, min(longest query, longest reference) <= 1024, and every pair shares
a symbol (a pair scoring 0 makes the reference's reverse pass write shared
memory with a length of (unsigned)-1, kernel.cpp:429-438).
"""
import json
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
HARNESS = os.path.join(HERE, "_ref", "ref_harness")
OURS_HARNESS = os.path.join(HERE, "_ref", "ours_harness")
SRC = os.path.join(HERE, "ref_harness.cpp")


def build():
    """Builds the reference harness from the reference's sources; False when they are absent."""
    r = subprocess.run(["bash", os.path.join(HERE, "build_ref.sh")], stdout=subprocess.DEVNULL,
                       stderr=subprocess.PIPE, text=True)
    if r.returncode == 3:
        return False
    if r.returncode != 0:
        raise RuntimeError("build_ref.sh failed: " + r.stderr[-2000:])
    return os.path.exists(HARNESS)


def build_ours(lib_path):
    """ref_harness.cpp compiled against include/gpu_bsw and libgbsw.so (the drop-in)."""
    if os.path.exists(OURS_HARNESS) and os.path.getmtime(OURS_HARNESS) > max(os.path.getmtime(SRC),
                                                                            os.path.getmtime(lib_path)):
        return OURS_HARNESS
    os.makedirs(os.path.dirname(OURS_HARNESS), exist_ok=True)
    libdir = os.path.dirname(lib_path)
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-I" + os.path.join(REPO, "include", "gpu_bsw"),
                           "-I" + os.path.join(cuda, "include"), SRC, "-o", OURS_HARNESS, "-L" + libdir, "-lgbsw",
                           "-Wl,-rpath," + libdir, "-L" + os.path.join(cuda, "lib64"), "-lcudart"])
    return OURS_HARNESS


def reference_safe(batch):
    """True when every pair shares a symbol and the batch fits the reference's block size."""
    rl, ql = batch.ref_lengths(), batch.query_lengths()
    if batch.n < 2 or min(int(rl.max()), int(ql.max())) > 1024:
        return False
    for k in range(batch.n):
        r, q = batch.strings(k)
        if not set(r) & set(q):
            return False
    return True


def write_pairs(batch, path):
    """One pair per line, reference TAB query."""
    with open(path, "wb") as f:
        rb, ro, qb, qo = batch.ref.tobytes(), batch.ref_off, batch.query.tobytes(), batch.query_off
        f.write(b"".join(rb[ro[k]:ro[k + 1]] + b"\t" + qb[qo[k]:qo[k + 1]] + b"\n" for k in range(batch.n)))


def _run(exe, batch, kind, reps, scores, matrix, gaps, tmp):
    pairs = os.path.join(tmp, "pairs.tsv")
    if not os.path.exists(pairs):
        write_pairs(batch, pairs)
    out = os.path.join(tmp, os.path.basename(exe) + ".out.tsv")
    if kind == "dna":
        cmd = [exe, "dna", pairs, out] + [str(v) for v in scores]
    else:
        mat = os.path.join(tmp, "matrix.txt")
        with open(mat, "w") as f:
            f.write(" ".join(str(int(v)) for v in matrix))
        cmd = [exe, "aa", pairs, out, mat, str(gaps[0]), str(gaps[1])]
    r = subprocess.run(cmd, stdout=subprocess.DEVNULL, stderr=subprocess.PIPE, text=True,
                       env=dict(os.environ, GBSW_REF_REPS=str(reps)))
    if r.returncode != 0:
        raise RuntimeError("%s failed: %s" % (os.path.basename(exe), r.stderr[-2000:]))
    info = json.loads(r.stderr.strip().splitlines()[-1])
    info["results"] = np.loadtxt(out, dtype=np.int32, ndmin=2).reshape(-1, 5)
    return info


def run_pair(batch, kind, reps=3, scores=(3, -3, -6, -1), matrix=None, gaps=(-6, -1), lib_path=None):
    """The reference's driver and (with lib_path) the drop-in built from the same
    harness source, on the same pairs file.  Returns {"reference": info, "dropin":
    info or None}; each info holds seconds, kernel_seconds and results (n x 5:
    score, ref_begin, ref_end, query_begin, query_end)."""
    with tempfile.TemporaryDirectory() as tmp:
        ref = _run(HARNESS, batch, kind, reps, scores, matrix, gaps, tmp)
        ours = None
        if lib_path:
            ours = _run(build_ours(lib_path), batch, kind, reps, scores, matrix, gaps, tmp)
    return {"reference": ref, "dropin": ours}
