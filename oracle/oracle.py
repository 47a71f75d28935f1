"""ctypes wrapper of the CPU oracle (oracle/gotoh.c, oracle/traceback.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()`` and by
``bench.py``'s CPU-baseline leg, as the oracle and the CPU baseline.  The product library
never imports it.

``align(kind, A, offA, B, offB, ...)`` returns an ``(n, 5)`` int32 array with
columns ``score, ref_begin, ref_end, query_begin, query_end`` in the reference's
conventions (ends 1-based inclusive, begins 0-based; A = reference/contig,
B = query/read).  ``traceback(...)`` returns each aligned pair's path as
run-length operations (see oracle/traceback.c).
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "gotoh.c")
SOURCES = [SRC, os.path.join(HERE, "traceback.c")]
LIB = os.path.join(HERE, "liboracle.so")

DNA = 0
AA = 1


class _Scoring(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int),
        ("match", ctypes.c_int),
        ("mismatch", ctypes.c_int),
        ("open", ctypes.c_int),
        ("extend", ctypes.c_int),
        ("matrix", ctypes.POINTER(ctypes.c_int16)),
        ("encoding", ctypes.POINTER(ctypes.c_int16)),
    ]


def build(force=False):
    """Compile the oracle sources into liboracle.so with gcc (OpenMP, -O2, portable flags)."""
    if not force and os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(s) for s in SOURCES):
        return LIB
    tmp = LIB + ".tmp"
    subprocess.check_call(["gcc", "-O2", "-fopenmp", "-shared", "-fPIC", "-o", tmp] + SOURCES)
    os.replace(tmp, LIB)
    return LIB


_lib = None


def load():
    global _lib
    if _lib is None:
        build()
        lib = ctypes.CDLL(LIB)
        lib.oracle_align_batch.restype = ctypes.c_int
        lib.oracle_align_batch.argtypes = [
            ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
            ctypes.c_int64, ctypes.POINTER(_Scoring), ctypes.c_void_p, ctypes.c_void_p,
            ctypes.c_int,
        ]
        lib.oracle_threads.restype = ctypes.c_int
        lib.oracle_traceback_batch.restype = ctypes.c_int
        lib.oracle_traceback_batch.argtypes = [
            ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
            ctypes.POINTER(_Scoring), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
            ctypes.c_void_p, ctypes.c_int,
        ]
        _lib = lib
    return _lib


def threads():
    return load().oracle_threads()


def _as_u8(x):
    if isinstance(x, (bytes, bytearray)):
        return np.frombuffer(bytes(x), dtype=np.uint8)
    return np.ascontiguousarray(x, dtype=np.uint8)


def align(kind, A, offA, B, offB, scores=None, matrix=None, encoding=None, gaps=None,
          nthreads=0, return_flags=False):
    """Align pairs k = 0..n-1: A[offA[k]:offA[k+1]] (reference) vs B[offB[k]:offB[k+1]] (query).

    DNA: ``scores = (match, mismatch, open, extend)``.
    Protein: ``matrix`` (576 ints), ``encoding`` (91 ints), ``gaps = (open, extend)``.
    """
    lib = load()
    A = _as_u8(A)
    B = _as_u8(B)
    offA = np.ascontiguousarray(offA, dtype=np.int64)
    offB = np.ascontiguousarray(offB, dtype=np.int64)
    n = len(offA) - 1
    if len(offB) - 1 != n:
        raise ValueError("offset arrays differ in length")
    sc = _Scoring()
    keep = []
    if kind == DNA:
        m, mm, o, e = scores
        sc.kind, sc.match, sc.mismatch, sc.open, sc.extend = DNA, m, mm, o, e
    else:
        o, e = gaps
        mat = np.ascontiguousarray(matrix, dtype=np.int16)
        enc = np.ascontiguousarray(encoding, dtype=np.int16)
        keep += [mat, enc]
        sc.kind, sc.open, sc.extend = AA, o, e
        sc.matrix = mat.ctypes.data_as(ctypes.POINTER(ctypes.c_int16))
        sc.encoding = enc.ctypes.data_as(ctypes.POINTER(ctypes.c_int16))
    out = np.zeros((n, 5), dtype=np.int32)
    flags = np.zeros(n, dtype=np.int32)
    # empty buffers still need a valid pointer
    Ab = A if A.size else np.zeros(1, np.uint8)
    Bb = B if B.size else np.zeros(1, np.uint8)
    rc = lib.oracle_align_batch(Ab.ctypes.data, offA.ctypes.data, Bb.ctypes.data, offB.ctypes.data,
                                n, ctypes.byref(sc), out.ctypes.data, flags.ctypes.data, int(nthreads))
    if rc != 0:
        raise ValueError("oracle_align_batch failed with status %d" % rc)
    return (out, flags) if return_flags else out


def align_strings(kind, refs, queries, **kw):
    """Convenience form over two lists of str/bytes."""
    def pack(seqs):
        bs = [s.encode() if isinstance(s, str) else bytes(s) for s in seqs]
        off = np.zeros(len(bs) + 1, dtype=np.int64)
        off[1:] = np.cumsum([len(b) for b in bs])
        return np.frombuffer(b"".join(bs), dtype=np.uint8), off
    A, offA = pack(refs)
    B, offB = pack(queries)
    return align(kind, A, offA, B, offB, **kw)


OPS = {1: "I", 2: "D", 7: "=", 8: "X"}


def traceback(kind, A, offA, B, offB, results, scores=None, matrix=None, encoding=None, gaps=None, nthreads=0):
    """Paths of aligned pairs.  ``results``: (n, 5) score, ref_begin, ref_end,
    query_begin, query_end.  Returns (ops, ops_off, path_score): the run-length
    operations of pair k are ops[ops_off[k]:ops_off[k+1]] (length << 4 | op)."""
    lib = load()
    A = _as_u8(A)
    B = _as_u8(B)
    offA = np.ascontiguousarray(offA, dtype=np.int64)
    offB = np.ascontiguousarray(offB, dtype=np.int64)
    res = np.ascontiguousarray(results, dtype=np.int32).reshape(-1, 5)
    n = len(offA) - 1
    sc = _Scoring()
    keep = []
    if kind == DNA:
        m, mm, o, e = scores
        sc.kind, sc.match, sc.mismatch, sc.open, sc.extend = DNA, m, mm, o, e
    else:
        o, e = gaps
        mat = np.ascontiguousarray(matrix, dtype=np.int16)
        enc = np.ascontiguousarray(encoding, dtype=np.int16)
        keep += [mat, enc]
        sc.kind, sc.open, sc.extend = AA, o, e
        sc.matrix = mat.ctypes.data_as(ctypes.POINTER(ctypes.c_int16))
        sc.encoding = enc.ctypes.data_as(ctypes.POINTER(ctypes.c_int16))
    cap = np.where(res[:, 0] > 0, (res[:, 2] - res[:, 1]) + (res[:, 4] - res[:, 3]), 0).astype(np.int64)
    slot = np.zeros(n + 1, dtype=np.int64)
    slot[1:] = np.cumsum(np.maximum(cap, 0))
    ops = np.zeros(max(int(slot[-1]), 1), dtype=np.uint32)
    nops = np.zeros(n, dtype=np.int32)
    pscore = np.zeros(n, dtype=np.int32)
    Ab = A if A.size else np.zeros(1, np.uint8)
    Bb = B if B.size else np.zeros(1, np.uint8)
    rc = lib.oracle_traceback_batch(Ab.ctypes.data, offA.ctypes.data, Bb.ctypes.data, offB.ctypes.data, n,
                                    ctypes.byref(sc), res.ctypes.data, ops.ctypes.data, slot.ctypes.data,
                                    nops.ctypes.data, pscore.ctypes.data, int(nthreads))
    if rc != 0:
        raise ValueError("oracle_traceback_batch failed with status %d" % rc)
    off = np.zeros(n + 1, dtype=np.int64)
    off[1:] = np.cumsum(nops)
    packed = np.concatenate([ops[slot[k]:slot[k] + nops[k]] for k in range(n)]) if n else np.zeros(0, np.uint32)
    return packed.astype(np.uint32), off, pscore


def cigar(ops):
    """Run-length operations -> CIGAR string."""
    return "".join("%d%s" % (int(v) >> 4, OPS[int(v) & 15]) for v in ops)
