"""Seeded synthetic workloads for the tests and the benchmark (ctypes over libgbsw_synth.so).

The presets follow the five benchmark configurations of this project:

1. ``plain_dna``     -- 1,000 pairs: reference U[200,500] bp, query a mutated
                        U[100,150] bp substring (5% substitutions, 1% indel events,
                        indel length geometric with mean 2).
2. ``dna_throughput``-- 100,000 pairs: reference U[400,1024], query U[150,300];
                        80% mutated substrings, 20% unrelated.
3. ``protein``       -- 30,000 pairs: log-normal lengths (median 300, sigma 0.5,
                        clipped to [50,1000]); 70% homologs at ~40% identity from
                        BLOSUM62-conditional substitution plus 5% indels
                        (2.5% events, mean length 2); 30% unrelated.
4. ``mixed_dna``     -- 200,000 pairs: 70% short (query U[100,150] vs a 300 bp
                        reference), 30% long (query U[1000,2048] vs reference
                        U[1500,4096]); all mutated substrings.
5. serving jobs draw 60% ``dna_throughput`` pairs and 40% ``protein`` pairs.

All scoring uses +3/-3/-6/-1 for DNA and BLOSUM62 with -6/-1 for protein.
"""
import ctypes
import os

import numpy as np

from . import scoring
from ._paths import LIBDIR

SYNTH_LIB = os.path.join(LIBDIR, "libgbsw_synth.so")

DNA, PROTEIN = 0, 1
UNIFORM, LOGNORMAL = 0, 1


class _Len(ctypes.Structure):
    _fields_ = [("dist", ctypes.c_int32), ("min", ctypes.c_int32), ("max", ctypes.c_int32),
                ("median", ctypes.c_double), ("sigma", ctypes.c_double)]


class _Comp(ctypes.Structure):
    _fields_ = [("weight", ctypes.c_double), ("alphabet", ctypes.c_int32),
                ("query_from_ref_length", ctypes.c_int32),
                ("ref_len", _Len), ("query_len", _Len),
                ("related_fraction", ctypes.c_double), ("substitution_rate", ctypes.c_double),
                ("target_identity", ctypes.c_double), ("indel_rate", ctypes.c_double),
                ("indel_mean", ctypes.c_double)]


class _Params(ctypes.Structure):
    _fields_ = [("ncomponents", ctypes.c_int32), ("components", _Comp * 4),
                ("aa_background", ctypes.c_double * 20), ("aa_matrix", ctypes.c_int32 * 400)]


class _Batch(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int64), ("ref", ctypes.c_void_p), ("ref_off", ctypes.c_void_p),
                ("query", ctypes.c_void_p), ("query_off", ctypes.c_void_p),
                ("component", ctypes.c_void_p), ("ref_total", ctypes.c_int64),
                ("query_total", ctypes.c_int64)]


_lib = None


def _load():
    global _lib
    if _lib is None:
        if not os.path.exists(SYNTH_LIB):
            from . import build as _build
            _build.build_synth()
        lib = ctypes.CDLL(SYNTH_LIB)
        lib.gbsw_synth_generate.restype = ctypes.c_int
        lib.gbsw_synth_generate.argtypes = [ctypes.POINTER(_Params), ctypes.c_int64,
                                            ctypes.c_uint64, ctypes.POINTER(_Batch)]
        lib.gbsw_synth_free.argtypes = [ctypes.POINTER(_Batch)]
        _lib = lib
    return _lib


class PairBatch:
    """Concatenated pairs: ``ref[ref_off[k]:ref_off[k+1]]`` vs ``query[query_off[k]:...]``."""

    def __init__(self, kind, ref, ref_off, query, query_off, component=None):
        self.kind = kind
        self.ref = np.ascontiguousarray(ref, dtype=np.uint8)
        self.ref_off = np.ascontiguousarray(ref_off, dtype=np.int64)
        self.query = np.ascontiguousarray(query, dtype=np.uint8)
        self.query_off = np.ascontiguousarray(query_off, dtype=np.int64)
        self.component = component

    @property
    def n(self):
        return len(self.ref_off) - 1

    def ref_lengths(self):
        return np.diff(self.ref_off)

    def query_lengths(self):
        return np.diff(self.query_off)

    def cells(self):
        """Forward cells, sum |ref| * |query| (the reference's "Total Cells", main.cpp:226-229)."""
        return int(np.sum(self.ref_lengths().astype(np.int64) * self.query_lengths()))

    def subset(self, idx):
        idx = np.asarray(idx, dtype=np.int64)
        return PairBatch(self.kind, *_gather(self.ref, self.ref_off, idx),
                         *_gather(self.query, self.query_off, idx),
                         None if self.component is None else self.component[idx])

    def strings(self, k):
        r = bytes(self.ref[self.ref_off[k]:self.ref_off[k + 1]])
        q = bytes(self.query[self.query_off[k]:self.query_off[k + 1]])
        return r, q

    @staticmethod
    def from_strings(kind, refs, queries):
        def pack(seqs):
            bs = [s.encode() if isinstance(s, str) else bytes(s) for s in seqs]
            off = np.zeros(len(bs) + 1, dtype=np.int64)
            if bs:
                off[1:] = np.cumsum([len(b) for b in bs])
            return np.frombuffer(b"".join(bs), dtype=np.uint8).copy(), off
        r, ro = pack(refs)
        q, qo = pack(queries)
        return PairBatch(kind, r, ro, q, qo)

    @staticmethod
    def concat(batches):
        kind = batches[0].kind
        refs = np.concatenate([b.ref for b in batches])
        qs = np.concatenate([b.query for b in batches])
        ro = [np.zeros(1, np.int64)]
        qo = [np.zeros(1, np.int64)]
        ra = qa = 0
        for b in batches:
            ro.append(b.ref_off[1:] + ra)
            qo.append(b.query_off[1:] + qa)
            ra += int(b.ref_off[-1])
            qa += int(b.query_off[-1])
        return PairBatch(kind, refs, np.concatenate(ro), qs, np.concatenate(qo))


def _gather(buf, off, idx):
    lens = off[idx + 1] - off[idx]
    new_off = np.zeros(len(idx) + 1, dtype=np.int64)
    new_off[1:] = np.cumsum(lens)
    total = int(new_off[-1])
    if total == 0:
        return np.zeros(0, np.uint8), new_off
    # position of every output byte in the source buffer
    starts = np.repeat(off[idx] - new_off[:-1], lens)
    src = starts + np.arange(total, dtype=np.int64)
    return buf[src], new_off


def _len(dist, lo, hi, median=0.0, sigma=0.0):
    return _Len(dist, lo, hi, median, sigma)


def _dna_comp(weight, ref_len, query_len, related=1.0):
    return _Comp(weight, DNA, 0, ref_len, query_len, related, 0.05, 0.0, 0.01, 2.0)


def _protein_comp(weight, related=0.7):
    ln = _len(LOGNORMAL, 50, 1000, 300.0, 0.5)
    return _Comp(weight, PROTEIN, 1, ln, ln, related, 0.0, 0.40, 0.025, 2.0)


def _params(comps):
    p = _Params()
    p.ncomponents = len(comps)
    for k, c in enumerate(comps):
        p.components[k] = c
    order20 = scoring.AA_ORDER[:20]
    for k, ch in enumerate(order20):
        p.aa_background[k] = scoring.AA_BACKGROUND[ch]
    for a in range(20):
        for b in range(20):
            p.aa_matrix[a * 20 + b] = scoring.BLOSUM62[a * 24 + b]
    return p


def generate(comps, n, seed, kind):
    lib = _load()
    p = _params(comps)
    b = _Batch()
    rc = lib.gbsw_synth_generate(ctypes.byref(p), int(n), int(seed), ctypes.byref(b))
    if rc != 0:
        raise ValueError("gbsw_synth_generate failed (%d)" % rc)
    try:
        def arr(ptr, count, dt):
            if count == 0:
                return np.zeros(0, dt)
            return np.ctypeslib.as_array(ctypes.cast(ptr, ctypes.POINTER(np.ctypeslib.as_ctypes_type(dt))),
                                         shape=(count,)).copy()
        ref = arr(b.ref, b.ref_total, np.uint8)
        query = arr(b.query, b.query_total, np.uint8)
        ro = arr(b.ref_off, n + 1, np.int64)
        qo = arr(b.query_off, n + 1, np.int64)
        comp = arr(b.component, n, np.int32) if n else np.zeros(0, np.int32)
    finally:
        lib.gbsw_synth_free(ctypes.byref(b))
    return PairBatch(kind, ref, ro, query, qo, comp)


# ---- presets ---------------------------------------------------------------

def plain_dna(n=1000, seed=1):
    return generate([_dna_comp(1.0, _len(UNIFORM, 200, 500), _len(UNIFORM, 100, 150))], n, seed, DNA)


def dna_throughput(n=100_000, seed=2):
    return generate([_dna_comp(1.0, _len(UNIFORM, 400, 1024), _len(UNIFORM, 150, 300), 0.8)],
                    n, seed, DNA)


def protein(n=30_000, seed=3):
    return generate([_protein_comp(1.0)], n, seed, PROTEIN)


def mixed_dna(n=200_000, seed=4):
    return generate([_dna_comp(0.7, _len(UNIFORM, 300, 300), _len(UNIFORM, 100, 150)),
                     _dna_comp(0.3, _len(UNIFORM, 1500, 4096), _len(UNIFORM, 1000, 2048))],
                    n, seed, DNA)


def mixed_dna_short(n=140_000, seed=4):
    """The short bin of ``mixed_dna`` alone (the part the reference can run)."""
    return generate([_dna_comp(1.0, _len(UNIFORM, 300, 300), _len(UNIFORM, 100, 150))], n, seed, DNA)


def custom_protein(n, seed, len_min, len_max, related=0.7):
    """Protein pairs of lengths U[len_min, len_max] (both sequences), otherwise
    like ``protein``: homologs at ~40% identity with 5% indels, the rest unrelated."""
    ln = _len(UNIFORM, len_min, len_max)
    return generate([_Comp(1.0, PROTEIN, 1, ln, ln, related, 0.0, 0.40, 0.025, 2.0)], n, seed, PROTEIN)


def custom_dna(n, seed, ref_min, ref_max, q_min, q_max, related=1.0):
    return generate([_dna_comp(1.0, _len(UNIFORM, ref_min, ref_max), _len(UNIFORM, q_min, q_max),
                               related)], n, seed, DNA)


def long_dna(n=400, seed=7):
    """Few long pairs: references U[4,000, 16,000] bp, queries U[3,000, 12,000] bp, 80% mutated
    substrings (shorter sides far above the reference's 1,024 limit)."""
    return custom_dna(n, seed, 4000, 16000, 3000, 12000, related=0.8)


PRESETS = {
    "plain_dna": plain_dna,
    "long_dna": long_dna,
    "dna_throughput": dna_throughput,
    "protein": protein,
    "mixed_dna": mixed_dna,
    "mixed_dna_short": mixed_dna_short,
}


def serving_jobs(count, seed=5, max_pairs=5000, dna_fraction=0.6):
    """Jobs of the serving stream: each holds U[1, max_pairs] pairs, drawn from the
    ``dna_throughput`` distribution with probability ``dna_fraction`` and from
    ``protein`` otherwise.  Returns a list of (kind, PairBatch)."""
    rng = np.random.default_rng(seed)
    jobs = []
    for k in range(count):
        n = int(rng.integers(1, max_pairs + 1))
        job_seed = int(seed) * 1_000_003 + k
        if rng.random() < dna_fraction:
            jobs.append((DNA, dna_throughput(n, job_seed)))
        else:
            jobs.append((PROTEIN, protein(n, job_seed)))
    return jobs
