"""GB300-native batched Smith-Waterman (affine gaps) -- Python host side.

A ctypes layer over ``_lib/libgbsw.so`` (C ABI in ``include/gbsw.h``).  The
functions mirror the reference's driver API (ADEPT / GPU-BSW ``driver.hpp``):

* ``kernel_driver_dna(reads, contigs, scores, factor=1.0)``
* ``kernel_driver_aa(reads, contigs, scoring_matrix, openGap, extendGap, factor=1.0)``
* ``get_tot_gpu_mem(id)``

with the same argument meaning (reads = queries = seqB, contigs = references =
seqA, ``scores = [match, mismatch, gap open, gap extend]``).  Where the C++
functions fill an ``alignment_results`` struct, these return an
:class:`AlignmentResults` of int16 numpy arrays with the same five fields; errors
raise :class:`GbswError` (the C++ drop-in exits the process instead, like the
reference).  ``Aligner`` exposes the int32 and device-resident entry points.

Import with ``importlib.import_module("gpu-bsw_gb300")`` (the directory name is
not a Python identifier).
"""
import collections
import ctypes
import os

import numpy as np

from . import scoring
from ._paths import GBSW_LIB, LIBDIR

DNA = 0
PROTEIN = 1

STATUS = {0: "ok", -1: "invalid argument", -2: "protein symbol outside the encoding table",
          -3: "sequence too long", -4: "CUDA error", -5: "out of memory", -6: "internal error",
          -7: "batch larger than the fixed scratch of the allocation-free entry",
          -8: "job not finished within the timeout"}

AlignmentResults = collections.namedtuple(
    "AlignmentResults", ["ref_begin", "query_begin", "ref_end", "query_end", "top_scores"])


class GbswError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("%s (%d): %s" % (STATUS.get(status, "error"), status, message))
        self.status = status


class _Scoring(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("match", ctypes.c_int16), ("mismatch", ctypes.c_int16),
                ("gap_open", ctypes.c_int16), ("gap_extend", ctypes.c_int16),
                ("matrix", ctypes.POINTER(ctypes.c_int16))]


class _Options(ctypes.Structure):
    _fields_ = [("use_dpx", ctypes.c_int32), ("blocks_per_sm", ctypes.c_int32), ("lane_group", ctypes.c_int32)]


class _Calibration(ctypes.Structure):
    _fields_ = [("sms", ctypes.c_int32), ("sm_mhz", ctypes.c_double),
                ("addmax_relu_s32", ctypes.c_double), ("max3_relu_s32", ctypes.c_double),
                ("plain_addmax_s32", ctypes.c_double), ("addmax_relu_s16x2", ctypes.c_double),
                ("max3_relu_s16x2", ctypes.c_double), ("iadd_s32", ctypes.c_double),
                ("cell_dpx", ctypes.c_double), ("cell_plain", ctypes.c_double),
                ("cell_dual", ctypes.c_double), ("cell_dpx_gcups", ctypes.c_double),
                ("cell_dual_gcups", ctypes.c_double), ("cell_int32", ctypes.c_double),
                ("cell_int32_gcups", ctypes.c_double)]


class _Stats(ctypes.Structure):
    _fields_ = [("forward_ms", ctypes.c_double), ("reverse_ms", ctypes.c_double),
                ("h2d_ms", ctypes.c_double), ("d2h_ms", ctypes.c_double),
                ("total_ms", ctypes.c_double), ("cells", ctypes.c_int64),
                ("launches", ctypes.c_int32), ("lane_group", ctypes.c_int32), ("dual", ctypes.c_int32),
                ("reruns", ctypes.c_int64), ("bin_pairs", ctypes.c_int64 * 2), ("bin_dual", ctypes.c_int32 * 2),
                ("bin_lanes", ctypes.c_int32 * 2), ("bin_tuned", ctypes.c_int32 * 2),
                ("rev_dual", ctypes.c_int32 * 2), ("rev_lanes", ctypes.c_int32 * 2)]


BINS = 2
COUNT_BUCKETS = 6
# upper pair counts of the tuning table's buckets (the last is open-ended)
BUCKET_EDGES = (1000, 3000, 10000, 30000, 100000)
TUNE_CANDIDATES = 8


class _Variant(ctypes.Structure):
    _fields_ = [("dual", ctypes.c_int32), ("lanes", ctypes.c_int32)]


class _Tuning(ctypes.Structure):
    _fields_ = [("variant", _Variant * COUNT_BUCKETS * BINS * 2), ("reverse", _Variant * COUNT_BUCKETS * BINS * 2)]


class _TuneReport(ctypes.Structure):
    _fields_ = [("ncandidates", ctypes.c_int32), ("candidates", _Variant * TUNE_CANDIDATES),
                ("ms_forward", ctypes.c_double * TUNE_CANDIDATES * BINS),
                ("ms_reverse", ctypes.c_double * TUNE_CANDIDATES * BINS), ("pairs", ctypes.c_int64 * BINS),
                ("bucket", ctypes.c_int32 * BINS), ("chosen", _Variant * BINS), ("chosen_reverse", _Variant * BINS)]


class _ServerOptions(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int32), ("slots", ctypes.c_int32), ("hbm_budget", ctypes.c_uint64),
                ("max_batch_pairs", ctypes.c_int64)]


class _JobInfo(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int32), ("pairs", ctypes.c_int64), ("cells", ctypes.c_int64),
                ("queue_ms", ctypes.c_double), ("latency_ms", ctypes.c_double)]


class _ServerStats(ctypes.Structure):
    _fields_ = [("jobs", ctypes.c_int64), ("batches", ctypes.c_int64), ("peak_running", ctypes.c_int64),
                ("pairs", ctypes.c_int64), ("cells", ctypes.c_int64),
                ("queued", ctypes.c_int64), ("hbm_in_use", ctypes.c_uint64), ("p50_ms", ctypes.c_double),
                ("p99_ms", ctypes.c_double), ("max_ms", ctypes.c_double), ("gcups", ctypes.c_double),
                ("staged", ctypes.c_int64)]


class _Packed(ctypes.Structure):
    _fields_ = [("words", ctypes.c_void_p), ("nsym", ctypes.c_int64), ("nruns", ctypes.c_int64),
                ("run_at", ctypes.c_void_p), ("run_off", ctypes.c_void_p), ("run_bytes", ctypes.c_void_p)]


# Every symbol include/gbsw.h declares (checked by the CPU tests).
EXPORTS = ["gbsw_create", "gbsw_destroy", "gbsw_strerror", "gbsw_last_error", "gbsw_align_host16",
           "gbsw_align_host32", "gbsw_align_device", "gbsw_check", "gbsw_device_memory", "gbsw_split_pairs",
           "gbsw_set_options", "gbsw_get_options", "gbsw_last_stats", "gbsw_calibrate",
           "gbsw_get_tuning", "gbsw_set_tuning", "gbsw_tune_device",
           "gbsw_align_device_noalloc", "gbsw_server_create", "gbsw_server_destroy", "gbsw_server_submit",
           "gbsw_server_wait", "gbsw_server_get_stats", "gbsw_server_reset_stats", "gbsw_traceback_host",
           "gbsw_packed_words", "gbsw_pack", "gbsw_unpack_device", "gbsw_align_packed_host16",
           "gbsw_align_packed_host32", "gbsw_server_submit_packed"]

_lib = None
_vp = ctypes.c_void_p
_i64 = ctypes.c_int64


def lib_path():
    return GBSW_LIB


def load():
    """Load libgbsw.so; raises if it has not been built (there is no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(GBSW_LIB):
        raise ImportError("libgbsw.so is not built (%s); run __graft_entry__.build()" % GBSW_LIB)
    lib = ctypes.CDLL(GBSW_LIB)
    lib.gbsw_create.argtypes = [ctypes.c_int, ctypes.POINTER(_vp)]
    lib.gbsw_destroy.argtypes = [_vp]
    lib.gbsw_destroy.restype = None
    lib.gbsw_strerror.restype = ctypes.c_char_p
    lib.gbsw_strerror.argtypes = [ctypes.c_int]
    lib.gbsw_last_error.restype = ctypes.c_char_p
    lib.gbsw_last_error.argtypes = [_vp]
    host_args = [_vp, ctypes.POINTER(_Scoring), _vp, _vp, _vp, _vp, _i64] + [_vp] * 5
    lib.gbsw_align_host16.argtypes = host_args
    lib.gbsw_align_host32.argtypes = host_args
    lib.gbsw_align_device.argtypes = [_vp, ctypes.POINTER(_Scoring), _vp, _vp, _vp, _vp, _i64,
                                      ctypes.c_int32] + [_vp] * 5 + [_vp]
    lib.gbsw_check.argtypes = [_vp, _vp]
    lib.gbsw_device_memory.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_uint64)]
    lib.gbsw_split_pairs.argtypes = [_vp, _i64, ctypes.c_int, _vp]
    lib.gbsw_set_options.argtypes = [_vp, ctypes.POINTER(_Options)]
    lib.gbsw_get_options.argtypes = [_vp, ctypes.POINTER(_Options)]
    lib.gbsw_last_stats.argtypes = [_vp, ctypes.POINTER(_Stats)]
    lib.gbsw_calibrate.argtypes = [ctypes.c_int, ctypes.POINTER(_Calibration)]
    lib.gbsw_get_tuning.argtypes = [_vp, ctypes.POINTER(_Tuning)]
    lib.gbsw_set_tuning.argtypes = [_vp, ctypes.POINTER(_Tuning)]
    lib.gbsw_tune_device.argtypes = [_vp, ctypes.POINTER(_Scoring), _vp, _vp, _vp, _vp, _i64, ctypes.c_int32,
                                     ctypes.c_int32, _vp, ctypes.POINTER(_TuneReport)]
    lib.gbsw_align_device_noalloc.argtypes = [ctypes.POINTER(_Scoring), _vp, _vp, _vp, _vp, _i64,
                                              ctypes.c_int32] + [_vp] * 5 + [_vp]
    lib.gbsw_traceback_host.argtypes = [_vp, ctypes.POINTER(_Scoring), _vp, _vp, _vp, _vp, _i64] + [_vp] * 5 + [
        _vp, ctypes.POINTER(ctypes.POINTER(ctypes.c_uint32))]
    lib.gbsw_server_create.argtypes = [ctypes.POINTER(_ServerOptions), ctypes.POINTER(_vp)]
    lib.gbsw_server_destroy.argtypes = [_vp]
    lib.gbsw_server_destroy.restype = None
    lib.gbsw_server_submit.argtypes = [_vp, ctypes.POINTER(_Scoring), _vp, _vp, _vp, _vp, _i64, _vp,
                                       ctypes.POINTER(ctypes.c_uint64)]
    lib.gbsw_server_wait.argtypes = [_vp, ctypes.c_uint64, ctypes.c_double, ctypes.POINTER(_JobInfo)]
    lib.gbsw_server_get_stats.argtypes = [_vp, ctypes.POINTER(_ServerStats)]
    lib.gbsw_server_reset_stats.argtypes = [_vp]
    lib.gbsw_packed_words.argtypes = [ctypes.c_int, _i64]
    lib.gbsw_packed_words.restype = _i64
    lib.gbsw_pack.argtypes = [ctypes.c_int, _vp, _i64, ctypes.c_int, _vp, _i64, _vp, _vp, _i64, _vp, _vp, _vp]
    lib.gbsw_unpack_device.argtypes = [ctypes.c_int, ctypes.POINTER(_Packed), _vp, _vp]
    packed_args = [_vp, ctypes.POINTER(_Scoring), ctypes.POINTER(_Packed), _vp, ctypes.POINTER(_Packed), _vp,
                   _i64] + [_vp] * 5
    lib.gbsw_align_packed_host16.argtypes = packed_args
    lib.gbsw_server_submit_packed.argtypes = [_vp, ctypes.POINTER(_Scoring), ctypes.POINTER(_Packed), _vp,
                                              ctypes.POINTER(_Packed), _vp, _i64, _vp, _vp]
    lib.gbsw_align_packed_host32.argtypes = packed_args
    _lib = lib
    return lib


def make_scoring(kind, scores=None, matrix=None, gaps=None):
    """DNA: ``scores = (match, mismatch, open, extend)``; protein: ``matrix`` (576) and ``gaps``."""
    sc = _Scoring()
    keep = None
    if kind == DNA:
        m, mm, o, e = scores
        sc.kind, sc.match, sc.mismatch, sc.gap_open, sc.gap_extend = DNA, m, mm, o, e
    else:
        o, e = gaps
        keep = np.ascontiguousarray(matrix, dtype=np.int16)
        if keep.size != 576:
            raise ValueError("protein matrix must have 576 entries")
        sc.kind, sc.gap_open, sc.gap_extend = PROTEIN, o, e
        sc.matrix = keep.ctypes.data_as(ctypes.POINTER(ctypes.c_int16))
    sc._keep = keep
    return sc


def _concat(seqs):
    bs = [s.encode() if isinstance(s, str) else bytes(s) for s in seqs]
    off = np.zeros(len(bs) + 1, dtype=np.int64)
    if bs:
        off[1:] = np.cumsum([len(b) for b in bs])
    buf = np.frombuffer(b"".join(bs) or b"\0", dtype=np.uint8)
    return buf, off


def _ptr(a):
    return a.ctypes.data if a is not None else None


class PackedStream:
    """A packed sequence stream (gbsw_packed): 2-bit DNA or 5-bit protein codes
    in uint32 words, and the escape runs that keep other bytes raw.  Symbol j
    is raw byte j of the buffer it was packed from."""

    def __init__(self, kind, words, nsym, run_at, run_off, run_bytes):
        self.kind = kind
        self.words = words
        self.nsym = int(nsym)
        self.run_at = run_at
        self.run_off = run_off
        self.run_bytes = run_bytes

    @property
    def nruns(self):
        return len(self.run_at)

    @property
    def nbytes(self):
        """Bytes a copy of the stream moves: words, run positions, offsets and bytes."""
        if self.nruns == 0:
            return self.words.nbytes
        return self.words.nbytes + self.run_at.nbytes + self.run_off.nbytes + self.run_bytes.nbytes

    def struct(self):
        p = _Packed()
        p.words = _ptr(self.words)
        p.nsym = self.nsym
        p.nruns = self.nruns
        p.run_at = _ptr(self.run_at)
        p.run_off = _ptr(self.run_off)
        p.run_bytes = _ptr(self.run_bytes)
        return p


def pack(kind, raw, threads=0, out=None):
    """Pack a raw byte buffer (gbsw_pack).  ``out``: optional uint32 array to
    hold the words (for example page-locked memory)."""
    lib = load()
    raw = np.ascontiguousarray(raw, dtype=np.uint8)
    nsym = raw.size
    nw = int(lib.gbsw_packed_words(kind, nsym))
    if nw < 0:
        raise ValueError("bad kind")
    words = out[:nw] if out is not None else np.empty(max(nw, 1), dtype=np.uint32)[:nw]
    nruns = ctypes.c_int64()
    nbytes = ctypes.c_int64()
    run_off = np.zeros(1, np.int64)
    src = raw if nsym else np.zeros(1, np.uint8)
    wp = words.ctypes.data if nw else np.zeros(1, np.uint32).ctypes.data
    rc = lib.gbsw_pack(kind, _ptr(src), nsym, int(threads), wp, 0, None, None, 0, None, ctypes.byref(nruns),
                       ctypes.byref(nbytes))
    if rc == -7:  # escapes: a second call with room for them
        run_at = np.empty(nruns.value, np.int64)
        run_off = np.empty(nruns.value + 1, np.int64)
        run_bytes = np.empty(max(nbytes.value, 1), np.uint8)
        rc = lib.gbsw_pack(kind, _ptr(src), nsym, int(threads), wp, nruns.value, _ptr(run_at), _ptr(run_off),
                           nbytes.value, _ptr(run_bytes), ctypes.byref(nruns), ctypes.byref(nbytes))
        run_bytes = run_bytes[:nbytes.value]
    else:
        run_at = np.zeros(0, np.int64)
        run_bytes = np.zeros(0, np.uint8)
    if rc != 0:
        raise GbswError(rc, "gbsw_pack")
    return PackedStream(kind, words, nsym, run_at, run_off, run_bytes)


class Aligner:
    """One library context on one CUDA device."""

    def __init__(self, device=0, use_dpx=None, blocks_per_sm=None, lane_group=None):
        self.lib = load()
        h = _vp()
        rc = self.lib.gbsw_create(int(device), ctypes.byref(h))
        if rc != 0:
            raise GbswError(rc, "gbsw_create(%d)" % device)
        self.handle = h
        self.set_options(use_dpx=use_dpx, blocks_per_sm=blocks_per_sm, lane_group=lane_group)

    def set_options(self, use_dpx=None, blocks_per_sm=None, lane_group=None):
        """Change execution options; None keeps the current value.  ``lane_group``:
        0 chooses the lanes per pair from the batch size, 4/8/16/32 forces it."""
        o = _Options()
        self._check(self.lib.gbsw_get_options(self.handle, ctypes.byref(o)))
        if use_dpx is not None:
            o.use_dpx = 1 if use_dpx else 0
        if blocks_per_sm is not None:
            o.blocks_per_sm = int(blocks_per_sm)
        if lane_group is not None:
            o.lane_group = int(lane_group)
        self._check(self.lib.gbsw_set_options(self.handle, ctypes.byref(o)))

    def close(self):
        if getattr(self, "handle", None):
            self.lib.gbsw_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != 0:
            msg = self.lib.gbsw_last_error(self.handle).decode(errors="replace")
            raise GbswError(rc, msg)

    def align_host(self, sc, ref, ref_off, query, query_off, int16=False):
        """Raw host buffers in, host results out: (n, 5) array of score, ref_begin, ref_end,
        query_begin, query_end."""
        ref = np.ascontiguousarray(ref, dtype=np.uint8)
        query = np.ascontiguousarray(query, dtype=np.uint8)
        ref_off = np.ascontiguousarray(ref_off, dtype=np.int64)
        query_off = np.ascontiguousarray(query_off, dtype=np.int64)
        n = len(ref_off) - 1
        dt = np.int16 if int16 else np.int32
        out = np.empty((5, max(n, 0)), dtype=dt)
        if ref.size == 0:
            ref = np.zeros(1, np.uint8)
        if query.size == 0:
            query = np.zeros(1, np.uint8)
        fn = self.lib.gbsw_align_host16 if int16 else self.lib.gbsw_align_host32
        rc = fn(self.handle, ctypes.byref(sc), _ptr(ref), _ptr(ref_off), _ptr(query), _ptr(query_off),
                n, _ptr(out[1]), _ptr(out[2]), _ptr(out[3]), _ptr(out[4]), _ptr(out[0]))
        self._check(rc)
        return out.T  # (n, 5) view of the five result arrays

    def align_packed(self, sc, pref, ref_off, pquery, query_off, int16=False):
        """Packed host streams in (``pack``), host results out, as ``align_host``:
        the copy to the device carries the packed words, unpacked there."""
        ref_off = np.ascontiguousarray(ref_off, dtype=np.int64)
        query_off = np.ascontiguousarray(query_off, dtype=np.int64)
        n = len(ref_off) - 1
        dt = np.int16 if int16 else np.int32
        out = np.empty((5, max(n, 0)), dtype=dt)
        pr, pq = pref.struct(), pquery.struct()
        fn = self.lib.gbsw_align_packed_host16 if int16 else self.lib.gbsw_align_packed_host32
        rc = fn(self.handle, ctypes.byref(sc), ctypes.byref(pr), _ptr(ref_off), ctypes.byref(pq), _ptr(query_off),
                n, _ptr(out[1]), _ptr(out[2]), _ptr(out[3]), _ptr(out[4]), _ptr(out[0]))
        self._check(rc)
        return out.T

    def traceback(self, sc, ref, ref_off, query, query_off, results):
        """Paths of aligned pairs (gbsw_traceback_host).  ``results``: the (n, 5)
        int32 array ``align_host`` returned for the same pairs and scoring.
        Returns (ops, ops_off): pair k's run-length operations (length << 4 | op)
        are ops[ops_off[k]:ops_off[k+1]]; ``cigar(ops)`` formats them."""
        ref = np.ascontiguousarray(ref, dtype=np.uint8)
        query = np.ascontiguousarray(query, dtype=np.uint8)
        ref_off = np.ascontiguousarray(ref_off, dtype=np.int64)
        query_off = np.ascontiguousarray(query_off, dtype=np.int64)
        n = len(ref_off) - 1
        res = np.ascontiguousarray(np.asarray(results, dtype=np.int32).reshape(-1, 5).T)
        if ref.size == 0:
            ref = np.zeros(1, np.uint8)
        if query.size == 0:
            query = np.zeros(1, np.uint8)
        off = np.zeros(n + 1, dtype=np.int64)
        ptr = ctypes.POINTER(ctypes.c_uint32)()
        rc = self.lib.gbsw_traceback_host(self.handle, ctypes.byref(sc), _ptr(ref), _ptr(ref_off), _ptr(query),
                                          _ptr(query_off), n, _ptr(res[0]), _ptr(res[1]), _ptr(res[2]),
                                          _ptr(res[3]), _ptr(res[4]), _ptr(off), ctypes.byref(ptr))
        self._check(rc)
        total = int(off[-1])
        ops = np.ctypeslib.as_array(ptr, shape=(total,)).copy() if total else np.zeros(0, np.uint32)
        return ops, off

    def traceback_batch(self, batch, sc, results):
        return self.traceback(sc, batch.ref, batch.ref_off, batch.query, batch.query_off, results)

    def align_batch(self, batch, sc, int16=False):
        return self.align_host(sc, batch.ref, batch.ref_off, batch.query, batch.query_off, int16)

    def align_device(self, sc, ref_ptr, ref_off_ptr, query_ptr, query_off_ptr, n, max_len,
                     score_ptr, ref_begin_ptr, ref_end_ptr, query_begin_ptr, query_end_ptr,
                     stream=None):
        """Device pointers (ints, e.g. ``tensor.data_ptr()``); asynchronous on ``stream``."""
        rc = self.lib.gbsw_align_device(self.handle, ctypes.byref(sc), ref_ptr, ref_off_ptr, query_ptr,
                                        query_off_ptr, int(n), int(max_len), score_ptr,
                                        ref_begin_ptr, ref_end_ptr, query_begin_ptr,
                                        query_end_ptr, stream)
        self._check(rc)

    def check(self, stream=None):
        self._check(self.lib.gbsw_check(self.handle, stream))

    def stats(self):
        s = _Stats()
        self._check(self.lib.gbsw_last_stats(self.handle, ctypes.byref(s)))
        out = {}
        for k, _ in _Stats._fields_:
            v = getattr(s, k)
            out[k] = list(v) if isinstance(v, ctypes.Array) else v
        return out

    # ---- per-length-bin plans ----
    def get_tuning(self, reverse=False):
        """The tuning table of the forward pass (``reverse``: of the reverse pass) as
        {(kind, bin, bucket): (dual, lanes)} (entries only)."""
        t = _Tuning()
        self._check(self.lib.gbsw_get_tuning(self.handle, ctypes.byref(t)))
        tab = t.reverse if reverse else t.variant
        return {(k, b, q): (tab[k][b][q].dual, tab[k][b][q].lanes)
                for k in range(2) for b in range(BINS) for q in range(COUNT_BUCKETS) if tab[k][b][q].lanes}

    def set_tuning(self, entries, reverse_entries=None):
        """Replace the table with {(kind, bin, bucket): (dual, lanes)} for the forward
        pass and, optionally, the reverse pass; missing entries fall back (a missing
        reverse entry: the forward one)."""
        t = _Tuning()
        for tab, ents in ((t.variant, entries), (t.reverse, reverse_entries or {})):
            for (k, b, q), (dual, lanes) in ents.items():
                tab[k][b][q].dual, tab[k][b][q].lanes = int(dual), int(lanes)
        self._check(self.lib.gbsw_set_tuning(self.handle, ctypes.byref(t)))

    def tune_device(self, sc, ref_ptr, ref_off_ptr, query_ptr, query_off_ptr, n, max_len, reps=2, stream=None):
        """gbsw_tune_device: times every candidate variant per bin on this batch and
        stores each bin's fastest in the table.  Returns the report as a dict."""
        r = _TuneReport()
        self._check(self.lib.gbsw_tune_device(self.handle, ctypes.byref(sc), ref_ptr, ref_off_ptr, query_ptr,
                                              query_off_ptr, int(n), int(max_len), int(reps), stream,
                                              ctypes.byref(r)))
        cands = [(r.candidates[c].dual, r.candidates[c].lanes) for c in range(r.ncandidates)]
        nc = r.ncandidates
        return {"candidates": cands,
                "bins": [{"pairs": r.pairs[b], "bucket": r.bucket[b],
                          "chosen": (r.chosen[b].dual, r.chosen[b].lanes) if r.pairs[b] > 0 else None,
                          "chosen_reverse": ((r.chosen_reverse[b].dual, r.chosen_reverse[b].lanes)
                                             if r.pairs[b] > 0 else None),
                          "ms_forward": [r.ms_forward[b][c] for c in range(nc)],
                          "ms_reverse": [r.ms_reverse[b][c] for c in range(nc)],
                          "ms": [r.ms_forward[b][c] + r.ms_reverse[b][c] for c in range(nc)]}
                         for b in range(BINS)]}


class Job:
    """A submitted job: ``wait()`` returns its (n, 5) int32 results."""

    def __init__(self, server, job_id, out, keep):
        self.server, self.id, self.out, self._keep = server, job_id, out, keep
        self.info = None

    def wait(self, timeout=None):
        if self.info is None:
            info = _JobInfo()
            rc = self.server.lib.gbsw_server_wait(self.server.handle, self.id,
                                                  -1.0 if timeout is None else float(timeout),
                                                  ctypes.byref(info))
            if rc == -8:
                raise TimeoutError("job %d not finished after %s s" % (self.id, timeout))
            self.server._pending.pop(self.id, None)
            if rc != 0:
                raise GbswError(rc, "job %d" % self.id)
            self.info = {k: getattr(info, k) for k, _ in _JobInfo._fields_}
            self._keep = None
        return self.out


class Server:
    """Serving loop on one device (gbsw_server_*): jobs from any thread, batched
    continuously onto ``slots`` concurrent contexts within an HBM budget."""

    def __init__(self, device=0, slots=4, hbm_budget=16 << 30, max_batch_pairs=50_000):
        self.lib = load()
        o = _ServerOptions(int(device), int(slots), int(hbm_budget), int(max_batch_pairs))
        h = _vp()
        rc = self.lib.gbsw_server_create(ctypes.byref(o), ctypes.byref(h))
        if rc != 0:
            raise GbswError(rc, "gbsw_server_create(device=%d, slots=%d)" % (device, slots))
        self.handle = h
        # jobs not yet waited for: their result arrays must outlive the workers' writes
        self._pending = {}

    def submit(self, sc, ref, ref_off, query, query_off):
        ref = np.ascontiguousarray(ref, dtype=np.uint8)
        query = np.ascontiguousarray(query, dtype=np.uint8)
        ref_off = np.ascontiguousarray(ref_off, dtype=np.int64)
        query_off = np.ascontiguousarray(query_off, dtype=np.int64)
        n = len(ref_off) - 1
        out = np.zeros((max(n, 0), 5), dtype=np.int32)
        jid = ctypes.c_uint64()
        rc = self.lib.gbsw_server_submit(self.handle, ctypes.byref(sc), _ptr(ref) if ref.size else None,
                                         _ptr(ref_off), _ptr(query) if query.size else None,
                                         _ptr(query_off), n, _ptr(out), ctypes.byref(jid))
        if rc != 0:
            raise GbswError(rc, "gbsw_server_submit")
        job = Job(self, jid.value, out, sc)
        self._pending[job.id] = job
        return job

    def submit_batch(self, batch, sc):
        return self.submit(sc, batch.ref, batch.ref_off, batch.query, batch.query_off)

    def submit_packed(self, sc, pref, ref_off, pquery, query_off):
        """A job as packed streams (``pack``): it stays packed until a worker
        gathers its batch on the device.  Offsets start at 0."""
        ref_off = np.ascontiguousarray(ref_off, dtype=np.int64)
        query_off = np.ascontiguousarray(query_off, dtype=np.int64)
        n = len(ref_off) - 1
        out = np.zeros((max(n, 0), 5), dtype=np.int32)
        jid = ctypes.c_uint64()
        pr, pq = pref.struct(), pquery.struct()
        rc = self.lib.gbsw_server_submit_packed(self.handle, ctypes.byref(sc), ctypes.byref(pr), _ptr(ref_off),
                                                ctypes.byref(pq), _ptr(query_off), n, _ptr(out), ctypes.byref(jid))
        if rc != 0:
            raise GbswError(rc, "gbsw_server_submit_packed")
        job = Job(self, jid.value, out, (sc, pref, pquery))
        self._pending[job.id] = job
        return job

    def stats(self):
        s = _ServerStats()
        rc = self.lib.gbsw_server_get_stats(self.handle, ctypes.byref(s))
        if rc != 0:
            raise GbswError(rc, "gbsw_server_get_stats")
        return {k: getattr(s, k) for k, _ in _ServerStats._fields_}

    def reset_stats(self):
        self.lib.gbsw_server_reset_stats(self.handle)

    def close(self):
        """Finishes the queued jobs, then stops the workers."""
        if getattr(self, "handle", None):
            self.lib.gbsw_server_destroy(self.handle)
            self.handle = None
            self._pending.clear()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default = {}


def _aligner():
    import threading
    key = threading.get_ident()
    if key not in _default:
        _default[key] = Aligner(0)
    return _default[key]


def _driver(reads, contigs, sc, factor):
    if len(reads) != len(contigs):
        raise ValueError("reads and contigs differ in count")
    ref, ref_off = _concat(contigs)
    query, query_off = _concat(reads)
    out = _aligner().align_host(sc, ref, ref_off, query, query_off, int16=True)
    return AlignmentResults(ref_begin=out[:, 1].copy(), query_begin=out[:, 3].copy(),
                            ref_end=out[:, 2].copy(), query_end=out[:, 4].copy(),
                            top_scores=out[:, 0].copy())


def kernel_driver_dna(reads, contigs, scores, factor=1.0):
    """Mirror of ``gpu_bsw_driver::kernel_driver_dna`` (driver.hpp:32-33 of the reference)."""
    return _driver(reads, contigs, make_scoring(DNA, scores=tuple(scores)), factor)


def kernel_driver_aa(reads, contigs, scoring_matrix, openGap, extendGap, factor=1.0):
    """Mirror of ``gpu_bsw_driver::kernel_driver_aa`` (driver.hpp:36-37 of the reference)."""
    return _driver(reads, contigs, make_scoring(PROTEIN, matrix=scoring_matrix,
                                                gaps=(openGap, extendGap)), factor)


CIGAR_OPS = {1: "I", 2: "D", 7: "=", 8: "X"}


def cigar(ops):
    """Run-length operations (length << 4 | op) -> CIGAR string, e.g. "12=1X3I40=" """
    return "".join("%d%s" % (int(v) >> 4, CIGAR_OPS[int(v) & 15]) for v in ops)


def calibrate(device=0):
    """Integer-pipe probe rates (per clock64 tick per SM) and the cell probes'
    throughput in 1e9 cells per second -- see gbsw_calibrate."""
    c = _Calibration()
    rc = load().gbsw_calibrate(int(device), ctypes.byref(c))
    if rc != 0:
        raise GbswError(rc, "gbsw_calibrate(%d)" % device)
    return {k: getattr(c, k) for k, _ in _Calibration._fields_}


def get_tot_gpu_mem(id=0):
    """Mirror of ``gpu_bsw_driver::get_tot_gpu_mem`` (driver.hpp:29-30)."""
    v = ctypes.c_uint64()
    rc = load().gbsw_device_memory(int(id), ctypes.byref(v))
    if rc != 0:
        raise GbswError(rc, "gbsw_device_memory(%d)" % id)
    return v.value


__all__ = ["cigar", "Aligner", "Server", "Job", "AlignmentResults", "GbswError", "kernel_driver_dna", "kernel_driver_aa",
           "get_tot_gpu_mem", "make_scoring", "load", "scoring", "DNA", "PROTEIN", "LIBDIR"]
