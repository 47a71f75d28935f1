"""CPU tests of the packed sequence format (gbsw_pack): the word layout, escape
runs, multi-threaded packing and the round trip, checked by a numpy unpack
written here from the format's definition in gbsw.h."""
import ctypes

import numpy as np
import pytest

DNA_LETTERS = np.frombuffer(b"ACTG", np.uint8)


def unpack_np(p):
    """Raw bytes of a PackedStream, from the format's definition."""
    per, bits = (16, 2) if p.kind == 0 else (6, 5)
    j = np.arange(p.nsym, dtype=np.int64)
    codes = (p.words[j // per].astype(np.int64) >> (bits * (j % per))) & ((1 << bits) - 1)
    raw = DNA_LETTERS[codes] if p.kind == 0 else (codes + ord("A")).astype(np.uint8)
    raw = raw.astype(np.uint8)
    for r in range(p.nruns):
        a, b = int(p.run_off[r]), int(p.run_off[r + 1])
        raw[int(p.run_at[r]):int(p.run_at[r]) + (b - a)] = p.run_bytes[a:b]
    return raw


def _dna(rng, n, escapes=0.0):
    raw = rng.choice(np.frombuffer(b"ACGT", np.uint8), n)
    if escapes:
        k = rng.random(n) < escapes
        raw[k] = rng.choice(np.frombuffer(b"Nacgtn-", np.uint8), int(k.sum()))
    return raw


def test_word_layout(built):
    p = built.pack(built.DNA, np.frombuffer(b"ACTG" * 4 + b"GA", np.uint8))
    assert p.words.tolist() == [0xE4E4E4E4, 0x3]  # A C T G -> 0 1 2 3, lowest bits first
    assert p.nruns == 0 and p.nsym == 18
    q = built.pack(built.PROTEIN, np.frombuffer(b"ABCDEFZ", np.uint8))
    assert q.words.tolist() == [sum(c << (5 * k) for k, c in enumerate(range(6))), 25]
    assert q.words[0] >> 30 == 0


@pytest.mark.parametrize("n", [0, 1, 15, 16, 17, 1000, 4099])
def test_round_trip_dna(built, n):
    rng = np.random.default_rng(n)
    raw = _dna(rng, n, escapes=0.02)
    p = built.pack(built.DNA, raw)
    assert len(p.words) == (n + 15) // 16
    assert np.array_equal(unpack_np(p), raw)
    # runs: increasing, disjoint, maximal (no two touch), bytes outside A/C/G/T only
    ends = p.run_at + np.diff(p.run_off)
    assert np.all(p.run_at[1:] > ends[:-1])
    assert not np.isin(p.run_bytes, np.frombuffer(b"ACGT", np.uint8)).any()
    assert p.run_off[-1] == np.count_nonzero(~np.isin(raw, np.frombuffer(b"ACGT", np.uint8)))


@pytest.mark.parametrize("n", [0, 5, 6, 7, 48, 1001])
def test_round_trip_protein(built, n):
    rng = np.random.default_rng(100 + n)
    alpha = np.frombuffer(b"ARNDCQEGHILKMFPSTWYVBZX*abz", np.uint8)
    raw = rng.choice(alpha, n)
    p = built.pack(built.PROTEIN, raw)
    assert len(p.words) == (n + 5) // 6
    assert np.array_equal(unpack_np(p), raw)
    assert not (p.words >> 30).any()


def test_every_byte_value_round_trips(built):
    raw = np.arange(256, dtype=np.uint8).repeat(3)
    for kind in (built.DNA, built.PROTEIN):
        assert np.array_equal(unpack_np(built.pack(kind, raw)), raw)


def test_threads_and_chunk_edges(built):
    """A run across the packer's chunk edges (65,536 words) comes out as one run,
    and any thread count gives the same stream."""
    rng = np.random.default_rng(7)
    n = 16 * 65536 * 2 + 300
    raw = _dna(rng, n)
    edge = 16 * 65536
    raw[edge - 5:edge + 7] = ord("N")
    raw[2 * edge - 1:2 * edge + 1] = ord("n")
    a = built.pack(built.DNA, raw, threads=1)
    b = built.pack(built.DNA, raw, threads=7)
    assert np.array_equal(a.words, b.words)
    assert a.run_at.tolist() == b.run_at.tolist() == [edge - 5, 2 * edge - 1]
    assert a.run_off.tolist() == [0, 12, 14]
    assert np.array_equal(unpack_np(b), raw)


def test_capacities_and_arguments(built):
    lib = built.load()
    raw = np.frombuffer(b"ACGNNACGTNA", np.uint8)
    words = np.zeros(1, np.uint32)
    nr, nb = ctypes.c_int64(), ctypes.c_int64()
    # measuring call: every word written, counts returned, ETOOBIG
    rc = lib.gbsw_pack(0, raw.ctypes.data, raw.size, 1, words.ctypes.data, 0, None, None, 0, None,
                       ctypes.byref(nr), ctypes.byref(nb))
    assert rc == -7 and (nr.value, nb.value) == (2, 3)
    assert words[0] == built.pack(0, raw).words[0]
    at, off, by = np.zeros(2, np.int64), np.zeros(3, np.int64), np.zeros(2, np.uint8)
    rc = lib.gbsw_pack(0, raw.ctypes.data, raw.size, 1, words.ctypes.data, 2, at.ctypes.data, off.ctypes.data,
                       2, by.ctypes.data, ctypes.byref(nr), ctypes.byref(nb))
    assert rc == -7  # three bytes do not fit two
    by = np.zeros(3, np.uint8)
    rc = lib.gbsw_pack(0, raw.ctypes.data, raw.size, 1, words.ctypes.data, 2, at.ctypes.data, off.ctypes.data,
                       3, by.ctypes.data, ctypes.byref(nr), ctypes.byref(nb))
    assert rc == 0 and at.tolist() == [3, 9] and off.tolist() == [0, 2, 3] and bytes(by) == b"NNN"
    assert lib.gbsw_pack(2, raw.ctypes.data, raw.size, 1, words.ctypes.data, 0, None, None, 0, None,
                         ctypes.byref(nr), ctypes.byref(nb)) == -1
    assert lib.gbsw_pack(0, None, 5, 1, words.ctypes.data, 0, None, None, 0, None, ctypes.byref(nr),
                         ctypes.byref(nb)) == -1
    assert lib.gbsw_pack(0, raw.ctypes.data, raw.size, 1, words.ctypes.data, 4, None, None, 0, None,
                         ctypes.byref(nr), ctypes.byref(nb)) == -1
    assert lib.gbsw_packed_words(0, 33) == 3 and lib.gbsw_packed_words(1, 13) == 3
    assert lib.gbsw_packed_words(0, -1) == -1 and lib.gbsw_packed_words(5, 1) == -1
    assert lib.gbsw_unpack_device(0, None, None, None) == -1


def test_packed_batch_sizes(built, workloads):
    """The packed form of the 100,000-pair DNA throughput batch is a quarter of
    its sequence bytes (no escapes in A/C/G/T sequences)."""
    b = workloads.dna_throughput(2000, seed=2)
    pr, pq = built.pack(0, b.ref), built.pack(0, b.query)
    assert pr.nruns == pq.nruns == 0
    assert pr.nbytes <= b.ref.size // 4 + 4 and pq.nbytes <= b.query.size // 4 + 4
    assert np.array_equal(unpack_np(pr), b.ref) and np.array_equal(unpack_np(pq), b.query)
