"""GPU test of gbsw_align_device_noalloc, the entry point for callers that must not
allocate GPU memory (code inside another framework's memory pool or caching
allocator, or running against a fixed device-memory budget).

Through the C ABI, its results must equal those of the existing device entry
(gbsw_align_device) on the same inputs -- bit for bit, as every result here is an
integer -- on two calls in a row: the second call runs on the scratch array the
first one left behind.  This file is collected last so that a run stopping at the
first failure has run every other test already.
"""
import ctypes
import importlib
import json
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _to_dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).to("cuda:0")


def _batches(wl, gbsw):
    # DNA: A/C/G/T pairs (profile kernels) mixed with raw-byte pairs (N, lower case)
    dna = wl.PairBatch.concat([
        wl.dna_throughput(2500, seed=41),
        wl.PairBatch.from_strings(0, ["ACGTNNACGTacgt" * 20, "NNNNACGT" * 30, "A" * 900],
                                  ["CGTNNACG" * 9, "ACGTNNNN" * 12, "A" * 700]),
        wl.mixed_dna(60, seed=42),
    ])
    prot = wl.protein(800, seed=43)
    return [
        (dna, gbsw.make_scoring(gbsw.DNA, scores=(3, -3, -6, -1))),
        (prot, gbsw.make_scoring(gbsw.PROTEIN, matrix=gbsw.scoring.BLOSUM62, gaps=(-6, -1))),
    ]


def test_noalloc_entry_matches_device_entry_on_two_calls():
    torch = pytest.importorskip("torch")
    importlib.import_module("gpu-bsw_gb300.build").build_all()
    gbsw = importlib.import_module("gpu-bsw_gb300")
    wl = importlib.import_module("gpu-bsw_gb300.workloads")
    lib = gbsw.load()
    aligner = gbsw.Aligner(0)
    for batch, sc in _batches(wl, gbsw):
        n = batch.n
        max_len = int(max(batch.ref_lengths().max(), batch.query_lengths().max()))
        assert n <= 65536 and max_len <= 8192
        ref, qry = _to_dev(torch, batch.ref), _to_dev(torch, batch.query)
        ro, qo = _to_dev(torch, batch.ref_off), _to_dev(torch, batch.query_off)
        expected = torch.full((5, n), -9, dtype=torch.int32, device="cuda:0")
        aligner.align_device(sc, ref.data_ptr(), ro.data_ptr(), qry.data_ptr(), qo.data_ptr(), n, max_len,
                             *[expected[k].data_ptr() for k in range(5)], None)
        aligner.check(None)
        exp = expected.cpu().numpy()
        for call in range(2):
            got = torch.full((5, n), -9, dtype=torch.int32, device="cuda:0")
            rc = lib.gbsw_align_device_noalloc(ctypes.byref(sc), ref.data_ptr(), ro.data_ptr(),
                                               qry.data_ptr(), qo.data_ptr(), n, max_len,
                                               *[got[k].data_ptr() for k in range(5)], None)
            assert rc == 0, lib.gbsw_strerror(rc)
            g = got.cpu().numpy()
            bad = np.nonzero(np.any(g != exp, axis=0))[0]
            assert len(bad) == 0, (call, bad[:5], g[:, bad[:3]].T, exp[:, bad[:3]].T)
    aligner.close()


def test_noalloc_entry_rejects_batches_beyond_its_scratch():
    gbsw = importlib.import_module("gpu-bsw_gb300")
    importlib.import_module("gpu-bsw_gb300.build").build_all()
    lib = gbsw.load()
    sc = gbsw.make_scoring(gbsw.DNA, scores=(3, -3, -6, -1))
    # NULL buffers: the size check comes first and reports GBSW_ETOOBIG; were it
    # to regress, the NULL check would refuse the call before any launch
    rc = lib.gbsw_align_device_noalloc(ctypes.byref(sc), None, None, None, None, 65537, 100,
                                       None, None, None, None, None, None)
    assert rc == -7 and b"fixed scratch" in lib.gbsw_strerror(rc)
    rc = lib.gbsw_align_device_noalloc(ctypes.byref(sc), None, None, None, None, 10, 8193,
                                       None, None, None, None, None, None)
    assert rc == -7


# Run in a fresh process with lazy module loading (CUDA's default): the n = 0
# call must load the scratch array onto the device, the second must add nothing.
_COMMIT_PROBE = r"""
import ctypes, importlib, json, sys
sys.path.insert(0, sys.argv[1])
import torch
gbsw = importlib.import_module("gpu-bsw_gb300")
lib = gbsw.load()
torch.cuda.set_device(0)
torch.cuda.synchronize()
sc = gbsw.make_scoring(gbsw.DNA, scores=(3, -3, -6, -1))
free = [torch.cuda.mem_get_info(0)[0]]
rcs = []
for _ in range(2):
    rcs.append(lib.gbsw_align_device_noalloc(ctypes.byref(sc), None, None, None, None, 0, 0,
                                             None, None, None, None, None, None))
    torch.cuda.synchronize()
    free.append(torch.cuda.mem_get_info(0)[0])
print(json.dumps({"rcs": rcs, "free": free}))
"""


def test_noalloc_first_call_commits_the_scratch_array():
    importlib.import_module("gpu-bsw_gb300.build").build_all()
    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, CUDA_MODULE_LOADING="LAZY")
    r = subprocess.run([sys.executable, "-c", _COMMIT_PROBE, repo], capture_output=True, text=True, env=env,
                       timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    out = json.loads(r.stdout.strip().splitlines()[-1])
    assert out["rcs"] == [0, 0]
    free = out["free"]
    assert free[0] - free[1] >= 64 << 20, free  # the 64 MiB array is now on the device
    assert abs(free[1] - free[2]) < 2 << 20, free  # and the next call commits nothing more
