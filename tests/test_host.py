"""CPU tests of the host side: the C ABI library loads and exports what the headers
declare, the synthetic workloads, and the input validation that runs before any
GPU work."""
import ctypes
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared(header):
    text = open(os.path.join(REPO, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gbsw_\w+)\s*\(", text)))


def test_library_exports_every_declared_symbol(built):
    lib = built.load()
    declared = _declared("gbsw.h")
    assert declared, "no declarations parsed"
    missing = [s for s in declared if not hasattr(lib, s)]
    assert not missing
    assert sorted(built.EXPORTS) == declared


def test_ctypes_structs_match_the_header(built, tmp_path):
    """Every struct of gbsw.h has the size and field offsets its Python mirror
    assumes (compiled here with the host C compiler)."""
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    mirrors = {"gbsw_scoring": built._Scoring, "gbsw_options": built._Options,
               "gbsw_calibration": built._Calibration, "gbsw_stats": built._Stats,
               "gbsw_server_options": built._ServerOptions, "gbsw_job_info": built._JobInfo,
               "gbsw_server_stats": built._ServerStats, "gbsw_variant": built._Variant,
               "gbsw_tuning": built._Tuning, "gbsw_tune_report": built._TuneReport, "gbsw_packed": built._Packed}
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "gbsw.h"', "int main(void) {"]
    for c_name, py in mirrors.items():
        lines.append('printf("%s %%zu\\n", sizeof(%s));' % (c_name, c_name))
        for field, _ in py._fields_:
            lines.append('printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (c_name, field, c_name, field))
    lines += ["return 0;", "}"]
    src = tmp_path / "sizes.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "sizes"
    subprocess.run([cc, "-I", os.path.join(REPO, "include"), str(src), "-o", str(exe)], check=True)
    got = dict(line.split() for line in subprocess.run([str(exe)], stdout=subprocess.PIPE, text=True,
                                                        check=True).stdout.splitlines())
    for c_name, py in mirrors.items():
        assert int(got[c_name]) == ctypes.sizeof(py), c_name
        for field, _ in py._fields_:
            assert int(got["%s.%s" % (c_name, field)]) == getattr(py, field).offset, (c_name, field)


def test_cpp_dropin_symbols_exported(built):
    nm = shutil.which("nm")
    if not nm:
        pytest.skip("nm not available")
    out = subprocess.run([nm, "-D", "-C", "--defined-only", built.lib_path()], stdout=subprocess.PIPE,
                         text=True).stdout
    for sym in ["gpu_bsw_driver::kernel_driver_dna", "gpu_bsw_driver::kernel_driver_aa",
                "gpu_bsw_driver::get_tot_gpu_mem", "free_alignments"]:
        assert sym in out, sym


def test_synth_library_exports(workloads):
    lib = ctypes.CDLL(workloads.SYNTH_LIB)
    for s in re.findall(r"\b(gbsw_synth_\w+)\s*\(", open(os.path.join(REPO, "include", "gbsw_synth.h")).read()):
        assert hasattr(lib, s)


def test_strerror_without_gpu(built):
    lib = built.load()
    assert lib.gbsw_strerror(0) == b"ok"
    assert lib.gbsw_strerror(-2).startswith(b"protein symbol")


def test_synth_deterministic_and_in_bounds(workloads):
    a = workloads.plain_dna(200, seed=5)
    b = workloads.plain_dna(200, seed=5)
    c = workloads.plain_dna(200, seed=6)
    assert np.array_equal(a.ref, b.ref) and np.array_equal(a.query_off, b.query_off)
    assert not np.array_equal(a.ref[:100], c.ref[:100])
    rl = a.ref_lengths()
    assert rl.min() >= 200 and rl.max() <= 500
    assert set(np.unique(a.ref).tolist()) <= set(b"ACGT")


def test_synth_presets_shapes(workloads):
    t = workloads.dna_throughput(2000, seed=2)
    assert t.ref_lengths().min() >= 400 and t.ref_lengths().max() <= 1024
    p = workloads.protein(500, seed=3)
    assert p.ref_lengths().min() >= 50 and p.ref_lengths().max() <= 1000
    assert set(np.unique(p.ref).tolist()) <= set(b"ARNDCQEGHILKMFPSTWYV")
    m = workloads.mixed_dna(2000, seed=4)
    long_ = m.ref_lengths() >= 1500
    assert 0.25 < long_.mean() < 0.35
    assert m.query_lengths()[~long_].max() <= 160


def test_pairbatch_subset_and_concat(workloads):
    a = workloads.plain_dna(50, seed=9)
    s = a.subset([3, 1, 7])
    for k, src in enumerate([3, 1, 7]):
        assert s.strings(k) == a.strings(src)
    cat = workloads.PairBatch.concat([s, s])
    assert cat.n == 6 and cat.strings(4) == a.strings(1)


def test_shard_ranges_balance_cells():
    import importlib
    shard = importlib.import_module("gpu-bsw_gb300.shard")
    cells = np.array([100, 1, 1, 1, 50, 50, 300, 2, 2, 2], dtype=np.int64)
    for world in (1, 2, 3, 4):
        rs = shard.shard_ranges(cells, world)
        assert rs[0][0] == 0 and rs[-1][1] == len(cells)
        assert all(rs[k][1] == rs[k + 1][0] for k in range(len(rs) - 1))
    r2 = shard.shard_ranges(cells, 2)
    loads = [cells[a:b].sum() for a, b in r2]
    assert max(loads) <= cells.sum() * 0.5 + cells.max()


def test_server_api_without_gpu(built):
    """Argument checks of the serving loop, and a clean refusal (no hang, no
    leaked worker threads) when no device can be opened."""
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("covered by the GPU server tests")
    lib = built.load()
    h = ctypes.c_void_p()
    assert lib.gbsw_server_create(None, None) == -1
    bad = built._ServerOptions(0, 0, 1 << 30, 100)
    assert lib.gbsw_server_create(ctypes.byref(bad), ctypes.byref(h)) == -1
    rc = lib.gbsw_server_create(ctypes.byref(built._ServerOptions(0, 3, 1 << 30, 100)), ctypes.byref(h))
    assert rc == -4 and not h.value
    with pytest.raises(built.GbswError):
        built.Server(0, slots=2)
    jid = ctypes.c_uint64()
    sc = built.make_scoring(built.DNA, scores=(3, -3, -6, -1))
    off = np.zeros(2, np.int64)
    assert lib.gbsw_server_submit(None, ctypes.byref(sc), None, off.ctypes.data, None, off.ctypes.data, 1,
                                  None, ctypes.byref(jid)) == -1
    assert lib.gbsw_server_submit_packed(None, ctypes.byref(sc), None, off.ctypes.data, None, off.ctypes.data, 1,
                                         None, ctypes.byref(jid)) == -1
    assert lib.gbsw_server_wait(None, 1, 0.0, None) == -1
    assert lib.gbsw_server_get_stats(None, None) == -1
    assert lib.gbsw_server_reset_stats(None) == -1
    lib.gbsw_server_destroy(None)
