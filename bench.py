#!/usr/bin/env python3
"""GCUPS of the batched Smith-Waterman path on GB300.

One step = the forward (end) and reverse (begin) passes over one batch of the
DNA throughput workload: 100,000 synthetic pairs, references U[400,1024] bp,
queries U[150,300] bp (80% mutated substrings of their reference with 5%
substitutions and 1% indel events, 20% unrelated), scoring +3/-3/-6/-1.
Cells are forward cells, sum |ref|*|query| (the reference's "Total Cells").
``--workload`` selects one of the other synthetic batches as the headline
instead (plain_dna, protein, mixed_dna).

value   : GCUPS with the inputs resident in HBM (gbsw_align_device), CUDA events
          around each step on the launching stream, L2 flushed between steps.
e2e     : GCUPS through the host-buffer C ABI call on packed inputs
          (gbsw_align_packed_host16): the batch packed once (2 bits a base, 5 bits
          a residue) in pinned host memory, copied in, unpacked on the device,
          int16 results copied out, per step; ``pack_ms`` is the host packing time
          for a caller that starts from raw bytes.  ``e2e_raw``: the same through
          gbsw_align_host16 on raw pinned bytes (the drop-in's form).
roofline: the forward pass kernel against the integer-pipe peak measured by the
          calibration probe (gbsw_calibrate): cells per second of the kernel's own
          cell block from registers, every SM busy, timed with CUDA events.
cpu_baseline: the CPU oracle (oracle/gotoh.c, OpenMP, every host thread) over the
          whole headline batch, timed.  Its results are also the parity check of
          the GPU results: every pair of the timed device step and of the
          end-to-end call (``parity``).
workloads: the other configurations, each timed on the device (and the mixed
          batch end to end), with its roofline and every pair checked against the
          oracle, whose timed run is that workload's CPU baseline:
          mixed_dna (200,000 pairs, 30% of them 1-4 kb), protein (30,000),
          plain_dna (1,000), long_dna (400 pairs of 4-16 kb, beyond the reference's
          1,024 limit; block-per-pair passes).
reference_cuda: the reference's own CUDA build (its driver and kernels compiled
          for sm_103a from its sources, oracle/build_ref.sh) on the same GPU, on
          the headline batch, the reference-runnable short bin of the mixed batch
          (140,000 pairs), the protein and the plain batch: its end-to-end call
          time and the kernel time of its own launches, against this library's
          end-to-end call and device step on the same pairs, and the pairs whose
          results differ.
serving : the serving loop (gbsw_server_*) under Poisson job arrivals: peak
          closed-loop GCUPS of the job mix, then p50/p99 job latency and
          sustained GCUPS at 20-100% of that peak (``--serve-only`` prints just
          this part).
traceback: one path per pair of the headline batch (gbsw_traceback_host, host
          buffers in and out), time and run-length operations.

``--impl reference`` times the reference's algorithm on the host cores instead:
the reference has no CPU implementation of its own, so this is the CPU oracle
restating it (kind "port"), with every host thread, on a bounded sample.

Multi-GPU (torchrun, N > 1): one batch of N x 100,000 pairs is split into N
contiguous, cell-balanced shards (shard.shard_ranges), one per rank (weak
scaling: per-GPU work stays fixed as N grows); ranks share only a barrier, the
sum of their cells and the max of their step times.
"""
import argparse
import gc
import importlib
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "oracle"))

WORKLOAD = "dna_throughput"
SCORES = (3, -3, -6, -1)
AA_GAPS = (-6, -1)
# DRAM bytes (read + write) of one forward launch, from an ncu capture of this
# workload (dram__bytes_read.sum + dram__bytes_write.sum); the algorithmic input
# is the sequences and offsets, about 95 MB for the default batch
TRAFFIC = {"dna_throughput": 430.4e6 + 542.2e6, "protein": 21.5e6 + 1.1e6}
# workload -> (pairs, seed, kind, description); the default is the headline batch
WORKLOADS = {
    "dna_throughput": (100_000, 2, "dna", "refs U[400,1024] bp, queries U[150,300] bp, 80% mutated substrings"),
    "plain_dna": (1_000, 1, "dna", "refs U[200,500] bp, queries mutated U[100,150] bp substrings"),
    "protein": (30_000, 3, "aa", "log-normal lengths (median 300, clipped 50-1000), 70% homologs at ~40% id"),
    "mixed_dna": (200_000, 4, "dna", "70% 100-150 bp vs 300 bp, 30% 1000-2048 bp vs 1500-4096 bp"),
    "mixed_dna_short": (140_000, 4, "dna", "the short bin of mixed_dna alone: 100-150 bp vs 300 bp"),
    "long_dna": (400, 7, "dna", "refs U[4000,16000] bp, queries U[3000,12000] bp, 80% mutated substrings"),
}
METRIC = "GCUPS on 1 GB300 (DNA, protein): batched vs plain path; p50/p99 serve latency"
CLOCK_QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
               "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
               "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=WORKLOAD, choices=sorted(WORKLOADS))
    ap.add_argument("--pairs", type=int, default=None, help="override the workload's pair count")
    ap.add_argument("--no-extra", action="store_true",
                    help="skip the side measurements (other workloads, reference, traceback, serving)")
    ap.add_argument("--serve-only", action="store_true", help="print only the serving sweep (JSON)")
    ap.add_argument("--skip-cpu", action="store_true",
                    help="skip the CPU oracle leg (cpu_baseline and parity), e.g. under a profiler")
    return ap.parse_args()


class ClockSampler:
    """nvidia-smi clock/throttle samples while the GPU works."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + CLOCK_QUERY,
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.1)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for ln in open(self.path):
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) >= 9 and parts[1].isdigit():
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [int(r[1]) for r in rows]
        smax = max(int(r[2]) for r in rows)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k] == "Active"})
        loaded = [v for v in sm if v >= 0.5 * smax] or sm
        return {"sm_mhz": float(statistics.median(loaded)), "sm_max_mhz": float(smax),
                "reasons": reasons, "samples": len(rows),
                "power_w_max": max(float(r[3]) for r in rows if r[3].replace(".", "", 1).isdigit())
                if any(r[3].replace(".", "", 1).isdigit() for r in rows) else None}


def oracle_run(batch, kind, threads):
    import oracle
    sc = importlib.import_module("gpu-bsw_gb300.scoring")
    if kind == "dna":
        return oracle.align(oracle.DNA, batch.ref, batch.ref_off, batch.query, batch.query_off,
                            scores=SCORES, nthreads=threads)
    return oracle.align(oracle.AA, batch.ref, batch.ref_off, batch.query, batch.query_off,
                        matrix=sc.BLOSUM62, encoding=sc.ENCODING, gaps=AA_GAPS, nthreads=threads)


def generate(name, n=None, seed_offset=0):
    wl = importlib.import_module("gpu-bsw_gb300.workloads")
    pairs, seed, kind, _ = WORKLOADS[name]
    return wl.PRESETS[name](n or pairs, seed=seed + seed_offset), kind


def make_batch(args, rank=0, world=1):
    """This rank's shard of one batch of world x pairs (cell-balanced, contiguous)."""
    shard = importlib.import_module("gpu-bsw_gb300.shard")
    pairs = args.pairs or WORKLOADS[args.workload][0]
    batch, kind = generate(args.workload, pairs * world)
    if world > 1:
        batch = shard.rank_slice(batch, rank, world)[2]
    return batch, kind


def cpu_sample(batch, seconds, threads, kind="dna"):
    """Oracle GCUPS on a prefix of the batch sized to take about `seconds`."""
    probe = batch.subset(np.arange(min(300, batch.n)))
    t = time.perf_counter()
    oracle_run(probe, kind, threads)
    rate = probe.cells() / max(time.perf_counter() - t, 1e-6)
    cells = batch.ref_lengths().astype(np.int64) * batch.query_lengths()
    want = rate * seconds
    k = int(np.searchsorted(np.cumsum(cells), want)) + 1
    k = max(300, min(k, batch.n))
    sample = batch.subset(np.arange(k))
    return sample


def time_cpu(sample, threads, kind="dna"):
    t = time.perf_counter()
    oracle_run(sample, kind, threads)
    return time.perf_counter() - t


def cpu_leg(batch, kind, threads):
    """The oracle over the whole batch on every host thread: (results, seconds)."""
    t = time.perf_counter()
    res = oracle_run(batch, kind, threads)
    return res, time.perf_counter() - t


def parity(name, batch, gpu_results, expected):
    """Pairs of each GPU result array that differ from the oracle's, in any of the five fields."""
    out = {"workload": name, "checked_pairs": int(batch.n), "reference": "CPU oracle (the reference's "
           "algorithm and tie rules restated, oracle/gotoh.c), every pair"}
    total = 0
    for label, got in gpu_results.items():
        bad = np.nonzero(np.any(np.asarray(got, dtype=np.int32) != expected, axis=1))[0]
        out[label + "_mismatches"] = int(len(bad))
        if len(bad):
            out[label + "_first_mismatches"] = [int(k) for k in bad[:5]]
        total += len(bad)
    out["mismatches"] = int(total)
    return out


def run_reference(args):
    """CPU arm: the reference's algorithm (restated by the oracle) on all host threads."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import oracle
    threads = oracle.threads()
    batch, kind = make_batch(args)
    sample = cpu_sample(batch, 4.0, threads, kind)
    for _ in range(args.warmup):
        time_cpu(sample.subset(np.arange(min(200, sample.n))), threads, kind)
    times = [time_cpu(sample, threads, kind) for _ in range(args.steps)]
    gcups = sample.cells() / statistics.mean(times) / 1e9
    line = {
        "metric": METRIC, "impl": "reference", "value": round(gcups, 4), "unit": "GCUPS",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(statistics.mean(times) * 1e3, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic",
        "config": {"workload": args.workload, "pairs_per_step": sample.n, "cells_per_step": sample.cells(),
                   "scoring": "+3/-3/-6/-1" if kind == "dna" else "BLOSUM62 -6/-1",
                   "seed": WORKLOADS[args.workload][1],
                   "note": "the reference ships only CUDA kernels; its algorithm is timed through the "
                           "CPU oracle that restates it (tie rules included)"},
        "cpu_baseline": {"value": round(gcups, 4), "unit": "GCUPS", "cores": threads, "kind": "port",
                         "sample": "first %d of the %d pairs (%d cells) of the %s batch, "
                                   "forward + reverse passes" % (sample.n, batch.n, sample.cells(), args.workload)},
        "e2e": {"value": round(gcups, 4), "unit": "GCUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def scoring_for(gbsw, kind):
    if kind == "dna":
        return gbsw.make_scoring(gbsw.DNA, scores=SCORES)
    return gbsw.make_scoring(gbsw.PROTEIN, matrix=gbsw.scoring.BLOSUM62, gaps=AA_GAPS)


class DeviceBatch:
    """One batch resident in HBM, aligned through gbsw_align_device on `stream`."""

    def __init__(self, torch, al, batch, sc, dev, stream):
        self.al, self.sc, self.stream, self.n = al, sc, stream, batch.n
        self.ref = torch.from_numpy(batch.ref).to(dev)
        self.qry = torch.from_numpy(batch.query).to(dev)
        self.ro = torch.from_numpy(batch.ref_off).to(dev)
        self.qo = torch.from_numpy(batch.query_off).to(dev)
        self.out = torch.empty((5, batch.n), dtype=torch.int32, device=dev)
        self.max_len = int(max(batch.ref_lengths().max(), batch.query_lengths().max()))

    def step(self):
        o = self.out
        self.al.align_device(self.sc, self.ref.data_ptr(), self.ro.data_ptr(), self.qry.data_ptr(),
                             self.qo.data_ptr(), self.n, self.max_len, o[0].data_ptr(), o[1].data_ptr(),
                             o[2].data_ptr(), o[3].data_ptr(), o[4].data_ptr(), self.stream.cuda_stream)

    def results(self):
        """(n, 5) int32: score, ref_begin, ref_end, query_begin, query_end."""
        return np.ascontiguousarray(self.out.cpu().numpy().T)


def time_device(torch, al, db, steps, warmup, flush, barrier=None):
    """CUDA-event time of `steps` device-resident steps, L2 flushed between them."""
    stream = db.stream
    for _ in range(warmup):
        db.step()
    al.check(stream.cuda_stream)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    fwd, rev = [], []
    if barrier:
        barrier()
    for k in range(steps):
        flush.zero_()  # L2 flush between steps (256 MiB > 129 MB L2), outside the step events
        starts[k].record(stream)
        db.step()
        ends[k].record(stream)
        st = al.stats()  # waits for this step's kernels; per-kernel event times on the same stream
        fwd.append(st["forward_ms"])
        rev.append(st["reverse_ms"])
    if barrier:
        barrier()
    torch.cuda.synchronize()
    al.check(stream.cuda_stream)
    st = al.stats()
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    return {"step_ms": step_ms, "ms": statistics.mean(step_ms), "best_ms": min(step_ms),
            "forward_ms": statistics.mean(fwd), "reverse_ms": statistics.mean(rev),
            "launches": st["launches"], "lane_group": st["lane_group"], "dual": st["dual"],
            "plans": plans_of(st)}


def plans_of(st):
    """The plan each length bin ran with (gbsw_stats): pairs, dual int16x2 or int32,
    lanes per group, and whether the tuning table chose it."""
    return [{"bin": "shorter side < 512" if b == 0 else "shorter side >= 512", "pairs": st["bin_pairs"][b],
             "variant": ("dual%d" if st["bin_dual"][b] else "int32_%d") % st["bin_lanes"][b],
             "reverse_variant": ("dual%d" if st["rev_dual"][b] else "int32_%d") % st["rev_lanes"][b],
             "from_table": bool(st["bin_tuned"][b])} for b in range(2)]


def tuning_report(torch, gbsw, device, batch, sc, dev):
    """gbsw_tune_device on this batch, on a context of its own (the timed contexts
    keep the committed table): every candidate variant's forward + reverse kernel
    time per length bin and pass, and the bin's fastest in each pass."""
    al = gbsw.Aligner(device)
    d = [torch.from_numpy(x).to(dev) for x in (batch.ref, batch.ref_off, batch.query, batch.query_off)]
    ml = int(max(batch.ref_lengths().max(), batch.query_lengths().max()))
    rep = al.tune_device(sc, d[0].data_ptr(), d[1].data_ptr(), d[2].data_ptr(), d[3].data_ptr(), batch.n, ml, reps=2)
    al.close()
    names = [("dual%d" if c[0] else "int32_%d") % c[1] for c in rep["candidates"]]
    def name(v):
        return names[rep["candidates"].index(v)] if v else None
    return [{"bin": "shorter side < 512" if b == 0 else "shorter side >= 512", "pairs": info["pairs"],
             "bucket": info["bucket"], "chosen_forward": name(info["chosen"]),
             "chosen_reverse": name(info["chosen_reverse"]),
             "ms_forward": {n: round(v, 3) for n, v in zip(names, info["ms_forward"])} if info["pairs"] > 0 else None,
             "ms_reverse": {n: round(v, 3) for n, v in zip(names, info["ms_reverse"])} if info["pairs"] > 0 else None}
            for b, info in enumerate(rep["bins"])]


def pinned(torch, batch):
    pin = lambda a: torch.from_numpy(a).pin_memory().numpy()  # noqa: E731
    return pin(batch.ref), pin(batch.ref_off), pin(batch.query), pin(batch.query_off)


def pinned_packed(torch, gbsw, batch, kind, reps=3):
    """The batch's sequences packed (gbsw_pack: 2-bit DNA / 5-bit protein) into
    page-locked words, with page-locked offsets; and the packing time (best of
    ``reps``, every host thread) for a caller that starts from raw bytes."""
    k = gbsw.DNA if kind == "dna" else gbsw.PROTEIN
    lib = gbsw.load()
    keep, streams, best = [], [], None
    for buf in (batch.ref, batch.query):
        w = torch.empty(max(int(lib.gbsw_packed_words(k, buf.size)), 1), dtype=torch.int32).pin_memory()
        keep.append(w)
        streams.append(gbsw.pack(k, buf, out=w.numpy().view(np.uint32)))
    for _ in range(reps):
        t0 = time.perf_counter()
        for buf, w in zip((batch.ref, batch.query), keep):
            gbsw.pack(k, buf, out=w.numpy().view(np.uint32))
        dt = time.perf_counter() - t0
        best = dt if best is None else min(best, dt)
    pin = lambda a: torch.from_numpy(a).pin_memory().numpy()  # noqa: E731
    return (streams[0], pin(batch.ref_off), streams[1], pin(batch.query_off), keep), best


def time_e2e(al, sc, host, steps, warmup, barrier=None, packed=False):
    """Wall time of gbsw_align_host16 on pinned raw host buffers, or (packed) of
    gbsw_align_packed_host16 on pinned packed streams; copies in and out included."""
    h_ref, h_ro, h_qry, h_qo = host[:4]
    call = al.align_packed if packed else al.align_host
    r16 = None
    for _ in range(warmup):
        r16 = call(sc, h_ref, h_ro, h_qry, h_qo, int16=True)
    if barrier:
        barrier()
    t = []
    for _ in range(steps):
        t0 = time.perf_counter()
        r16 = call(sc, h_ref, h_ro, h_qry, h_qo, int16=True)
        t.append(time.perf_counter() - t0)
    if barrier:
        barrier()
    return t, r16


def roofline(cells, fwd_ms, dual, lane_group, calib, mhz, traffic=None):
    """Forward pass against the integer-pipe peaks (calibrated and nominal).

    Pairs whose scores fit int16 run two per group in the dual-pair int16x2
    kernel: its roofline is the calibrated throughput of the DNA dual cell block
    (the protein variant's cell adds one shared-memory profile load per row).
    Everything else runs an int32 kernel, measured against the int32 pass's cell
    block.  Both are cells per second of a register-only probe of the kernel's
    own cell ops with every SM busy, timed with CUDA events.  Nominal: a cell
    pair of the dual kernel is 6.5 int16x2 ops, all on the integer ALU pipe,
    which takes a warp instruction every other cycle per SM sub-partition (64
    lane-ops per clock per SM); an int32 cell is 6.5 ops, some of which issue to
    other pipes, so its bound is the issue rate (128 lane-ops per clock per SM)."""
    peak_cal = calib["cell_dual_gcups"] if dual else calib["cell_int32_gcups"]
    ops_per_cell = 3.25 if dual else 6.5
    lane_ops = 64 if dual else 128
    peak_nom = calib["sms"] * lane_ops * mhz * 1e6 / ops_per_cell / 1e9
    achieved = cells / (fwd_ms / 1e3) / 1e9
    return {"bound": "int", "unit": "GCUPS", "achieved": round(achieved, 2),
            "peak": round(peak_cal, 2), "frac": round(achieved / peak_cal, 4), "traffic": traffic,
            "kernel": "forward pass (%s)" % ("sw_pass_dual, int16x2, 2 pairs per %d-lane group" % lane_group
                                             if dual else "sw_pass, int32, %d lanes per pair" % lane_group),
            "peak_source": "measured: gbsw_calibrate register-only probe of the kernel's own cell "
                           "block, %d SMs busy, timed with CUDA events (HBM and bf16 peaks do not "
                           "bound this integer path)" % calib["sms"],
            "nominal_peak": round(peak_nom, 2), "nominal_frac": round(achieved / peak_nom, 4),
            "nominal_source": "%d lane-ops/clk/SM (%s) x %d SMs x %.0f MHz / %.2f ops per cell"
                              % (lane_ops, "ALU pipe" if dual else "issue", calib["sms"], mhz, ops_per_cell)}


def side_workloads(torch, gbsw, al, dev, stream, flush, calib, mhz, threads, check=True):
    """The other configurations: device time, roofline, end to end (mixed), and
    every pair against the oracle, whose timed run is the workload's CPU baseline."""
    out = {}
    for name, steps, e2e_steps in (("mixed_dna", 3, 2), ("protein", 5, 0), ("plain_dna", 5, 0), ("long_dna", 3, 0)):
        batch, kind = generate(name)
        sc = scoring_for(gbsw, kind)
        db = DeviceBatch(torch, al, batch, sc, dev, stream)
        t = time_device(torch, al, db, steps, 2, flush)
        res = db.results()
        del db
        cells = batch.cells()
        leg = {"pairs": batch.n, "cells": cells, "shape": WORKLOADS[name][3],
               "scoring": "+3/-3/-6/-1" if kind == "dna" else "BLOSUM62 -6/-1", "seed": WORKLOADS[name][1],
               "value": round(cells / (t["ms"] / 1e3) / 1e9, 2), "unit": "GCUPS", "ms_per_step": round(t["ms"], 3),
               "steps": steps, "passes_ms": {"forward": round(t["forward_ms"], 3),
                                             "reverse": round(t["reverse_ms"], 3)},
               "launches_per_step": t["launches"], "lane_group": t["lane_group"], "dual": t["dual"],
               "plans": t["plans"],
               "roofline": roofline(cells, t["forward_ms"], t["dual"] == 1, t["lane_group"], calib, mhz,
                                    TRAFFIC.get(name))}
        gpu = {"device_int32": res}
        if e2e_steps:
            hpack, pack_s = pinned_packed(torch, gbsw, batch, kind, reps=1)
            et, r16p = time_e2e(al, sc, hpack, e2e_steps, 1, packed=True)
            h2d = int(hpack[0].nbytes + hpack[2].nbytes + batch.ref_off.nbytes + batch.query_off.nbytes)
            del hpack
            host = pinned(torch, batch)
            rt, r16 = time_e2e(al, sc, host, e2e_steps, 1)
            del host
            leg["e2e"] = {"value": round(cells / statistics.mean(et) / 1e9, 2), "unit": "GCUPS",
                          "ms_per_step": round(statistics.mean(et) * 1e3, 3), "call": "gbsw_align_packed_host16",
                          "h2d_bytes_per_step": h2d, "pack_ms": round(pack_s * 1e3, 3)}
            leg["e2e_raw"] = {"value": round(cells / statistics.mean(rt) / 1e9, 2), "unit": "GCUPS",
                              "ms_per_step": round(statistics.mean(rt) * 1e3, 3), "call": "gbsw_align_host16"}
            gpu["e2e_packed_int16"] = r16p
            gpu["e2e_raw_int16"] = r16
        torch.cuda.empty_cache()
        out[name] = leg
        if not check:
            continue
        expected, cpu_s = cpu_leg(batch, kind, threads)
        leg["cpu_baseline"] = {"value": round(cells / cpu_s / 1e9, 4), "unit": "GCUPS", "cores": threads,
                               "kind": "port", "sample": "all %d pairs (%d cells), forward + reverse"
                                                         % (batch.n, cells)}
        leg["parity"] = parity(name, batch, gpu, expected)
    return out


def reference_cuda_legs(torch, gbsw, al, dev, stream, flush):
    """The reference's own CUDA build against this library on the same GPU and pairs."""
    import ref_cuda
    if not os.path.exists(ref_cuda.HARNESS) and not ref_cuda.build():
        return {"unavailable": "the reference's sources are not present (oracle/build_ref.sh found none)"}
    out = {"how": "reference: its kernel_driver_dna/aa compiled for sm_103a from its own sources, called by "
                  "oracle/ref_harness.cpp (fastest of 3 calls; kernel time = union of its own launches, "
                  "bracketed by events through a link-time wrapper of the runtime's launch entry). "
                  "ours: gbsw_align_host16 on concatenated pinned raw buffers (e2e), the same harness source built "
                  "against gpu_bsw/driver.hpp (dropin, identical scope to the reference's call), and the "
                  "device-resident step (kernel), fastest of 3 each."}
    for name in ("dna_throughput", "mixed_dna_short", "protein", "plain_dna"):
        batch, kind = generate(name)
        if not ref_cuda.reference_safe(batch):
            out[name] = {"skipped": "outside the reference's limits"}
            continue
        sc = scoring_for(gbsw, kind)
        runs = ref_cuda.run_pair(batch, kind, reps=3, scores=SCORES, matrix=gbsw.scoring.BLOSUM62, gaps=AA_GAPS,
                                 lib_path=gbsw.lib_path())
        ref, dropin = runs["reference"], runs["dropin"]
        db = DeviceBatch(torch, al, batch, sc, dev, stream)
        t = time_device(torch, al, db, 3, 2, flush)
        del db
        host = pinned(torch, batch)
        et, r16 = time_e2e(al, sc, host, 3, 1)
        del host
        torch.cuda.empty_cache()
        cells = batch.cells()
        ours_e2e, ours_kernel = min(et), t["best_ms"] / 1e3
        leg = {"pairs": batch.n, "cells": cells,
               "reference_e2e_ms": round(ref["seconds"] * 1e3, 3),
               "reference_kernel_ms": round(ref["kernel_seconds"] * 1e3, 3),
               "reference_launches": ref["launches"],
               "reference_e2e_gcups": round(cells / ref["seconds"] / 1e9, 2),
               "reference_kernel_gcups": round(cells / ref["kernel_seconds"] / 1e9, 2)
               if ref["kernel_seconds"] > 0 else None,
               "ours_e2e_ms": round(ours_e2e * 1e3, 3), "ours_dropin_ms": round(dropin["seconds"] * 1e3, 3),
               "ours_kernel_ms": round(ours_kernel * 1e3, 3),
               "e2e_ratio": round(ref["seconds"] / ours_e2e, 2),
               "dropin_ratio": round(ref["seconds"] / dropin["seconds"], 2),
               "kernel_ratio": round(ref["kernel_seconds"] / ours_kernel, 2) if ref["kernel_seconds"] > 0 else None,
               "pairs_differing_from_reference": int(np.count_nonzero(
                   np.any(r16.astype(np.int32) != ref["results"], axis=1))),
               "dropin_pairs_differing_from_reference": int(np.count_nonzero(
                   np.any(dropin["results"] != ref["results"], axis=1)))}
        out[name] = leg
    return out


def serving_sweep(gbsw, wl, device, loads=(0.2, 0.4, 0.6, 0.8, 0.9, 1.0), seconds=2.5, pool=120, seed=5):
    """Serving stream through gbsw_server_*: Poisson arrivals of jobs of U[1,5000]
    pairs (60% dna_throughput pairs, 40% protein pairs), submitted with host
    buffers.  The peak is the closed-loop throughput of the same job mix (the
    whole pool submitted at once); each load point offers that fraction of it for
    `seconds` and reports job latency (submit -> results in host memory)."""
    jobs = wl.serving_jobs(pool, seed=seed)
    sc = {wl.DNA: gbsw.make_scoring(gbsw.DNA, scores=SCORES),
          wl.PROTEIN: gbsw.make_scoring(gbsw.PROTEIN, matrix=gbsw.scoring.BLOSUM62, gaps=AA_GAPS)}
    job_cells = np.array([b.cells() for _, b in jobs], dtype=np.float64)
    opts = {"slots": 4, "hbm_budget": 16 << 30, "max_batch_pairs": 50_000}
    srv = gbsw.Server(device, **opts)
    try:
        for _ in range(2):  # warm-up: staging and job buffers reach their size
            for h in [srv.submit_batch(b, sc[k]) for _ in range(2) for k, b in jobs]:
                h.wait()
        peaks = []
        for _ in range(3):  # closed loop: the whole pool at once, twice; median of three
            t0 = time.perf_counter()
            for h in [srv.submit_batch(b, sc[k]) for _ in range(2) for k, b in jobs]:
                h.wait()
            peaks.append(2 * job_cells.sum() / (time.perf_counter() - t0) / 1e9)
        peak = statistics.median(peaks)

        def measure(load, attempt):
            rng = np.random.default_rng(seed * 1000 + int(load * 100) + 7919 * attempt)
            rate = load * peak * 1e9 / job_cells.mean()  # jobs per second
            count = max(40, int(rate * seconds))
            gaps = rng.exponential(1.0 / rate, count)
            picks = rng.integers(0, len(jobs), count)
            srv.reset_stats()
            handles = []
            late, worst = 0, 0.0
            gc.disable()  # no collector pauses inside the arrival schedule
            try:
                t_next = t0 = time.perf_counter()
                for g, p in zip(gaps, picks):
                    t_next += g
                    now = time.perf_counter()
                    if t_next - now > 2e-4:
                        time.sleep(t_next - now - 1e-4)
                    while time.perf_counter() < t_next:
                        pass
                    lag = time.perf_counter() - t_next
                    worst = max(worst, lag)
                    late += lag > 1e-3
                    k, b = jobs[p]
                    handles.append(srv.submit_batch(b, sc[k]))
                span = time.perf_counter() - t0
            finally:
                gc.enable()
            for h in handles:
                h.wait()
            st = srv.stats()
            return {"load": load, "offered_gcups": round(load * peak, 1),
                    "sustained_gcups": round(st["gcups"], 1), "jobs": st["jobs"],
                    "batches": st["batches"], "peak_running": st["peak_running"],
                    "p50_ms": round(st["p50_ms"], 3), "p99_ms": round(st["p99_ms"], 3),
                    "max_ms": round(st["max_ms"], 3),
                    "submitted_late_1ms": int(late), "worst_submit_lag_ms": round(worst * 1e3, 3),
                    "arrival_span_s": round(span, 3)}

        points = []
        for load in loads:
            pt = measure(load, 0)
            if pt["worst_submit_lag_ms"] > 5.0:
                # the load generator itself stalled (host scheduling): jobs then
                # arrive in a burst that the offered load does not describe, so
                # the point is measured once more and the stall is recorded
                stalled = pt["worst_submit_lag_ms"]
                pt = measure(load, 1)
                pt["remeasured_after_submit_stall_ms"] = stalled
            points.append(pt)
    finally:
        srv.close()
    at80 = next(p for p in points if abs(p["load"] - 0.8) < 1e-9)
    # the batch rate of the same mix: the pool's pairs as two plain batches (every
    # DNA job's pairs, every protein job's pairs) through the host-buffer entry,
    # host buffers in and out like the jobs; the yardstick of the serving peak
    al = gbsw.Aligner(device)
    t_total, cells_total = 0.0, 0.0
    for kind in (wl.DNA, wl.PROTEIN):
        parts = [b for k, b in jobs if k == kind]
        if not parts:
            continue
        big = wl.PairBatch.concat(parts)
        al.align_host(sc[kind], big.ref, big.ref_off, big.query, big.query_off)  # warm-up
        ts = []
        for _ in range(3):
            t0 = time.perf_counter()
            al.align_host(sc[kind], big.ref, big.ref_off, big.query, big.query_off)
            ts.append(time.perf_counter() - t0)
        t_total += min(ts)
        cells_total += big.cells()
    al.close()
    batch_rate = cells_total / t_total / 1e9
    return {"workload": "Poisson jobs of U[1,5000] pairs, 60% dna_throughput / 40% protein pairs, "
                        "host buffers in and out",
            "server": opts, "pool_jobs": pool, "mean_job_cells": int(job_cells.mean()),
            "peak_gcups": round(peak, 1), "peak_runs_gcups": [round(v, 1) for v in peaks],
            "batch_same_mix_gcups": round(batch_rate, 1), "peak_over_batch": round(peak / batch_rate, 3),
            "at_80pct": {"p50_ms": at80["p50_ms"], "p99_ms": at80["p99_ms"],
                         "sustained_gcups": at80["sustained_gcups"]},
            "points": points}


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    build = importlib.import_module("gpu-bsw_gb300.build")
    build.build_all()
    gbsw = importlib.import_module("gpu-bsw_gb300")
    wl = importlib.import_module("gpu-bsw_gb300.workloads")
    import oracle

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    def over_ranks(v, op):
        if dist is None:
            return v
        t = torch.tensor([v], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=op)
        return float(t.item())

    if args.serve_only:
        print(json.dumps(serving_sweep(gbsw, wl, local)), flush=True)
        return
    dev = torch.device("cuda", local)
    batch, kind = make_batch(args, rank, world)
    cells = batch.cells()
    sc = scoring_for(gbsw, kind)
    al = gbsw.Aligner(local)
    calib = gbsw.calibrate(local)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.Stream(dev)  # the passes and the step events share this stream
    torch.cuda.set_stream(stream)
    torch.cuda.synchronize()

    # ---- device-resident timing (value) ----
    try:
        uuid = str(torch.cuda.get_device_properties(local).uuid)
        smi_id = uuid if uuid.startswith("GPU-") else "GPU-" + uuid
    except Exception:
        smi_id = os.environ.get("CUDA_VISIBLE_DEVICES", str(local)).split(",")[local]
    sampler = ClockSampler(smi_id)
    sampler.start()
    db = DeviceBatch(torch, al, batch, sc, dev, stream)
    t = time_device(torch, al, db, args.steps, args.warmup, flush, barrier)
    res_dev = db.results()  # the last timed step's results
    del db
    ms = over_ranks(t["ms"], dist.ReduceOp.MAX if dist else None)

    # ---- end to end through the host-buffer C ABI: packed inputs (e2e), raw bytes (e2e_raw) ----
    hpack, pack_s = pinned_packed(torch, gbsw, batch, kind)
    e2e_t, r16p = time_e2e(al, sc, hpack, args.steps, min(args.warmup, 2), barrier, packed=True)
    host = pinned(torch, batch)
    raw_t, r16 = time_e2e(al, sc, host, args.steps, min(args.warmup, 2), barrier)
    clocks = sampler.stop()
    e2e_s = over_ranks(statistics.mean(e2e_t), dist.ReduceOp.MAX if dist else None)
    raw_s = over_ranks(statistics.mean(raw_t), dist.ReduceOp.MAX if dist else None)
    offsets_bytes = int(batch.ref_off.nbytes + batch.query_off.nbytes)
    packed_bytes = int(hpack[0].nbytes + hpack[2].nbytes) + offsets_bytes
    total_cells = over_ranks(float(cells), dist.ReduceOp.SUM if dist else None)
    total_pairs = over_ranks(float(batch.n), dist.ReduceOp.SUM if dist else None)

    value = total_cells / (ms / 1e3) / 1e9
    e2e = total_cells / e2e_s / 1e9
    mhz = clocks.get("sm_mhz") or 2070.0
    line = {
        "metric": METRIC, "value": round(value, 2), "unit": "GCUPS", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic",
        "config": {"workload": args.workload, "pairs": int(total_pairs), "pairs_per_gpu": batch.n,
                   "cells_per_step": int(total_cells), "cells_per_step_per_gpu": cells,
                   "shape": WORKLOADS[args.workload][3],
                   "scoring": "+3/-3/-6/-1" if kind == "dna" else "BLOSUM62 -6/-1",
                   "seed": WORKLOADS[args.workload][1], "path": "batched persistent work-queue passes",
                   "l2": "flushed between steps (256 MiB memset outside the step events)",
                   "sharding": "one batch of %d pairs, contiguous cell-balanced shards, one per rank"
                               % int(total_pairs) if world > 1 else "one GPU, the whole batch",
                   "parallelism": "dp%d" % world},
        "e2e": {"value": round(e2e, 2), "unit": "GCUPS", "h2d_bytes_per_step": packed_bytes,
                "d2h_bytes_per_step": int(5 * 2 * batch.n), "ms_per_step": round(e2e_s * 1e3, 3),
                "call": "gbsw_align_packed_host16",
                "inputs": "the batch packed once before timing (gbsw_pack, %s) in page-locked host memory; "
                          "each step copies the packed words and offsets in, unpacks them on the device, "
                          "aligns and copies the int16 results out" % ("2 bits a base" if kind == "dna"
                                                                       else "5 bits a residue"),
                "pack_ms": round(pack_s * 1e3, 3), "pack_threads": os.cpu_count()},
        "e2e_raw": {"value": round(total_cells / raw_s / 1e9, 2), "unit": "GCUPS",
                    "h2d_bytes_per_step": int(batch.ref.nbytes + batch.query.nbytes) + offsets_bytes,
                    "d2h_bytes_per_step": int(5 * 2 * batch.n), "ms_per_step": round(raw_s * 1e3, 3),
                    "call": "gbsw_align_host16", "inputs": "raw bytes in page-locked host memory"},
        "gpu_launches": t["launches"] * args.steps,
        "passes_ms": {"forward": round(t["forward_ms"], 3), "reverse": round(t["reverse_ms"], 3)},
        "plans": t["plans"],
        "roofline": roofline(cells, t["forward_ms"], t["dual"] == 1, t["lane_group"], calib, mhz,
                             TRAFFIC.get(args.workload)),
        "calibration": {k: (round(v, 3) if isinstance(v, float) else v) for k, v in calib.items()},
        "clocks": clocks,
    }
    if rank == 0 and world == 1 and not args.skip_cpu:
        # CPU baseline: the oracle over the whole batch on every host thread; its
        # results check every pair of the device step and of the end-to-end call
        threads = oracle.threads()
        expected, cpu_s = cpu_leg(batch, kind, threads)
        line["cpu_baseline"] = {"value": round(cells / cpu_s / 1e9, 4), "unit": "GCUPS", "cores": threads,
                                "kind": "port", "sample": "all %d pairs (%d cells) of the batch, forward + "
                                                          "reverse, timed once" % (batch.n, cells)}
        line["parity"] = parity(args.workload, batch, {"device_int32": res_dev, "e2e_packed_int16": r16p,
                                                       "e2e_raw_int16": r16}, expected)
    del host, hpack
    if rank == 0 and world == 1:
        threads = oracle.threads()
        if not args.no_extra:
            side_clock = ClockSampler(smi_id)
            side_clock.start()
            line["workloads"] = side_workloads(torch, gbsw, al, dev, stream, flush, calib, mhz, threads,
                                               check=not args.skip_cpu)
            line["workloads"]["clocks"] = side_clock.stop()
            line["reference_cuda"] = reference_cuda_legs(torch, gbsw, al, dev, stream, flush)
            # the autotuner on the headline and mixed batches (a context of its own)
            mixed, _ = generate("mixed_dna")
            line["tuning"] = {"how": "gbsw_tune_device: each candidate variant forced on every length bin, "
                                     "2 timed runs after a warm-up, forward and reverse kernel ms per bin",
                              args.workload: tuning_report(torch, gbsw, local, batch, sc, dev),
                              "mixed_dna": tuning_report(torch, gbsw, local, mixed, scoring_for(gbsw, "dna"), dev),
                              "table": {"%s bin%d bucket%d" % ("dna" if k == 0 else "protein", b, q):
                                        ("dual%d" if v[0] else "int32_%d") % v[1]
                                        for (k, b, q), v in sorted(al.get_tuning().items())},
                              "table_reverse": {"%s bin%d bucket%d" % ("dna" if k == 0 else "protein", b, q):
                                                ("dual%d" if v[0] else "int32_%d") % v[1]
                                                for (k, b, q), v in sorted(al.get_tuning(reverse=True).items())}}
            del mixed
            torch.cuda.empty_cache()
            # traceback of the headline batch (host buffers in, run-length paths out)
            hres = np.ascontiguousarray(al.align_batch(batch, sc))
            seg = np.where(hres[:, 0] > 0, (hres[:, 2] - hres[:, 1]).astype(np.int64) * (hres[:, 4] - hres[:, 3]), 0)
            # host buffers in and out, the sequences in page-locked memory as for e2e
            th = pinned(torch, batch)
            tt, tk = [], []
            for _ in range(3):
                t0 = time.perf_counter()
                tops, _ = al.traceback(sc, th[0], th[1], th[2], th[3], hres)
                tt.append(time.perf_counter() - t0)
                tst = al.stats()
                tk.append((tst["forward_ms"], tst["h2d_ms"], tst["d2h_ms"]))
            del th
            best = int(np.argmin(tt))
            line["traceback"] = {"workload": args.workload, "pairs": batch.n, "segment_cells": int(seg.sum()),
                                 "ms": round(tt[best] * 1e3, 3), "ops": int(len(tops)),
                                 "segment_gcups": round(seg.sum() / tt[best] / 1e9, 2),
                                 "kernel_ms": round(tk[best][0], 3), "copy_in_ms": round(tk[best][1], 3),
                                 "copy_out_ms": round(tk[best][2], 3),
                                 "call": "gbsw_traceback_host, sequences in page-locked host memory"}
            al.close()
            line["serving"] = serving_sweep(gbsw, wl, local)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
