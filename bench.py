#!/usr/bin/env python3
"""GCUPS of the batched Smith-Waterman path on GB300.

One step = the forward (end) and reverse (begin) passes over one batch of the
DNA throughput workload: 100,000 synthetic pairs, references U[400,1024] bp,
queries U[150,300] bp (80% mutated substrings of their reference with 5%
substitutions and 1% indel events, 20% unrelated), scoring +3/-3/-6/-1.
Cells are forward cells, sum |ref|*|query| (the reference's "Total Cells").
``--workload`` selects one of the other synthetic batches instead (plain_dna,
protein, mixed_dna) for side measurements.

value   : GCUPS with the inputs resident in HBM (gbsw_align_device), CUDA events
          around each step on the launching stream, L2 flushed between steps.
e2e     : GCUPS through the host-buffer C ABI call (gbsw_align_host16, the drop-in
          path): pinned host inputs copied in, int16 results copied out, per step.
roofline: the forward pass kernel against the integer-pipe peak measured by the
          calibration probe (gbsw_calibrate): cells per second of the kernel's own
          cell block from registers, every SM busy, timed with CUDA events.
cpu_baseline: the CPU oracle (oracle/gotoh.c, OpenMP) on a bounded sample.
serving : the serving loop (gbsw_server_*) under Poisson job arrivals: peak
          closed-loop GCUPS of the job mix, then p50/p99 job latency and
          sustained GCUPS at 20-100% of that peak (``--serve-only`` prints just
          this part).
traceback: one path per pair of the headline batch (gbsw_traceback_host, host
          buffers in and out), time and run-length operations.

``--impl reference`` times the reference's algorithm on the host cores instead:
the reference has no CPU implementation of its own, so this is the CPU oracle
restating it (kind "port"), with every host thread, on a bounded sample.

Multi-GPU (torchrun, N > 1): every rank aligns its own 100,000-pair batch
(weak scaling); ranks share only a barrier and the max of their step times.
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
PAIRS = 100_000
SCORES = (3, -3, -6, -1)
AA_GAPS = (-6, -1)
# DRAM bytes (read + write) of one forward launch, from an ncu capture of this
# workload (dram__bytes_read.sum + dram__bytes_write.sum); the algorithmic input
# is the sequences and offsets, about 95 MB for the default batch
TRAFFIC = {"dna_throughput": 742.8e6 + 710.0e6, "protein": 21.5e6 + 1.1e6}
# workload -> (pairs, seed, kind, description); the default is the headline batch
WORKLOADS = {
    "dna_throughput": (100_000, 2, "dna", "refs U[400,1024] bp, queries U[150,300] bp, 80% mutated substrings"),
    "plain_dna": (1_000, 1, "dna", "refs U[200,500] bp, queries mutated U[100,150] bp substrings"),
    "protein": (30_000, 3, "aa", "log-normal lengths (median 300, clipped 50-1000), 70% homologs at ~40% id"),
    "mixed_dna": (200_000, 4, "dna", "70% 100-150 bp vs 300 bp, 30% 1000-2048 bp vs 1500-4096 bp"),
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
                    help="skip the side measurements (protein batch, serving sweep)")
    ap.add_argument("--serve-only", action="store_true", help="print only the serving sweep (JSON)")
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


def make_batch(args, rank=0):
    wl = importlib.import_module("gpu-bsw_gb300.workloads")
    pairs, seed, kind, _ = WORKLOADS[args.workload]
    n = args.pairs or pairs
    gen = {"dna_throughput": wl.dna_throughput, "plain_dna": wl.plain_dna, "protein": wl.protein,
           "mixed_dna": wl.mixed_dna}[args.workload]
    return gen(n, seed=seed + rank), kind


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
    return {"workload": "Poisson jobs of U[1,5000] pairs, 60% dna_throughput / 40% protein pairs, "
                        "host buffers in and out",
            "server": opts, "pool_jobs": pool, "mean_job_cells": int(job_cells.mean()),
            "peak_gcups": round(peak, 1), "peak_runs_gcups": [round(v, 1) for v in peaks],
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

    def max_over_ranks(v):
        if dist is None:
            return v
        t = torch.tensor([v], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    if args.serve_only:
        print(json.dumps(serving_sweep(gbsw, wl, local)), flush=True)
        return
    dev = torch.device("cuda", local)
    batch, kind = make_batch(args, rank)
    cells = batch.cells()
    max_len = int(max(batch.ref_lengths().max(), batch.query_lengths().max()))
    if kind == "dna":
        sc = gbsw.make_scoring(gbsw.DNA, scores=SCORES)
    else:
        sc = gbsw.make_scoring(gbsw.PROTEIN, matrix=gbsw.scoring.BLOSUM62, gaps=AA_GAPS)
    al = gbsw.Aligner(local)
    calib = gbsw.calibrate(local)

    # ---- device-resident timing (value) ----
    d_ref = torch.from_numpy(batch.ref).to(dev)
    d_qry = torch.from_numpy(batch.query).to(dev)
    d_ro = torch.from_numpy(batch.ref_off).to(dev)
    d_qo = torch.from_numpy(batch.query_off).to(dev)
    out = torch.empty((5, batch.n), dtype=torch.int32, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.Stream(dev)  # the passes and the step events share this stream
    torch.cuda.set_stream(stream)
    torch.cuda.synchronize()

    def step():
        al.align_device(sc, d_ref.data_ptr(), d_ro.data_ptr(), d_qry.data_ptr(), d_qo.data_ptr(),
                        batch.n, max_len, out[0].data_ptr(), out[1].data_ptr(), out[2].data_ptr(),
                        out[3].data_ptr(), out[4].data_ptr(), stream.cuda_stream)

    try:
        uuid = str(torch.cuda.get_device_properties(local).uuid)
        smi_id = uuid if uuid.startswith("GPU-") else "GPU-" + uuid
    except Exception:
        smi_id = os.environ.get("CUDA_VISIBLE_DEVICES", str(local)).split(",")[local]
    sampler = ClockSampler(smi_id)
    sampler.start()
    for _ in range(args.warmup):
        step()
    al.check(stream.cuda_stream)
    # spot check of the device results against the oracle (not timed)
    res = out.cpu().numpy().T
    idx = np.random.default_rng(rank).choice(batch.n, min(200, batch.n), replace=False)
    sub = batch.subset(idx)
    exp = oracle_run(sub, kind, 0)
    checked = bool(np.array_equal(res[idx], exp))

    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    fwd_ms, rev_ms = [], []
    barrier()
    for k in range(args.steps):
        flush.zero_()  # L2 flush between steps (256 MiB > 129 MB L2), outside the step events
        starts[k].record(stream)
        step()
        ends[k].record(stream)
        st = al.stats()  # waits for this step's kernels; per-kernel event times on the same stream
        fwd_ms.append(st["forward_ms"])
        rev_ms.append(st["reverse_ms"])
    barrier()
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    launches_per_step = al.stats()["launches"]
    lane_group = al.stats()["lane_group"]
    dual_used = al.stats()["dual"]
    ms = max_over_ranks(statistics.mean(step_ms))
    al.check(stream.cuda_stream)

    # ---- end to end through the host-buffer C ABI (e2e) ----
    pin = lambda a: torch.from_numpy(a).pin_memory().numpy()  # noqa: E731
    h_ref, h_qry, h_ro, h_qo = pin(batch.ref), pin(batch.query), pin(batch.ref_off), pin(batch.query_off)
    for _ in range(min(args.warmup, 2)):
        al.align_packed(sc, h_ref, h_ro, h_qry, h_qo, int16=True)
    barrier()
    e2e_t = []
    for _ in range(args.steps):
        t = time.perf_counter()
        r16 = al.align_packed(sc, h_ref, h_ro, h_qry, h_qo, int16=True)
        e2e_t.append(time.perf_counter() - t)
    barrier()
    clocks = sampler.stop()
    e2e_s = max_over_ranks(statistics.mean(e2e_t))
    checked = checked and bool(np.array_equal(r16[idx].astype(np.int32), exp))

    value = cells * world / (ms / 1e3) / 1e9
    e2e = cells * world / e2e_s / 1e9
    fwd = statistics.mean(fwd_ms)
    mhz = clocks.get("sm_mhz") or 2070.0
    # Pairs whose scores fit int16 run two per group in the dual-pair int16x2
    # kernel: its roofline is the calibrated throughput of the DNA dual cell
    # block (the protein variant's cell adds one shared-memory profile load per
    # row).  Everything else runs an int32 kernel, measured against the int32
    # pass's cell block.  Both are cells per second of a register-only probe of
    # the kernel's own cell ops with every SM busy, timed with CUDA events.
    dual = dual_used == 1
    peak_cal = calib["cell_dual_gcups"] if dual else calib["cell_int32_gcups"]
    # nominal: a cell pair of the dual kernel is 6.5 int16x2 ops, all on the
    # integer ALU pipe, which takes a warp instruction every other cycle per SM
    # sub-partition (64 lane-ops per clock per SM); an int32 cell is 6.5 ops,
    # some of which issue to other pipes, so its bound is the issue rate (128
    # lane-ops per clock per SM)
    ops_per_cell = 3.25 if dual else 6.5
    lane_ops = 64 if dual else 128
    peak_nom = calib["sms"] * lane_ops * mhz * 1e6 / ops_per_cell / 1e9
    achieved = cells / (fwd / 1e3) / 1e9

    line = {
        "metric": METRIC, "value": round(value, 2), "unit": "GCUPS", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic",
        "config": {"workload": args.workload, "pairs": batch.n, "cells_per_step_per_gpu": cells,
                   "shape": WORKLOADS[args.workload][3],
                   "scoring": "+3/-3/-6/-1" if kind == "dna" else "BLOSUM62 -6/-1",
                   "seed": WORKLOADS[args.workload][1], "path": "batched persistent work-queue passes",
                   "l2": "flushed between steps (256 MiB memset outside the step events)",
                   "parallelism": "dp%d" % world},
        "e2e": {"value": round(e2e, 2), "unit": "GCUPS",
                "h2d_bytes_per_step": int(batch.ref.nbytes + batch.query.nbytes + batch.ref_off.nbytes
                                          + batch.query_off.nbytes),
                "d2h_bytes_per_step": int(5 * 2 * batch.n), "ms_per_step": round(e2e_s * 1e3, 3),
                "call": "gbsw_align_host16"},
        "gpu_launches": launches_per_step * args.steps,
        "passes_ms": {"forward": round(fwd, 3), "reverse": round(statistics.mean(rev_ms), 3)},
        "roofline": {"bound": "int", "unit": "GCUPS", "achieved": round(achieved, 2),
                     "peak": round(peak_cal, 2), "frac": round(achieved / peak_cal, 4),
                     "traffic": TRAFFIC.get(args.workload), "kernel": "forward pass (%s)" %
                     ("sw_pass_dual, int16x2, 2 pairs per %d-lane group" % lane_group if dual else
                      "sw_pass, int32, %d lanes per pair" % lane_group),
                     "peak_source": "measured: gbsw_calibrate register-only probe of the kernel's own cell "
                                    "block, %d SMs busy, timed with CUDA events (HBM and bf16 peaks do not "
                                    "bound this integer path)" % calib["sms"],
                     "nominal_peak": round(peak_nom, 2), "nominal_frac": round(achieved / peak_nom, 4),
                     "nominal_source": "%d lane-ops/clk/SM (%s) x %d SMs x %.0f MHz / %.2f ops per cell"
                                       % (lane_ops, "ALU pipe" if dual else "issue", calib["sms"], mhz,
                                          ops_per_cell)},
        "calibration": {k: (round(v, 3) if isinstance(v, float) else v) for k, v in calib.items()},
        "clocks": clocks,
        "checked_vs_oracle": checked,
    }
    if rank == 0:
        # CPU baseline: the oracle on a bounded sample, all host threads
        threads = oracle.threads()
        sample = cpu_sample(batch, 10.0, threads, kind)
        cpu_s = time_cpu(sample, threads, kind)
        line["cpu_baseline"] = {"value": round(sample.cells() / cpu_s / 1e9, 4), "unit": "GCUPS",
                                "cores": threads, "kind": "port",
                                "sample": "first %d of %d pairs (%d cells), forward + reverse"
                                          % (sample.n, batch.n, sample.cells())}
        if not args.no_extra and world == 1 and args.workload == WORKLOAD:
            pb = wl.protein(30_000, seed=3)
            psc = gbsw.make_scoring(gbsw.PROTEIN, matrix=gbsw.scoring.BLOSUM62, gaps=(-6, -1))
            al.align_batch(pb, psc)
            t = []
            for _ in range(3):
                al.align_batch(pb, psc)
                s = al.stats()
                t.append(s["forward_ms"] + s["reverse_ms"])
            line["protein"] = {"workload": "protein 30,000 pairs, BLOSUM62 -6/-1",
                               "kernel_gcups": round(pb.cells() / (min(t) / 1e3) / 1e9, 2),
                               "cells": pb.cells()}
            # traceback of the headline batch (host buffers in, run-length paths out)
            hres = np.ascontiguousarray(al.align_batch(batch, sc))
            seg = np.where(hres[:, 0] > 0, (hres[:, 2] - hres[:, 1]).astype(np.int64) * (hres[:, 4] - hres[:, 3]), 0)
            tt = []
            for _ in range(3):
                t = time.perf_counter()
                tops, _ = al.traceback_batch(batch, sc, hres)
                tt.append(time.perf_counter() - t)
            line["traceback"] = {"workload": args.workload, "pairs": batch.n, "segment_cells": int(seg.sum()),
                                 "ms": round(min(tt) * 1e3, 3), "ops": int(len(tops)),
                                 "segment_gcups": round(seg.sum() / min(tt) / 1e9, 2),
                                 "call": "gbsw_traceback_host"}
            al.close()
            line["serving"] = serving_sweep(gbsw, wl, local)
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
