"""World-size-2 gloo test of the multi-rank path on CPU: each rank aligns its
cell-balanced shard (with the CPU oracle standing in for the GPU) and the
gathered slices equal the single-process result."""
import importlib
import multiprocessing as mp
import os
import socket
import sys

import numpy as np

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out_q):
    sys.path.insert(0, REPO)
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import torch.distributed as dist
    import oracle
    shard = importlib.import_module("gpu-bsw_gb300.shard")
    wl = importlib.import_module("gpu-bsw_gb300.workloads")
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank,
                            world_size=world)
    batch = wl.custom_dna(300, 77, 50, 400, 20, 200, related=0.7)
    a, b, sub = shard.rank_slice(batch, rank, world)
    local = oracle.align(oracle.DNA, sub.ref, sub.ref_off, sub.query, sub.query_off,
                         scores=(3, -3, -6, -1), nthreads=1)
    full = shard.gather_results(local, rank, world)
    if rank == 0:
        ref = oracle.align(oracle.DNA, batch.ref, batch.ref_off, batch.query, batch.query_off,
                           scores=(3, -3, -6, -1), nthreads=1)
        out_q.put((bool(np.array_equal(full, ref)), int(b - a)))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_shards_equal_single_process(workloads):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    ok, n0 = q.get(timeout=240)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert ok and 0 < n0 < 300
