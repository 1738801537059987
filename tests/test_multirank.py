"""The bench's multi-rank host logic as two gloo ranks on the CPU (no GPU): one vesicle
per rank (independent replicas, different noise seeds), the slowest rank's time taken
by every rank, the whole-job throughput from it, and the reference arm's non-zero ranks
leaving without work.  Rendezvous on 127.0.0.1."""
import os
import socket
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import importlib

    import torch.distributed as dist

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        bench = importlib.import_module("bench")
        S = importlib.import_module(bench.PKG + ".shapes")
        # each rank's own vesicle, a small grid of the benchmark's shape
        F = S.vesicle_256(24, seed=bench.replica_seed(rank))[3]
        ms = 10.0 + 7.5 * rank  # rank 1 is the slow one
        slowest = bench.max_over_ranks(ms, dist, "cpu")
        value = bench.whole_job_gpt_s(world, 1e9, slowest / 1e3)

        class Args:
            steps, warmup, gpus = 1, 0, world

        ref = bench.run_reference(Args, rank, world) if rank != 0 else None
        q.put((rank, float(np.abs(F).sum()), slowest, value, ref))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = {}
    for _ in procs:
        rank, checksum, slowest, value, ref = q.get(timeout=180)
        out[rank] = (checksum, slowest, value, ref)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out[0][0] != out[1][0]  # different replicas
    assert out[0][1] == out[1][1] == 17.5  # every rank takes the slowest time
    assert abs(out[0][2] - 2 / 0.0175) < 1e-9 and out[0][2] == out[1][2]
    assert out[1][3] is None  # the reference arm runs on rank 0 only
