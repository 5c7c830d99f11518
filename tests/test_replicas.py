"""Multi-process replica path of bench.py on CPU (gloo, world size 2).

The closest-point path has no exchange step: `bench.py --gpus N` runs N
replicas of the same per-rank workload and reports the whole job's rate over
the slowest rank's time.  These tests run that aggregation with two gloo
ranks on the host, each rank timing its own small query batch through the
CPU restatement, and check that every rank agrees on the job's time and rate.
"""
import os
import socket

import numpy as np
import pytest


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import sys
    import time

    import torch.distributed as td

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path[:0] = [root, os.path.join(root, "gpu-rt_gb300")]
    import bench
    from oracle import oracle as O
    from gpurt_cpq import workloads as W

    td.init_process_group("gloo", rank=rank, world_size=world)
    try:
        assert bench.dist_env() == (rank, world, rank)
        v, t = W.icosphere(2)
        q = W.uniform_queries(2000 * (rank + 1), -2.0, 2.0, 100 + rank)  # uneven on purpose
        tree = O.Tree(v, t, 2, 4, 0)
        td.barrier()
        t0 = time.perf_counter()
        r = tree.query(q, threads=1)
        mine = time.perf_counter() - t0
        job = bench.max_over_ranks(mine, world, "cpu")
        rate = bench.whole_job_rate(2000, world, job)
        ref = O.brute_f64(v, t, q, threads=1)
        err = float(np.max(np.abs(r["dist"] - ref["dist"]) / np.maximum(ref["dist"], 1e-30)))
        out.put((rank, mine, job, rate, err))
    finally:
        td.destroy_process_group()


def test_two_gloo_replicas_agree_on_time_and_rate():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=180) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, m0, j0, v0, e0), (r1, m1, j1, v1, e1) = res
    assert (r0, r1) == (0, 1)
    assert j0 == j1 == max(m0, m1)  # the slowest replica sets the job's time
    assert v0 == v1 == pytest.approx(2 * 2000 / j0)
    assert e0 <= 1e-6 and e1 <= 1e-6  # each replica's answers are right


def test_single_rank_helpers():
    import sys

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path[:0] = [root, os.path.join(root, "gpu-rt_gb300")]
    import bench

    assert bench.max_over_ranks(1.25, 1, "cpu") == 1.25
    assert bench.whole_job_rate(1000, 1, 0.5) == 2000.0
    assert bench.whole_job_rate(1000, 4, 0.5) == 8000.0
