#!/usr/bin/env python
"""Closest-point queries/s on one GB300: the large heightfield workload.

Workload (seeded, synthetic; no dataset involved): a 1024 x 1024-vertex
heightfield over [0,1]^2 (2,093,058 triangles; z = 8 sinusoids, frequencies
U[1,32], amplitude 0.05/f, + N(0,1e-3)), 16,777,216 queries (half within
N(0, 0.01^2) of random surface points, half uniform in [-0.1,1.1]^2 x
[-0.5,0.5]); 4-wide BVH, leaf size autotuned (cp_autotune, branching fixed).

A step is one cp_query over all 16M queries with the inputs resident in HBM
(Hilbert ordering of the queries + persistent warp-packet traversal + exact
re-evaluation of each winner).  `value` is queries/s over K timed steps (CUDA events on the
launching stream).  `e2e` is the same metric through cp_query_host: pinned
host queries in, closest point / distance / triangle out, copies included.

Roofline (dominant kernel = the traversal): algorithmic bytes per query are
B_io = 32 (query 12 + point 12 + distance 4 + index 4) plus
B_trav = 32 V_node + 36 V_tri, with V_node / V_tri the mean binary-node visits
and triangle tests of the canonical algorithm (binary Morton LBVH, leaf <= 4,
closest-first), measured by the CPU restatement on a seeded 65,536-query
sample of this workload.  t_roof = B_io / BW_HBM + B_trav / BW_L2 with BW_HBM
from MEASURED_PEAKS.json and BW_L2 measured here; frac = t_roof / t_kernel.

Multi-GPU: the path needs no exchange; each rank runs the same workload on its
own GPU (replicas, weak scaling), barrier + max-over-ranks timing.

The headline line also carries `forms`: the three other targets, each measured
in the same run on the same GPU with its own clock record (forward + backward
over forward on the torus workload, the batched workload against per-mesh
launches, and the dynamic soup loop's time per iteration).

--impl reference: the reference's closest-point code is not in its mounted
tree (its FCPW-GPU branch is absent), so the reference arm times the CPU
restatement of the same algorithm (the oracle port) on all host cores, on the
same workload and config: every step is all 16,777,216 queries.  It loads the
workload generator by file path, so no CUDA library of this package is mapped
into that process.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
PKG = ROOT / "gpu-rt_gb300"
for p in (str(ROOT), str(PKG)):
    if p not in sys.path:
        sys.path.insert(0, p)

import numpy as np  # noqa: E402

METRIC = "closest-point queries/s (large heightfield, 2.09M tris, 16M queries)"
UNIT = "queries/s"
N_QUERIES = 16 * (1 << 20)
DATA = "synthetic (seeded heightfield + queries, generated on the host)"


def bench_config(world: int) -> dict:
    """The workload both arms run, identical in each arm's JSON line."""
    return {"workload": "large heightfield: 1024x1024 vertices (2,093,058 tris), 16,777,216 queries "
                        "(50% near-surface sigma 0.01, 50% box)",
            "l2": "inputs larger than L2 (201 MB queries + 336 MB outputs per step, and the BVH's "
                  "nodes and triangle records); no flush",
            "parallelism": f"replicas x{world}"}
B_IO = 32.0
# canonical visit counts (binary LBVH, leaf 4) of this seeded workload, from the
# CPU restatement on the first 65,536 queries; re-measured in the CPU leg
CANON_V_NODE = 84.273
CANON_V_TRI = 44.413
# DRAM bytes (read + write) per query of one traversal launch at the leaf size
# the autotuner picks for this workload, from one ncu capture of
# dram__bytes_read.sum + dram__bytes_write.sum on the same command; keyed by
# leaf size so a run that picks another leaf reports null, not a stale figure
NCU_TRAFFIC_PER_QUERY = {8: 378.1}
# Adjoint per query: reads q 12 + triangle 4 + barycentrics 8 + upstream
# gradient 4 + 3 vertex indices 12 + 3 vertices 36; writes d/dq 12 and three
# atomic read-modify-writes of 12 B to d/dvertices (72)
BWD_BYTES_PER_QUERY = 160
# Build per triangle (algorithmic): validation 48 (indices + vertex gather),
# centroid bounds 48, Morton keys 60 (gather + key and index out), 7 radix
# passes of 64-bit keys with an index 224 (histogram read 8, scatter 12 in and
# 12 out), Karras nodes 28 (key reads, three child/parent words out), refit
# 252 (gather 48, exact and test records out 48 + 80, box 24, inverse order 4,
# child boxes in and box out per inner node 48)
BUILD_BYTES_PER_TRI = 660


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=60)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-sample", type=int, default=1 << 21,
                    help="queries timed on the host cores for the CPU baseline")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--width", type=int, default=1920, help="shade workload: image width")
    ap.add_argument("--height", type=int, default=1440, help="shade workload: image height")
    ap.add_argument("--no-forms", action="store_true",
                    help="skip the torus, batched and dynamic forms in the headline run")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--leaf", type=int, default=0)
    ap.add_argument("--seed-chunk", type=int, default=1,
                    help="packets per claim of the seeded packet traversal without the autotuner (1: unseeded)")
    ap.add_argument("--workload", default="large",
                    choices=["large", "torus", "batched", "dynamic", "small", "rays", "scene", "camera",
                             "shade"],
                    help="large is the headline; the others measure the other forms")
    return ap.parse_args()


def dist_env():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


def host_cores() -> int:
    return len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)


def cpu_model() -> str:
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    return "unknown"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 100 ms while running."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.lines: list[str] = []
        self.proc = None
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(gpu_index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for name, val in zip(names, parts[4:8]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(max(smax)) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def max_over_ranks(x: float, world: int, device) -> float:
    """The largest of each rank's x (x itself on one rank): the job's time is
    its slowest replica's."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as td

    t = torch.tensor([x], dtype=torch.float64, device=device)
    td.all_reduce(t, op=td.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank: float, world: int, seconds: float) -> float:
    """Units all replicas processed per second (weak scaling: each rank runs
    the same per-rank workload)."""
    return world * units_per_rank / seconds


def measured_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        return json.loads(p.read_text())
    return {"hbm_gbs": 6800.0, "fallback": True}


def peaks_label(peaks: dict) -> str:
    """'measured' for MEASURED_PEAKS.json, 'fallback' for the stated stand-in
    (6.8 TB/s HBM, one earlier measurement on a GB300)."""
    return "fallback" if peaks.get("fallback") else "measured"


def measure_l2_gbs(torch) -> float:
    """L2 read bandwidth: best of 128-bit-load sweeps over 24/48/96 MB L2-resident buffers."""
    from ctypes import byref, c_double, c_void_p

    from gpurt_cpq._lib import check, lib

    best = 0.0
    for mb in (24, 48, 96):  # all below the 126 MB L2; the best is the denominator
        g = c_double()
        check(lib.cp_probe_read_bandwidth(mb << 20, 20, byref(g),
                                          c_void_p(torch.cuda.current_stream().cuda_stream)), "probe")
        best = max(best, g.value)
    return best


def workloads_module():
    """gpurt_cpq/workloads.py loaded by file path: the generators are numpy
    only, and importing them through the package would map its CUDA library
    into a process that must not use it (the reference arm)."""
    import importlib.util

    name = "gpurt_cpq_workloads_standalone"
    if name in sys.modules:
        return sys.modules[name]
    spec = importlib.util.spec_from_file_location(name, PKG / "gpurt_cpq" / "workloads.py")
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


def workload():
    return workloads_module().large()


def cpu_leg(v, t, q, sample: int) -> dict:
    """CPU restatement (oracle port) on all host cores: canonical tree, bounded sample."""
    from oracle import oracle as O

    O.build()
    threads = host_cores()
    t0 = time.perf_counter()
    tree = O.Tree(v, t, 2, 4, 0)
    build_s = time.perf_counter() - t0
    stat = tree.query(q[:65536], threads=threads, stats=True)
    s = q[:sample]
    r = tree.query(s, threads=threads)
    return {"value": s.shape[0] / r["seconds"], "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"first {s.shape[0]} of the {q.shape[0]} queries, canonical binary LBVH "
                      f"(leaf 4) built on the host in {build_s:.2f} s, {cpu_model()}",
            "build_s": build_s,
            "v_node": float(stat["node_visits"].mean()), "v_tri": float(stat["tri_tests"].mean())}


def emit(obj):
    print(json.dumps(obj), flush=True)


def reference_arm(args):
    """The CPU restatement (oracle port) on all host cores over the same
    workload: every warm-up and timed step queries all 16,777,216 points."""
    rank, world, _ = dist_env()
    if world > 1:
        import torch.distributed as td

        td.init_process_group("gloo")
        td.barrier()
        if rank != 0:
            td.destroy_process_group()
            return
    from oracle import oracle as O

    O.build()
    v, t, q = workload()
    threads = host_cores()
    t0 = time.perf_counter()
    tree = O.Tree(v, t, 2, 4, 0)
    build_s = time.perf_counter() - t0
    for _ in range(args.warmup):
        tree.query(q, threads=threads)
    secs = 0.0
    for _ in range(args.steps):
        t0 = time.perf_counter()
        tree.query(q, threads=threads)
        secs += time.perf_counter() - t0
    value = q.shape[0] * args.steps / secs
    emit({"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
          "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * secs / args.steps,
          "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
          "data": DATA, "config": bench_config(world),
          "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                           "sample": f"all {q.shape[0]} queries per step, canonical binary LBVH leaf 4 "
                                     f"(built in {build_s:.2f} s), {cpu_model()}; the reference's "
                                     "own closest-point code is absent from its tree"},
          "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}})
    if world > 1:
        import torch.distributed as td

        td.destroy_process_group()


def our_arm(args):
    import torch

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as td

        torch.cuda.set_device(local)
        td.init_process_group("nccl")
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    import gpurt_cpq as cpq
    from gpurt_cpq._lib import CP_TIMING_COUNTERS, CP_TIMING_EVENTS, lib

    v, t, q = workload()
    vd = torch.from_numpy(v).to(dev)
    td_ = torch.from_numpy(t).to(dev)
    qd = torch.from_numpy(q).to(dev)
    nq = q.shape[0]

    # 4-wide BVH; leaf size, block size and traversal kernel autotuned on the
    # workload's own query set (warp coherence depends on the query density)
    leaf, qopts = 4, cpq.query_opts(seed_chunk=args.seed_chunk)
    tuned = None
    if args.leaf:
        leaf = args.leaf
    elif not args.no_autotune:
        bo, qo = cpq.autotune(vd, td_, qd, cache_path=None, branching=4)
        leaf, qopts = bo.leaf_size, qo
        tuned = {"leaf_size": bo.leaf_size, "block_size": qo.block_size,
                 "traversal": ["auto", "thread", "packet"][qo.traversal],
                 "short_stack": qo.short_stack, "seed_chunk": qo.seed_chunk}
    mesh = cpq.Mesh(vd, td_, branching=4, leaf_size=leaf)
    info = mesh.info()
    ws = torch.empty(mesh.workspace_size(nq, qopts), dtype=torch.uint8, device=dev)
    out = mesh.query(qd, workspace=ws, opts=qopts)
    l2_gbs = measure_l2_gbs(torch)
    for _ in range(args.warmup):
        mesh.query(qd, workspace=ws, opts=qopts, out=out)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    lib.cp_timing_enable(CP_TIMING_EVENTS)
    from ctypes import byref, c_double, c_int64, c_uint64

    tms, tl = c_double(), c_int64()
    lib.cp_timing_read(byref(tms), byref(tl), 1)
    launches0 = lib.cp_kernel_launches()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        mesh.query(qd, workspace=ws, opts=qopts, out=out)
    e1.record()
    torch.cuda.synchronize()
    launches = lib.cp_kernel_launches() - launches0
    ms = e0.elapsed_time(e1)
    if world > 1:
        torch.distributed.barrier()
    clk = clocks.stop()
    lib.cp_timing_read(byref(tms), byref(tl), 1)
    trav_ms = tms.value / max(tl.value, 1)
    # packet kernel: per-warp node visits / triangle tests, from one more
    # (untimed) query through the counting build of the kernel
    counts = (c_uint64 * 7)()
    lib.cp_timing_enable(CP_TIMING_COUNTERS)
    lib.cp_traversal_stats(counts, 1)
    mesh.query(qd, workspace=ws, opts=qopts, out=out)
    lib.cp_traversal_stats(counts, 1)
    lib.cp_timing_enable(0)
    per_q = float(nq)
    packet_visits = {"node_visits_per_query": counts[0] * 32 / per_q / 32,
                     "warp_node_visits_per_32_queries": counts[0] * 32 / per_q,
                     "warp_tri_tests_per_32_queries": counts[1] * 32 / per_q,
                     "warp_pops_per_32_queries": counts[2] * 32 / per_q,
                     "warp_skipped_pops_per_32_queries": counts[3] * 32 / per_q,
                     "lane_tri_tests_per_query": counts[4] / per_q,
                     "warp_tri_rounds_per_32_queries": counts[5] * 32 / per_q,
                     "tri_round_lane_use": counts[4] / max(counts[5] * 32, 1),
                     "node_visit_lane_use": counts[6] / max(counts[0] * 32, 1)} if counts[0] else None
    ms = max_over_ranks(ms, world, dev)
    value = whole_job_rate(nq * args.steps, world, ms * 1e-3)
    assert mesh.device_status() == 0

    # end to end through the host entry points: pinned buffers, every step's
    # upload and download inside the timed region.  Headline: a stream of
    # batches through cp_query_host_async on two streams taking alternate
    # steps (double buffering: one step's copies under the other's kernels);
    # beside it the blocking cp_query_host, one step at a time.
    qh = torch.from_numpy(q).pin_memory()

    def host_outs():
        return {"dist": torch.empty(nq, dtype=torch.float32).pin_memory(),
                "tri": torch.empty(nq, dtype=torch.int32).pin_memory(),
                "point": torch.empty((nq, 3), dtype=torch.float32).pin_memory()}

    hout = [host_outs(), host_outs()]
    e2e_steps = max(1, min(args.steps, 30))
    mesh.query_host(qh, opts=qopts, out=hout[0])
    if world > 1:
        torch.distributed.barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        mesh.query_host(qh, opts=qopts, out=hout[0])
    sync_s = max_over_ranks(time.perf_counter() - t0, world, dev)
    streams = [torch.cuda.Stream(dev), torch.cuda.Stream(dev)]
    for k in range(2):
        mesh.query_host_async(qh, hout[k], opts=qopts, stream=streams[k])
    for st in streams:
        st.synchronize()
    if world > 1:
        torch.distributed.barrier()
    t0 = time.perf_counter()
    for k in range(e2e_steps):
        mesh.query_host_async(qh, hout[k % 2], opts=qopts, stream=streams[k % 2])
    for st in streams:
        st.synchronize()
    e2e_s = max_over_ranks(time.perf_counter() - t0, world, dev)
    # the downloaded answers are the device call's
    assert torch.equal(hout[(e2e_steps - 1) % 2]["dist"], out.dist.cpu())
    e2e = {"value": whole_job_rate(nq * e2e_steps, world, e2e_s), "unit": UNIT,
           "h2d_bytes_per_step": nq * 12, "d2h_bytes_per_step": nq * (12 + 4 + 4),
           "steps": e2e_steps,
           "path": "cp_query_host_async, pinned host buffers, two streams taking alternate steps",
           "blocking": {"value": whole_job_rate(nq * e2e_steps, world, sync_s), "unit": UNIT,
                        "path": "cp_query_host, one step at a time (copy in, query, copy out)"}}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_leg(v, t, q, min(args.cpu_sample, nq))
    v_node = cpu["v_node"] if cpu else CANON_V_NODE
    v_tri = cpu["v_tri"] if cpu else CANON_V_TRI
    peaks = measured_peaks()
    hbm = float(peaks["hbm_gbs"])
    b_trav = 32.0 * v_node + 36.0 * v_tri
    t_roof = B_IO / (hbm * 1e9) + b_trav / (l2_gbs * 1e9)          # s per query
    t_kernel = trav_ms * 1e-3 / nq                                  # s per query
    achieved = (B_IO + b_trav) / t_kernel / 1e9
    peak_eff = (B_IO + b_trav) / t_roof / 1e9
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak_eff, "unit": "GB/s",
                "frac": achieved / peak_eff, "of": peaks_label(peaks),
                "traffic": NCU_TRAFFIC_PER_QUERY[leaf] * nq if leaf in NCU_TRAFFIC_PER_QUERY else None,
                "kernel": "k_traverse_packet" if packet_visits else "k_traverse",
                "kernel_ms_per_launch": trav_ms,
                "model": "t_roof = B_io/BW_HBM + B_trav/BW_L2 (algorithmic bytes of the canonical "
                         "binary LBVH); peak = (B_io + B_trav)/t_roof",
                "bytes_per_query": {"io": B_IO, "trav": b_trav, "v_node": v_node, "v_tri": v_tri},
                "hbm_gbs": hbm, "l2_gbs_measured": l2_gbs,
                "hbm_only_frac": B_IO / t_kernel / 1e9 / hbm,
                # the structure a launch walks: wide nodes (32 K bytes each) and
                # the 80-byte test and 48-byte exact records per triangle
                "structure_bytes": int(info.num_wide_nodes * 32 * info.branching + info.num_triangles * (80 + 48)),
                "packet_counters": packet_visits}
    forms = None
    if world == 1 and not args.no_forms:
        forms = run_forms(args)
    if rank == 0:
        build_gbs = (BUILD_BYTES_PER_TRI * info.num_triangles / (info.build_ms * 1e-3) / 1e9
                     if info.build_ms > 0 else None)
        res = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
               "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
               "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": DATA,
               "config": bench_config(world),
               "build": {"branching": 4, "leaf_size": leaf, "autotuned": tuned,
                         "block_size": qopts.block_size, "short_stack": qopts.short_stack,
                         "seed_chunk": qopts.seed_chunk,
                         "sort_queries": bool(qopts.sort_queries),
                         "wide_nodes": info.num_wide_nodes, "build_ms": info.build_ms,
                         "build_roofline": {"bytes_per_triangle": BUILD_BYTES_PER_TRI,
                                            "achieved_gbs": build_gbs,
                                            "frac_of_hbm": build_gbs / hbm if build_gbs else None}},
               "e2e": e2e, "roofline": roofline, "gpu_launches": int(launches),
               "clocks": clk}
        if forms is not None:
            res["forms"] = forms
        if cpu is not None:
            res["cpu_baseline"] = {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample")}
        emit(res)
    if world > 1:
        torch.distributed.destroy_process_group()


# ---------------------------------------------------------------------------
# The other forms of the path (one GPU each).  These print their own JSON line;
# the default workload above is the headline.


def _timed(torch, fn, steps, warmup):
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


def _line(metric, value, unit, ms, args, config, extra):
    res = {"metric": metric, "value": value, "unit": unit, "n_gpus": 1, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)", "config": config}
    res.update(extra)
    emit(res)


def _form(metric, value, unit, ms, steps, warmup, config, extra) -> dict:
    """One form's result: what its own JSON line carries."""
    res = {"metric": metric, "value": value, "unit": unit, "ms_per_step": ms, "steps": steps,
           "warmup": warmup, "config": config}
    res.update(extra)
    return res


def _emit_form(args, f: dict):
    extra = {k: v for k, v in f.items()
             if k not in ("metric", "value", "unit", "ms_per_step", "steps", "warmup", "config")}
    _line(f["metric"], f["value"], f["unit"], f["ms_per_step"], args, f["config"], extra)


def torus_form(steps: int, warmup: int) -> dict:
    """Forward + adjoint on the differentiable workload vs forward alone."""
    import torch

    import gpurt_cpq as cpq
    from gpurt_cpq import workloads as W

    dev = torch.device("cuda", 0)
    v, t, q, g = W.torus_workload()
    vd, td, qd, gd = (torch.from_numpy(x).to(dev) for x in (v, t, q, g))
    nq = qd.shape[0]
    mesh = cpq.Mesh(vd, td, branching=4, leaf_size=2)
    o = cpq.query_opts()
    ws = torch.empty(mesh.workspace_size(nq, o), dtype=torch.uint8, device=dev)
    out = mesh.query(qd, want_point=False, want_bary=True, workspace=ws, opts=o)
    gv = torch.zeros_like(vd)

    def fwd():
        mesh.query(qd, want_point=False, want_bary=True, workspace=ws, opts=o, out=out)

    def fwd_bwd():
        fwd()
        gv.zero_()
        mesh.backward(qd, out.tri, out.bary, gd, grad_verts=gv)

    ms_f = _timed(torch, fwd, steps, warmup)
    ms_fb = _timed(torch, fwd_bwd, steps, warmup)

    def bwd():
        gv.zero_()
        mesh.backward(qd, out.tri, out.bary, gd, grad_verts=gv)

    ms_b = _timed(torch, bwd, steps, warmup)
    bwd_gbs = BWD_BYTES_PER_QUERY * nq / (ms_b * 1e-3) / 1e9
    return _form("closest-point fwd+bwd queries/s (torus 200k tris, 4M queries)", nq / (ms_fb * 1e-3),
                 "queries/s", ms_fb, steps, warmup,
                 {"workload": "torus R=1 r=0.3 500x200 (200,000 tris), 4,194,304 queries U[-1.5,1.5]^3, "
                              "upstream gradient N(0,1); forward caches (tri, bary), adjoint recomputes",
                  "branching": 4, "leaf_size": 2},
                 {"forward_only": {"value": nq / (ms_f * 1e-3), "ms_per_step": ms_f},
                  "backward_only": {"value": nq / (ms_b * 1e-3), "ms_per_step": ms_b,
                                    "roofline": {"bound": "hbm", "achieved": bwd_gbs, "peak": measured_peaks()["hbm_gbs"],
                                                 "unit": "GB/s", "frac": bwd_gbs / measured_peaks()["hbm_gbs"],
                                                 "of": peaks_label(measured_peaks()),
                                                 "bytes_per_query": BWD_BYTES_PER_QUERY}},
                  "fwd_bwd_over_fwd": ms_fb / ms_f, "target_fwd_bwd_over_fwd": 2.5})


def torus_arm(args):
    _emit_form(args, torus_form(args.steps, args.warmup))


def rays_arm(args):
    """Ray queries (cp_ray_query) through the large workload's BVH: 16M rays
    from the workload's query points in seeded random directions, closest hit
    (trace_ray) and any hit (visibility)."""
    import torch

    import gpurt_cpq as cpq

    dev = torch.device("cuda", 0)
    v, t, q = workload()
    rng = np.random.default_rng(17)
    d = rng.normal(size=q.shape).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    vd, td, od, dd = (torch.from_numpy(x).to(dev) for x in (v, t, q, d))
    n = od.shape[0]
    mesh = cpq.Mesh(vd, td, branching=4, leaf_size=4)
    closest, anyhit = cpq.ray_opts(), cpq.ray_opts(any_hit=True)
    r = mesh.ray_query(od, dd, opts=closest)
    ms_c = _timed(torch, lambda: mesh.ray_query(od, dd, opts=closest), args.steps, args.warmup)
    ms_a = _timed(torch, lambda: mesh.ray_query(od, dd, opts=anyhit), args.steps, args.warmup)
    _line("ray queries/s, closest hit (large heightfield, 2.09M tris, 16M rays)", n / (ms_c * 1e-3),
          "rays/s", ms_c, args,
          {"workload": "large heightfield mesh; origins = the 16,777,216 closest-point queries, "
                       "directions uniform on the sphere (seed 17); t in [0, inf)",
           "branching": 4, "leaf_size": 4, "sort_rays": True},
          {"any_hit": {"value": n / (ms_a * 1e-3), "ms_per_step": ms_a},
           "hit_fraction": float((r.tri >= 0).float().mean())})


def batched_form(steps: int, warmup: int) -> dict:
    """256 uneven meshes: a leaf size per size class (cp_batch_autotune), one
    batched build + one persistent graph-captured launch, against plain
    per-mesh builds (each with its mesh's leaf size) and launches on the same
    GPU."""
    import torch

    import gpurt_cpq as cpq
    from gpurt_cpq import workloads as W

    dev = torch.device("cuda", 0)
    meshes, queries = W.batched()
    V, voff, T, toff, Q, qoff = W.concat_batch(meshes, queries)
    Vd, Td, Qd = (torch.from_numpy(x).to(dev) for x in (V, T, Q))
    nq = Qd.shape[0]
    t0 = time.perf_counter()
    leaves, o = cpq.autotune_batch(Vd, voff, Td, toff, Qd, qoff, branching=4)
    tune_s = time.perf_counter() - t0
    cls = np.floor(np.log2(np.diff(toff))).astype(int)
    per_class = {int(c): int(leaves[cls == c][0]) for c in np.unique(cls)}
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    batch = cpq.Batch(Vd, voff, Td, toff, branching=4, leaf_sizes=leaves)
    torch.cuda.synchronize()
    build_batch_ms = (time.perf_counter() - t0) * 1e3
    ws = torch.empty(batch.workspace_size(nq, o), dtype=torch.uint8, device=dev)
    out = cpq.QueryResult(point=torch.empty((nq, 3), device=dev), dist=torch.empty(nq, device=dev),
                          tri=torch.empty(nq, dtype=torch.int32, device=dev), bary=None)

    def batched_step():
        batch.query(Qd, qoff, workspace=ws, opts=o, use_graph=True, out=out)

    ms_b = _timed(torch, batched_step, steps, warmup)
    d_batched = out.dist.clone()
    # plain per-mesh: one build and one launch sequence per mesh
    vparts = [Vd[voff[i]:voff[i + 1]] for i in range(len(meshes))]
    tparts = [Td[toff[i]:toff[i + 1]] for i in range(len(meshes))]
    qparts = [Qd[qoff[i]:qoff[i + 1]] for i in range(len(meshes))]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    plain = [cpq.Mesh(vparts[i], tparts[i].contiguous(), branching=4, leaf_size=int(leaves[i]))
             for i in range(len(meshes))]
    torch.cuda.synchronize()
    build_plain_ms = (time.perf_counter() - t0) * 1e3
    wss = [torch.empty(plain[i].workspace_size(qparts[i].shape[0], o), dtype=torch.uint8, device=dev)
           for i in range(len(meshes))]
    outs = [cpq.QueryResult(point=out.point[qoff[i]:qoff[i + 1]], dist=out.dist[qoff[i]:qoff[i + 1]],
                            tri=out.tri[qoff[i]:qoff[i + 1]], bary=None) for i in range(len(meshes))]

    def plain_step():
        for i in range(len(meshes)):
            plain[i].query(qparts[i], workspace=wss[i], opts=o, out=outs[i])

    ms_p = _timed(torch, plain_step, steps, warmup)
    rel = float(((out.dist - d_batched).abs() / d_batched.clamp_min(1e-30)).max())
    tri_counts = [int(toff[i + 1] - toff[i]) for i in range(len(meshes))]
    return _form("closest-point queries/s (batched: 256 uneven meshes, one launch)", nq / (ms_b * 1e-3),
                 "queries/s", ms_b, steps, warmup,
                 {"workload": f"256 deformed icospheres/tori, {int(toff[-1])} tris "
                              f"({min(tri_counts)}..{max(tri_counts)} per mesh), {nq} queries "
                              f"({int(np.diff(qoff).min())}..{int(np.diff(qoff).max())} per mesh)",
                  "branching": 4, "leaf_size": "per size class (autotuned)", "graph": True},
                 {"autotuned": {"leaf_size_by_tri_class": per_class, "tune_s": tune_s},
                  "per_mesh_launches": {"value": nq / (ms_p * 1e-3), "ms_per_step": ms_p},
                  "speedup_vs_per_mesh": ms_p / ms_b, "target_speedup": 3.0,
                  "max_rel_diff_batched_vs_per_mesh": rel,
                  "build_ms": {"batched": build_batch_ms, "per_mesh_total": build_plain_ms}})


def batched_arm(args):
    _emit_form(args, batched_form(args.steps, args.warmup))


def dynamic_form(steps: int, warmup: int) -> dict:
    """8M-triangle soup: per iteration perturb the vertices, refit, query 64M
    fixed points and 1M moving points, adjoint on the moving points, and a
    gradient step on their squared distance."""
    import torch

    import gpurt_cpq as cpq
    from gpurt_cpq import workloads as W

    dev = torch.device("cuda", 0)
    v, t = W.soup()
    vd, td = torch.from_numpy(v).to(dev), torch.from_numpy(t).to(dev)
    # 64M fixed queries drawn on the device from a seeded generator (host
    # generation of 64M points takes minutes); the moving points from numpy
    qfix = torch.rand((64 * (1 << 20), 3), device=dev,
                      generator=torch.Generator(device=dev).manual_seed(11))
    pts = torch.from_numpy(W.uniform_queries(1 << 20, 0.0, 1.0, 12)).to(dev)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    mesh = cpq.Mesh(vd, td, branching=4, leaf_size=2)
    torch.cuda.synchronize()
    build_ms = (time.perf_counter() - t0) * 1e3
    # seeded packets (4 per claim): 212 against 247 ms per iteration unseeded
    o = cpq.query_opts(seed_chunk=4)
    wsf = torch.empty(mesh.workspace_size(qfix.shape[0], o), dtype=torch.uint8, device=dev)
    wsp = torch.empty(mesh.workspace_size(pts.shape[0], o), dtype=torch.uint8, device=dev)
    outf = mesh.query(qfix, want_point=False, workspace=wsf, opts=o)
    outp = mesh.query(pts, want_point=False, want_bary=True, workspace=wsp, opts=o)
    torch.cuda.manual_seed(13)  # the default generator: captured graphs advance it per replay
    noise = torch.empty_like(vd)
    lr = 0.25

    def iteration():
        noise.normal_(0.0, 1e-4)
        vd.add_(noise)
        mesh.refit(vd)
        mesh.query(qfix, want_point=False, workspace=wsf, opts=o, out=outf)
        mesh.query(pts, want_point=False, want_bary=True, workspace=wsp, opts=o, out=outp)
        # d(d^2)/dq = 2 d * d(d)/dq
        gq, _ = mesh.backward(pts, outp.tri, outp.bary, 2.0 * outp.dist, need_verts=False)
        pts.sub_(lr * gq)

    iters = 50
    # warm up on a side stream, then capture one iteration (refit, two query
    # launch sequences, adjoint, step: every call stream-ordered) and replay it
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        for _ in range(max(1, warmup)):
            iteration()
    torch.cuda.current_stream().wait_stream(side)
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        iteration()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(iters):
        graph.replay()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / iters
    t0 = time.perf_counter()
    rebuilt = cpq.Mesh(vd, td, branching=4, leaf_size=2)
    torch.cuda.synchronize()
    rebuild_ms = (time.perf_counter() - t0) * 1e3
    del rebuilt
    nq = qfix.shape[0] + pts.shape[0]
    return _form("closest-point queries/s (dynamic soup loop: refit + fwd + bwd per iteration)",
                 nq / (ms * 1e-3), "queries/s", ms, iters, max(1, warmup),
                 {"workload": "4,096 Gaussian clusters x 2,048 tris (8,388,608-tri soup), vertices "
                              "perturbed N(0,1e-4) per iteration, 67,108,864 fixed + 1,048,576 moving "
                              "queries, 50 iterations of refit + forward + adjoint + step",
                  "branching": 4, "leaf_size": 2, "iterations": iters, "graph": True, "seed_chunk": 4},
                 {"build_ms": build_ms, "rebuild_ms": rebuild_ms, "final_mean_dist":
                  float(outp.dist.mean())})


def dynamic_arm(args):
    _emit_form(args, dynamic_form(args.steps, args.warmup))


def run_forms(args) -> dict:
    """The torus, batched and dynamic forms in the headline run, each timed
    like its own `--workload` line (at most 10 timed steps, at least 3 warm-up
    steps) with the SM clocks sampled while it runs."""
    import torch

    steps, warmup = max(1, min(args.steps, 10)), max(3, min(args.warmup, 5))
    out = {}
    for key, fn, keep in (
            ("torus_fwd_bwd", torus_form, ("fwd_bwd_over_fwd", "target_fwd_bwd_over_fwd", "forward_only",
                                           "backward_only")),
            ("batched", batched_form, ("speedup_vs_per_mesh", "target_speedup", "per_mesh_launches",
                                       "max_rel_diff_batched_vs_per_mesh", "autotuned")),
            ("dynamic", dynamic_form, ("build_ms", "rebuild_ms"))):
        torch.cuda.synchronize()
        clocks = ClockSampler(torch.cuda.current_device())
        f = fn(steps, warmup)
        torch.cuda.synchronize()
        clk = clocks.stop()
        entry = {k: f[k] for k in ("metric", "value", "unit", "ms_per_step", "steps", "warmup") if k in f}
        entry["workload"] = f["config"]["workload"]
        entry.update({k: f[k] for k in keep if k in f})
        entry["clocks"] = clk
        out[key] = entry
        torch.cuda.empty_cache()
    out["dynamic"]["ms_per_iteration"] = out["dynamic"]["ms_per_step"]
    return out


def small_arm(args):
    """The small CPU-runnable configuration on the GPU (binary BVH, leaf 4)."""
    import torch

    import gpurt_cpq as cpq
    from gpurt_cpq import workloads as W

    dev = torch.device("cuda", 0)
    v, t, q = W.small()
    vd, td, qd = (torch.from_numpy(x).to(dev) for x in (v, t, q))
    mesh = cpq.Mesh(vd, td, branching=2, leaf_size=4)
    o = cpq.query_opts()
    ws = torch.empty(mesh.workspace_size(qd.shape[0], o), dtype=torch.uint8, device=dev)
    out = mesh.query(qd, workspace=ws, opts=o)
    ms = _timed(torch, lambda: mesh.query(qd, workspace=ws, opts=o, out=out), args.steps, args.warmup)
    _line("closest-point queries/s (small: icosphere 5,120 tris, 65,536 queries)",
          qd.shape[0] / (ms * 1e-3), "queries/s", ms, args,
          {"workload": "icosphere level 4, 65,536 queries U[-2,2]^3", "branching": 2, "leaf_size": 4},
          {})


def scene_arm(args):
    """Instanced scene (cp_scene_query): 4,096 similarity-placed instances of
    three meshes on a 16^3 grid, 16M queries (half near the surfaces), against
    the same scene flattened into one world-space mesh (cp_query)."""
    import torch

    import gpurt_cpq as cpq
    from gpurt_cpq import workloads as W

    dev = torch.device("cuda", 0)
    meshes, inst_mesh, T, q = W.instanced_scene()
    nq = q.shape[0]
    wv, wt = W.flatten_instances(meshes, inst_mesh, T)
    V, voff, TT, toff, _, _ = W.concat_batch([(v, t, None) for v, t in meshes],
                                             [np.zeros((0, 3), np.float32)] * len(meshes))
    batch = cpq.Batch(torch.from_numpy(V).to(dev), voff, torch.from_numpy(TT).to(dev), toff,
                      branching=4, leaf_size=4)
    scene = cpq.Scene(batch, inst_mesh, T)
    qd = torch.from_numpy(q).to(dev)
    o = cpq.query_opts()
    ws = torch.empty(scene.workspace_size(nq, o), dtype=torch.uint8, device=dev)
    r = scene.query(qd, workspace=ws, opts=o)
    ms_s = _timed(torch, lambda: scene.query(qd, workspace=ws, opts=o), args.steps, args.warmup)
    flat = cpq.Mesh(torch.from_numpy(wv).to(dev), torch.from_numpy(wt).to(dev), branching=4, leaf_size=4)
    wsf = torch.empty(flat.workspace_size(nq, o), dtype=torch.uint8, device=dev)
    out = flat.query(qd, workspace=wsf, opts=o)
    ms_f = _timed(torch, lambda: flat.query(qd, workspace=wsf, opts=o, out=out), args.steps, args.warmup)
    diff = float((r.dist - out.dist).abs().max())
    # moving every instance: rebuild (cp_scene_update) against refit (cp_scene_refit)
    T2 = T.copy()
    T2[:, :, 3] += np.float32(0.25)
    upd_ms, refit_ms = [], []
    for _ in range(3):
        t0 = time.perf_counter()
        scene.update(T2 if len(upd_ms) % 2 == 0 else T)
        upd_ms.append((time.perf_counter() - t0) * 1e3)
        t0 = time.perf_counter()
        scene.refit(T if len(refit_ms) % 2 == 0 else T2)
        refit_ms.append((time.perf_counter() - t0) * 1e3)
    scene.update(T)
    # rays from the query points in seeded random directions, through the
    # instances (cp_scene_ray_query) and through the flattened mesh
    rd = np.random.default_rng(17).normal(size=q.shape).astype(np.float32)
    rd /= np.linalg.norm(rd, axis=1, keepdims=True)
    rdd = torch.from_numpy(rd).to(dev)
    rs = scene.ray_query(qd, rdd)
    ms_rs = _timed(torch, lambda: scene.ray_query(qd, rdd), args.steps, args.warmup)
    rf = flat.ray_query(qd, rdd)
    ms_rf = _timed(torch, lambda: flat.ray_query(qd, rdd), args.steps, args.warmup)
    both = torch.isfinite(rf.t) & torch.isfinite(rs.t)
    # rays grazing an edge may hit in one geometry and pass on in the other
    # (the flattened mesh's vertices are rounded copies): count them
    ray_t_off = float((((rs.t - rf.t).abs() / rf.t.abs().clamp_min(1.0))[both] > 1e-4).float().mean())
    _line("instanced-scene closest-point queries/s (4,096 instances, 16M queries)", nq / (ms_s * 1e-3),
          "queries/s", ms_s, args,
          {"workload": "4,096 similarity instances (random rotation, scale 0.6-1.2) of icosphere L4 / "
                       "torus 100x40 / heightfield 64^2 on a 16^3 grid of pitch 3 (%d tris placed); "
                       "16,777,216 queries, half uniform over the grid, half N(0, 0.02) off the surfaces"
                       % wt.shape[0],
           "branching": 4, "leaf_size": 4},
          {"flattened_mesh": {"value": nq / (ms_f * 1e-3), "ms_per_step": ms_f, "tris": int(wt.shape[0]),
                              "note": "world vertices rounded to FP32 (up to 2^-24 of coordinates <= 47); "
                                      "the scene places the exact FP32 object vertices"},
           "max_abs_diff_vs_flattened": diff,
           "instance_update_ms": {"rebuild": min(upd_ms), "refit": min(refit_ms)},
           "rays": {"value": nq / (ms_rs * 1e-3), "unit": "rays/s", "ms_per_step": ms_rs,
                    "flattened_mesh": {"value": nq / (ms_rf * 1e-3), "ms_per_step": ms_rf},
                    "hit_fraction": float(torch.isfinite(rs.t).float().mean()),
                    "hit_fraction_flattened": float(torch.isfinite(rf.t).float().mean()),
                    "frac_hits_t_off_by_1e-4_vs_flattened": ray_t_off}})


def camera_arm(args):
    """The reference's own render loop on its own scene: one primary ray per
    pixel through the Cornell box's instances (trace_ray against the TLAS,
    rt.rgen:551-565 make_camera_ray, 257-270), then one shadow ray per hit to
    a point on the ceiling light (visibility, rt.rgen:272-291, as
    integrate_direct uses it).  The scene comes from the committed fixture of
    media/cbox/cbox.gltf; 1920 x 1440 pixels."""
    import torch

    import gpurt_cpq as cpq
    from gpurt_cpq import workloads as W

    dev = torch.device("cuda", 0)
    g = np.load(ROOT / "tests" / "golden" / "cbox_scene.npz")
    batch = cpq.Batch(torch.from_numpy(g["verts"]).to(dev), g["vert_offsets"], torch.from_numpy(g["tris"]).to(dev),
                      g["tri_offsets"], branching=4, leaf_size=4)
    scene = cpq.Scene(batch, g["instance_primitive"], g["instance_transform"])
    w, h = 1920, 1440
    o, d = W.camera_rays(w, h, W.CBOX_EYE, W.CBOX_YFOV, W.CBOX_ASPECT)
    od, dd = torch.from_numpy(o).to(dev), torch.from_numpy(d).to(dev)
    n = od.shape[0]
    prim = scene.ray_query(od, dd)
    ms_p = _timed(torch, lambda: scene.ray_query(od, dd), args.steps, args.warmup)
    # shadow rays: from each hit to a seeded point on the light's lower face
    li = W.CBOX_LIGHT_INSTANCE
    m = int(g["instance_primitive"][li])
    lv = g["verts"][g["vert_offsets"][m]:g["vert_offsets"][m + 1]].astype(np.float64)
    t34 = g["instance_transform"][li].astype(np.float64)
    wl = lv @ t34[:, :3].T + t34[:, 3]
    lo, hi = wl.min(0), wl.max(0)
    rng = np.random.default_rng(21)
    tgt = np.stack([rng.uniform(lo[0], hi[0], n), np.full(n, lo[1]), rng.uniform(lo[2], hi[2], n)], -1)
    hit = torch.isfinite(prim.t)
    so = (od + dd * prim.t.clamp_max(1e30)[:, None])[hit].contiguous()
    sd = (torch.from_numpy(tgt.astype(np.float32)).to(dev)[hit] - so).contiguous()
    ns = so.shape[0]
    seg = torch.full((ns,), 1.0 - 1e-4, device=dev)
    sopts = cpq.ray_opts(any_hit=True, tmin=1e-4)
    shadow = scene.ray_query(so, sd, tmax_per_ray=seg, opts=sopts)
    ms_s = _timed(torch, lambda: scene.ray_query(so, sd, tmax_per_ray=seg, opts=sopts), args.steps, args.warmup)
    frame_ms = ms_p + ms_s
    _line("Cornell box frame: primary + shadow rays/s through its instances", (n + ns) / (frame_ms * 1e-3),
          "rays/s", frame_ms, args,
          {"workload": f"media/cbox/cbox.gltf (fixture: 9 primitives, 10 instances, {len(g['tris']):,} tris), "
                       f"{w}x{h} primary rays from its camera, one shadow ray per hit to its ceiling light",
           "branching": 4, "leaf_size": 4},
          {"primary": {"value": n / (ms_p * 1e-3), "ms_per_step": ms_p, "rays": n,
                       "hit_fraction": float(hit.float().mean())},
           "shadow": {"value": ns / (ms_s * 1e-3), "ms_per_step": ms_s, "rays": ns,
                      "occluded_fraction": float(torch.isfinite(shadow.t).float().mean())}})


def cbox_shading_arrays(g) -> dict:
    """The Cornell box fixture (media/cbox/cbox.gltf's primitives and
    instances) flattened to world space for the path tracer: each instance
    one object, vertices through its matrix, normals through the inverse
    transpose, the primitive's material factors."""
    V, N, obj, al, em, mr = [], [], [], [], [], []
    voff, toff = g["vert_offsets"], g["tri_offsets"]
    for i, (j, T) in enumerate(zip(g["instance_primitive"], g["instance_transform"])):
        M = T.astype(np.float64)
        tri = g["tris"][toff[j]:toff[j + 1]]
        V.append((g["verts"][voff[j]:voff[j + 1]].astype(np.float64) @ M[:, :3].T + M[:, 3])[tri])
        N.append((g["normals"][voff[j]:voff[j + 1]].astype(np.float64) @ np.linalg.inv(M[:, :3]))[tri])
        obj.append(np.full(len(tri), i, np.int32))
        al.append(g["prim_albedo"][j])
        em.append(g["prim_emissive"][j])
        mr.append(g["prim_metal_rough"][j])
    f32 = lambda a: np.ascontiguousarray(np.asarray(a), np.float32)  # noqa: E731
    return {"verts": f32(np.concatenate(V)).reshape(-1, 9), "normals": f32(np.concatenate(N)).reshape(-1, 9),
            "obj": np.concatenate(obj), "albedo": f32(al), "emissive": f32(em), "metal_rough": f32(mr)}


def shade_arm(args):
    """The reference's path tracer on its own scene: the Cornell box from its
    camera at 1920 x 1440, the reference's defaults (8 samples per pixel,
    depth 8, Russian roulette, Blinn-Phong), MIS; one frame per step.  The
    CPU baseline renders a 320 x 240 frame of the same view with the
    restatement of the same shaders on all host cores."""
    import torch

    from gpurt_cpq import shading as G

    dev = torch.device("cuda", 0)
    g = np.load(ROOT / "tests" / "golden" / "cbox_scene.npz")
    sa = cbox_shading_arrays(g)
    td = {k: torch.from_numpy(v).to(dev) for k, v in sa.items()}
    scene = G.ShadeScene(td["verts"], td["normals"], td["obj"], td["albedo"], td["emissive"], td["metal_rough"])
    from gpurt_cpq import workloads as W

    w, h, spp = args.width, args.height, 8
    target = (W.CBOX_EYE[0], W.CBOX_EYE[1], 0.0)
    cam = G.camera(W.CBOX_EYE, target, (0, 1, 0), W.CBOX_YFOV, w, h)
    img = torch.zeros((h, w, 3), dtype=torch.float32, device=dev)
    from gpurt_cpq._lib import lib

    def frame(integrator):
        scene.render(cam, integrator=integrator, samples=spp, max_depth=8, seed=7, image=img)

    frame(G.MIS)
    launches0 = lib.cp_kernel_launches()
    ms = _timed(torch, lambda: frame(G.MIS), args.steps, args.warmup)
    launches = (lib.cp_kernel_launches() - launches0) // (args.steps + args.warmup)
    ms_restir = _timed(torch, lambda: frame(G.RESTIR), args.steps, args.warmup)
    mean = float(img.mean())
    cpu = None
    if not args.no_cpu_baseline:
        from oracle import shade as S

        sw, sh_ = 320, 240
        osc = S.Scene(sa["verts"], sa["normals"], sa["obj"], sa["albedo"], sa["emissive"], sa["metal_rough"])
        ocam = S.camera(W.CBOX_EYE, target, (0, 1, 0), W.CBOX_YFOV, sw, sh_)
        t0 = time.perf_counter()
        osc.render(ocam, integrator=S.MIS, samples=spp, max_depth=8, seed=7)
        secs = time.perf_counter() - t0
        cpu = {"value": sw * sh_ * spp / secs, "unit": "samples/s", "cores": host_cores(), "kind": "port",
               "sample": f"one {sw}x{sh_} frame of the same view, {spp} samples per pixel, MIS, the restatement "
                         f"of the reference's shaders (equal to them bit for bit) on all host cores, "
                         f"brute-force scene tracing, {cpu_model()}"}
    extra = {"restir": {"value": w * h * spp / (ms_restir * 1e-3), "ms_per_step": ms_restir},
             "gpu_launches_per_frame": int(launches), "mean_radiance": mean}
    if cpu is not None:
        extra["cpu_baseline"] = cpu
    _line(f"path-traced samples/s (the reference's Cornell box, {w}x{h}, MIS, 8 spp, depth 8)",
          w * h * spp / (ms * 1e-3), "samples/s", ms, args,
          {"workload": f"media/cbox/cbox.gltf (fixture: {sa['verts'].shape[0]:,} world-space tris, 10 objects, "
                       f"1 light) from its camera, {w}x{h}, {spp} samples per pixel, max depth 8, Russian "
                       "roulette, Blinn-Phong, MIS; one frame per step",
           "integrator": "MIS"}, extra)


def main():
    args = parse()
    if args.impl == "reference":
        reference_arm(args)
    elif args.workload == "large":
        our_arm(args)
    else:
        {"torus": torus_arm, "batched": batched_arm, "dynamic": dynamic_arm,
         "small": small_arm, "rays": rays_arm, "scene": scene_arm,
         "camera": camera_arm, "shade": shade_arm}[args.workload](args)


if __name__ == "__main__":
    main()
