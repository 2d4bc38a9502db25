#!/usr/bin/env python3
"""Benchmark of the GB300 stress solve.

Default (--workload serve): the serving configuration the metric is quoted on. A seeded Poisson
stream of solve requests (5,000/s; sizes log-normal, median 500 fragments, 10-50,000; 30 % repeats
of a recent structure with 1-5 % of its bonds removed, warm-started) through the library's server:
each request's K assembled (or downdated in place), its multigrid built, PCG to rel. residual 1e-6
under the mixed-precision policy, and every bond's fibre-stress check. The stream has --requests
requests (20,000, the configuration's) or 1,000 a step if more; one step = requests / K of them.

  value   solves/s with the requests' graphs and loads already in device memory
  e2e     solves/s of the same stream from host arrays through the C ABI (graph and load copied in,
          results out), the headline against the reference arm
  p50/p99 request latency (submission -> result), also at 70 % of the measured capacity
  plain_fp64_per_request  the plain FP64 drop-in, one request after another (FP64 PCG per
          structure), over every eighth structure of the same stream with all its repeats
  cpu_baseline  the oracle (a C restatement of the reference's solve) on the host's cores, one
          single-threaded process per core (the reference's one small graph per pool thread)

--workload city: one complete solve of the city block per step (seeded towers of 5-40 storeys,
four jittered materials; FP64 PCG to rtol 1e-8), value device-resident, e2e through the C ABI with
host buffers, and the conjugate-gradient SpMV's roofline timed live with CUDA events (launches
that did work) against the measured HBM bandwidth and this GPU's measured FP64 FMA rate.

Launch: python bench.py [--gpus N --steps K --warmup W] (N > 1 under torchrun: one replica per
GPU, each with its own seeded stream or city block; value = all ranks' solves / the slowest rank's
time). --workload batch | cascade | sections | pieces run the batched solve, the judge's break
rounds, bonds from voxel faces and loose pieces' break rounds.
--impl reference times the reference's CPU implementation of the path (the oracle port on every
host core) on the same workload and prints the same JSON line.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

METRIC = "stress solves/sec & p99 latency at rel.resid 1e-6 vs plain FP64 PCG, 1 GB300"
L2_BYTES = 129 * 2**20


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def measured_peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            d = json.load(fh)
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def workload(args, rank: int):
    from opus_destruct_2_gb300 import synth
    if args.workload == "city":
        nodes, bonds, f, mats = synth.city_graph(lots_x=args.lots, lots_y=args.lots, seed=args.seed + rank)
        desc = (f"city block: {args.lots}x{args.lots} seeded towers of 5-40 storeys, 0.5 m voxels, concrete/steel/"
                f"masonry/wood +-20%")
    else:
        nodes, bonds, f, mats = synth.tower_graph(storeys=10, seed=args.seed + rank)
        desc = "tower: 10 storeys, 8 x 8 m plan, 0.5 m voxels, concrete E = 30 GPa"
    return nodes, bonds, f, mats, desc


# setup phases by the library's boundary labels (svxg_phase_times)
SETUP_GROUPS = {
    "assemble: DOF numbering": "K", "assemble: incidences": "K", "assemble: pattern": "K",
    "assemble: block values": "K", "K assembled": "K",
    "level 0 finalized": "level finalize (D^-1, FP32 copies)", "level coarsened": "level finalize (D^-1, FP32 copies)",
    "coarsen: aggregated": "aggregation", "coarsen: positions": "coarse positions",
    "coarsen: lmax": "lambda_max (power iteration)", "coarsen: prolongation": "prolongation",
    "coarsen: restriction lists": "restriction lists", "coarsen: A P": "Galerkin A P",
    "coarsen: coarse pattern": "Galerkin pattern", "coarsen: coarse values": "Galerkin P^T (A P)",
    "coarsest factored": "coarsest factor", "preconditioner built": "other",
}


def setup_phases(L, h, check) -> dict:
    """Milliseconds per setup phase of the last assemble (summed over levels), and per level."""
    from opus_destruct_2_gb300.graph import PhaseTime
    cnt = ctypes.c_int32()
    out = (PhaseTime * 512)()
    check(L.svxg_phase_times(h, out, 512, ctypes.byref(cnt)))
    groups: dict[str, float] = {}
    levels: list[float] = []
    cur = 0.0
    for i in range(min(cnt.value, 512)):
        label, ms = out[i].label.decode(), float(out[i].ms)
        g = SETUP_GROUPS.get(label, "other")
        groups[g] = groups.get(g, 0.0) + ms
        if g != "K":
            cur += ms
        if label in ("level 0 finalized", "level coarsened"):
            levels.append(cur)
            cur = 0.0
    return {"total": sum(groups.values()), "phases": groups, "per_level": levels,
            "how": "CUDA events on the problem's stream at each phase boundary of one assemble (no host waits)"}


class Clocks:
    """nvidia-smi samples (200 ms) during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.proc = None
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(index)], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self) -> dict | None:
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx = max(mx, float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def max_over_ranks(x: float, dist, device) -> float:
    """The largest x over the ranks (the slowest rank's time); x itself without a process group.
    `device`: where the collective's tensor lives (a CUDA device for NCCL, the CPU for gloo)."""
    if dist is None:
        return float(x)
    import torch
    t = torch.tensor([float(x)], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_reference(args, rank: int, world: int):
    """The reference's CPU implementation of the path: the oracle port, every host thread."""
    if rank != 0:
        return
    if args.workload == "serve":
        run_reference_serve(args, world)
        return
    import oracle
    from opus_destruct_2_gb300.graph import StressOptions
    nodes, bonds, f, mats, desc = workload(args, 0)
    threads = os.cpu_count() or 1
    oracle.set_threads(threads)
    times = []
    iters = 0
    for step in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        P = oracle.Port(nodes, bonds, mats)
        P.assemble(StressOptions(amg_min_nodes=160))
        u, res = P.solve(f, rtol=args.rtol, maxit=args.maxit)
        P.judge(u)
        dt = time.perf_counter() - t0
        if step >= args.warmup:
            times.append(dt)
        iters = res.iters
    total = sum(times)
    value = len(times) / total
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": desc, "nodes": int(len(nodes)), "bonds": int(len(bonds)), "rtol": args.rtol,
                   "pcg_iters": int(iters)},
        "cpu_baseline": {"value": value, "unit": "solves/s", "cores": threads, "kind": "port",
                         "sample": "each step: one full solve (assemble + multigrid build + PCG + judge) of the "
                                   "workload graph by the oracle's C restatement of the reference (the reference "
                                   "tree is not on this machine)"},
        "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "p50_ms": 1e3 * float(np.percentile(times, 50)), "p99_ms": 1e3 * float(np.percentile(times, 99)),
    }
    print(json.dumps(line), flush=True)


def cpu_baseline(args, nodes, bonds, f, mats) -> dict:
    import oracle
    from opus_destruct_2_gb300.graph import StressOptions
    threads = os.cpu_count() or 1
    oracle.set_threads(threads)
    t0 = time.perf_counter()
    P = oracle.Port(nodes, bonds, mats)
    P.assemble(StressOptions(amg_min_nodes=160))
    u, res = P.solve(f, rtol=args.rtol, maxit=args.maxit)
    P.judge(u)
    dt = time.perf_counter() - t0
    return {"value": 1.0 / dt, "unit": "solves/s", "cores": threads, "kind": "port",
            "sample": f"one full solve (assemble + multigrid build + PCG to rtol {args.rtol:g} + judge) of the "
                      f"workload graph by the oracle's C restatement of the reference; {dt:.2f} s, "
                      f"{res.iters} PCG iterations"}


def _cpu_serve_init():
    import oracle
    oracle.set_threads(1)


def _cpu_serve_noop(_):
    return 0


def _cpu_serve_run(job):
    """One structure's requests on the CPU, in arrival order: the first assembled and solved cold,
    each repeat removing its bonds and solving warm on the kept problem (the oracle restatement, one
    thread), each judged. Returns (requests done, converged)."""
    import oracle
    from opus_destruct_2_gb300.graph import StressOptions, default_materials
    nodes, bonds, f, removals, rtol = job
    P = oracle.Port(nodes, bonds, default_materials())
    P.assemble(StressOptions())
    u, res = P.solve(f, rtol=rtol, maxit=2000)
    P.judge(u)
    done, conv = 1, int(res.converged)
    for rm in removals:
        for b in rm:
            P.remove_bond(int(b))
        u, res = P.solve(f, u=u, rtol=rtol, maxit=2000, warm=True)
        P.judge(u)
        done += 1
        conv += int(res.converged)
    return done, conv


def cpu_jobs(stream, indices, rtol: float) -> dict:
    """The requests `indices` grouped by structure (a structure's new request, then its repeats'
    removals, in arrival order): {structure id: job}."""
    jobs = {}
    for k in indices:
        kind, sid, g, rm = stream.plan[k]
        if kind == "new":
            nodes, bonds, f = stream.geoms[g]
            jobs[sid] = (nodes, bonds, f, [], rtol)
        elif sid in jobs:
            jobs[sid][3].append(rm)
    return jobs


def cpu_pool(cores: int):
    import multiprocessing as mp
    pool = mp.get_context("spawn").Pool(cores, initializer=_cpu_serve_init)
    pool.map(_cpu_serve_noop, range(cores))  # (workers up)
    return pool


def cpu_serve(pool, job_list) -> tuple:
    """The reference's arrangement for many small graphs (world_pieces.cpp:1460-1463): one graph per
    thread, all cores at once - here one single-threaded oracle process per core, a structure's
    requests on one process. Returns (requests, converged, seconds)."""
    t0 = time.perf_counter()
    out = list(pool.imap_unordered(_cpu_serve_run, job_list, chunksize=1))
    return sum(o[0] for o in out), sum(o[1] for o in out), time.perf_counter() - t0


SERVE_DESC = ("serving: Poisson stream of {req} requests at {rate:g}/s, sizes log-normal (median 500 fragments, "
              "10-50,000), half free pieces (inertial relief, pinned) and half ground-supported, 30% repeats of "
              "one of the 256 latest structures with 1-5% of its bonds removed (warm start), 40 GB admission "
              "budget, rel. residual {rtol:g}")


def _serve_bytes(stream, way: str) -> int:
    """Bytes a host-input run copies per stream: graph records, materials and load in (new), load
    and removal list in (repeat); the request's result out (64 bytes; no u, no failure list)."""
    from opus_destruct_2_gb300.graph import MATERIAL_DTYPE
    tot = 0
    for kind, sid, g, rm in stream.plan:
        nodes, bonds, f = stream.geoms[g]
        if way == "h2d":
            tot += f.nbytes + (nodes.nbytes + bonds.nbytes + len(stream.mats) * MATERIAL_DTYPE.itemsize
                               if kind == "new" else 4 * len(rm))
        else:
            tot += 64
    return tot


def run_serve(args, rank: int, world: int):
    """The serving configuration: a Poisson stream of solve requests through the server (slots
    overlap requests on the device, queued new requests run in batches, kept batches serve their
    structures' repeats), each request's graph assembled, solved to rtol 1e-6 and judged. The stream:
    max(--requests, 1000 x steps) requests, one step = requests / steps of them; warm-up = 100
    requests a warm-up step on the same server before the timed stream.

      value   solves/s with every request's graph, materials and load already in device memory
              (svxg_server_submit_device)
      e2e     solves/s of the same stream from host arrays (svxg_server_submit / _repeat)
      plain   the plain FP64 drop-in per request (one StressProblem at a time, FP64 PCG) over every
              eighth structure of the same stream with all its repeats
      cpu_baseline  the oracle on the host's cores (one single-threaded process per core, the
              reference's arrangement for many small graphs) over the first requests of the stream
    """
    os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")
    import torch
    from opus_destruct_2_gb300 import load_library, workloads
    from opus_destruct_2_gb300.graph import PRECISION_FP64, PRECISION_MIXED, PRECISION_MIXED_ALL
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    L = load_library()
    L.svxg_launch_count.restype = ctypes.c_int64
    prec = {"fp64": PRECISION_FP64, "mixed": PRECISION_MIXED, "mixed-all": PRECISION_MIXED_ALL}[args.precision]
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    # (the configuration's stream of --requests requests, 20,000 by default, in K steps; at least
    # 1,000 requests a step)
    requests = max(args.requests, 1000 * args.steps)
    stream = workloads.Stream(requests=requests, rate=args.rate, seed=args.seed + 9 + rank)
    staged = workloads.DeviceGeometries(stream, local)
    kw = dict(workers=args.workers, precision=prec, rtol=args.rtol, warmup=100 * args.warmup)
    if args.batch_graphs is not None:
        kw["batching"] = (args.batch_graphs, 20000, 65536)
    # value: device-resident inputs
    if dist is not None:
        dist.barrier()
    clocks = Clocks(local)
    dev = workloads.serve_stream(stream, inputs="device", staged=staged, **kw)
    clk = clocks.stop()
    # e2e: host inputs, the same stream
    host = workloads.serve_stream(stream, inputs="host", **kw)
    # latency without a growing queue: the first quarter of the stream offered at 70 % of capacity
    sustained = 0.7 * dev["solves_per_s"]
    at70 = None
    if sustained < args.rate:
        at70 = workloads.serve_stream(stream, inputs="device", staged=staged, rate=sustained,
                                      indices=range(max(1000, requests // 4)), **kw)
    plain = workloads.plain_stream(stream, stream.subset(8), rtol=args.rtol)
    wall = max_over_ranks(dev["wall_s"], dist, "cpu")
    fewest = -max_over_ranks(-dev["completed"], dist, "cpu")  # (the fewest completed over ranks)
    if rank != 0:
        return
    cpu = None
    if not args.no_cpu_baseline:
        cores = os.cpu_count() or 1
        jobs = list(cpu_jobs(stream, range(min(requests, 2000)), args.rtol).values())
        with cpu_pool(cores) as pool:
            done, conv, dt = cpu_serve(pool, jobs)
        cpu = {"value": done / dt, "unit": "solves/s", "cores": cores, "kind": "port", "converged": conv,
               "sample": f"the structures of the first 2000 requests of the same stream with their repeats "
                         f"({done} requests), one single-threaded oracle process per core (the reference's one "
                         f"small graph per pool thread); {dt:.1f} s"}
    keys = ("solves_per_s", "p50_ms", "p99_ms", "new_p50_ms", "new_p99_ms", "repeat_p50_ms", "repeat_p99_ms",
            "p99_ms_8k_12k_dof", "requests_8k_12k_dof", "offered_rate", "completed", "failed_or_unconverged",
            "batches", "batched_requests", "pcg_iters_mean")
    line = {
        "metric": METRIC, "value": world * fewest / wall, "unit": "solves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * wall / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if prec == PRECISION_FP64 else "f32+f64", "data": "synthetic",
        "config": {"workload": SERVE_DESC.format(req=requests, rate=args.rate, rtol=args.rtol),
                   "requests": requests, "workers": args.workers, "rtol": args.rtol,
                   "precision": ("fp64" if prec == PRECISION_FP64 else
                                 "mixed policy: fp32 V-cycle, multigrid built with FMAs and a tree-summed "
                                 "power-iteration norm, fp64 K and Krylov vectors"),
                   "step": f"{requests / args.steps:g} requests of the stream: each assembled (or bonds "
                           f"removed in place), solved, judged",
                   "l2": "the stream's requests together exceed L2 (tens of GB admitted)",
                   "parallelism": f"replicas x{world}, {args.workers} server slots, new requests in batches "
                                  f"of <= {args.batch_graphs or 16} graphs"},
        "p50_ms": dev["p50_ms"], "p99_ms": dev["p99_ms"],
        "block_row_iterations_per_s": world * dev["block_row_iterations_per_s"],
        "serve": {k: dev[k] for k in keys}, "serve_at_70pct": ({k: at70[k] for k in keys} if at70 else None),
        "plain_fp64_per_request": plain, "vs_plain_fp64": dev["solves_per_s"] / plain["solves_per_s"],
        "e2e": {"value": world * host["solves_per_s"], "unit": "solves/s",
                "h2d_bytes_per_step": int(_serve_bytes(stream, "h2d") / args.steps),
                "d2h_bytes_per_step": int(_serve_bytes(stream, "d2h") / args.steps),
                "p50_ms": host["p50_ms"], "p99_ms": host["p99_ms"]},
        "gpu_launches": dev["launches"],
        "gpu_launches_in_graphs": dev["launches_in_graphs"],
        "host_launches_per_s": dev["host_launches_per_s"],
        "roofline": serve_roofline(stream, L, local),
    }
    if cpu is not None:
        line["cpu_baseline"] = cpu
    if clk is not None:
        line["clocks"] = clk
    print(json.dumps(line), flush=True)


def serve_roofline(stream, L, device: int) -> dict:
    """The serving step's dominant kernel by device time - the multigrid build's Galerkin A P values
    kernel (FP64 6x6 block products in the reference's summation order; the mixed-precision
    policy's build contracts them into FMAs) - timed with CUDA events on its problem's stream over
    five assembles of a typical batch of the stream (its first 16 new structures as one problem,
    as the server batches them), against this GPU's FP64 rate measured in the same run."""
    from opus_destruct_2_gb300 import Batch
    from opus_destruct_2_gb300.graph import StressOptions
    L.svxg_timer_enable_kernel.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32]
    L.svxg_timer_read_work.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double),
                                       ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64)]
    L.svxg_measure_fp64_rate.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
    news = [stream.geoms[p[2]] for p in stream.plan if p[0] == "new"][:16]
    B = Batch([(g[0], g[1]) for g in news], stream.mats, device=device)
    opt = StressOptions(precision=1)
    B.assemble(opt)
    L.svxg_timer_enable_kernel(B._h, 1, 1)
    for _ in range(5):
        B.assemble(opt)
    ms, launches, work = ctypes.c_double(), ctypes.c_int64(), ctypes.c_int64()
    L.svxg_timer_read_work(B._h, ctypes.byref(ms), ctypes.byref(launches), ctypes.byref(work))
    L.svxg_timer_enable_kernel(B._h, 1, 0)
    rate = ctypes.c_double()
    L.svxg_measure_fp64_rate(device, ctypes.byref(rate))
    flops = 432.0 * work.value  # (36 entries x 12 flops - 6 products, 5 sums, 1 accumulate - per block product)
    achieved = flops / (ms.value / 1e3) / 1e12 if ms.value > 0 else 0.0
    # (the fast build takes an entry's 12 flops as 7 FP64 instructions: a multiply, 5 FMAs and the
    # accumulating add; issue_frac is the fraction of the FP64 instruction rate those instructions use)
    instr_per_flop = 7.0 / 12.0
    return {"kernel": "Galerkin A P values of the mixed-precision policy's multigrid build (k_ap_values_acc on levels "
                      "of many rows, k_ap_values_warp on levels of <= 2,432 rows): FP64 6x6 block products in the "
                      "reference's summation order, as FMAs", "bound": "fp64",
            "achieved": achieved, "peak": rate.value, "unit": "TFLOP/s",
            "frac": achieved / rate.value if rate.value > 0 else None,
            "issue_frac": 2.0 * instr_per_flop * achieved / rate.value if rate.value > 0 else None,
            "peak_source": "this GPU's FP64 FMA rate measured in this run (an FMA = 2 flops); issue_frac: the FP64 "
                           "instructions executed (7 per 12-flop entry) against the FP64 instruction rate (half of it)",
            "traffic": None, "flops_per_launch": flops / max(launches.value, 1), "launches": int(launches.value),
            "avg_us": 1e3 * ms.value / max(launches.value, 1),
            "workload": f"one batch of the stream's first 16 new structures ({sum(len(g[0]) for g in news)} "
                        f"fragments), 5 assembles, every level's launch",
            "how": "CUDA events around each launch on the problem's stream; algorithmic FP64 operations from the "
                   "block products counted on the host (the reference's build-work count of A P / 6)",
            "traffic_note": "no HBM figure: the operands come from L1/L2 (ncu on levels 1 and 2 of this batch: "
                            "12.2 and 7.5 MB of DRAM reads in 320 and 160 us, profiles/galerkin_batch32_ncu.md)"}


def run_reference_serve(args, world: int):
    """The serving stream on the reference's CPU path: the oracle port on every host core, one
    single-threaded process per core (the reference's one small graph per pool thread), each
    structure's requests in arrival order on one process. Step i: the structures s of the stream
    with s mod (warmup + steps) = i, with all their requests; the first `warmup` steps untimed."""
    from opus_destruct_2_gb300 import workloads
    requests = max(args.requests, 1000 * args.steps)
    stream = workloads.Stream(requests=requests, rate=args.rate, seed=args.seed + 9)
    jobs = cpu_jobs(stream, range(requests), args.rtol)
    cores = os.cpu_count() or 1
    k_all = args.warmup + args.steps
    done = conv = 0
    secs = 0.0
    with cpu_pool(cores) as pool:
        for step in range(k_all):
            part = [j for sid, j in jobs.items() if sid % k_all == step]
            d, c, dt = cpu_serve(pool, part)
            if step >= args.warmup:
                done, conv, secs = done + d, conv + c, secs + dt
    value = done / secs
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * secs / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": SERVE_DESC.format(req=requests, rate=args.rate, rtol=args.rtol),
                   "requests": requests, "rtol": args.rtol, "timed_requests": done, "converged": conv},
        "cpu_baseline": {"value": value, "unit": "solves/s", "cores": cores, "kind": "port",
                         "sample": f"each step: the structures of the stream in one residue class of "
                                   f"{k_all} with all their requests ({done} timed requests in all), one "
                                   f"single-threaded oracle process per core (the reference tree is not on "
                                   f"this machine: the oracle's C restatement)"},
        "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_many(args, rank: int, world: int):
    """The batched solve (opus_destruct_2_gb300/workloads.py) on this GPU."""
    # (more hardware queues for the server's streams; read when the CUDA context is created)
    os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")
    from opus_destruct_2_gb300 import workloads
    from opus_destruct_2_gb300.graph import PRECISION_FP64, PRECISION_MIXED, PRECISION_MIXED_ALL
    prec = {"fp64": PRECISION_FP64, "mixed": PRECISION_MIXED, "mixed-all": PRECISION_MIXED_ALL}[args.precision]
    clocks = Clocks(int(os.environ.get("LOCAL_RANK", "0")))
    r = workloads.batch(count=args.graphs, workers=args.workers, precision=prec, rtol=args.rtol,
                        steps=min(args.steps, 5), warmup=args.warmup)
    desc = (f"batch: {args.graphs} fragment graphs, log-normal sizes (median 300, 10-20,000), half free pieces "
            f"with inertial relief, half ground-supported, gravity + one impact load; rtol {args.rtol:g}")
    clk = clocks.stop()
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": r["solves_per_s"] * world, "unit": "solves/s", "n_gpus": world,
        "steps": r["passes"], "warmup": r["warmup_passes"], "ms_per_step": 1e3 * r["wall_s"] / r["passes"],
        "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64" if prec == PRECISION_FP64 else "f32+f64", "data": "synthetic",
        "config": {"workload": desc, "workers": args.workers,
                   "precision": ("fp64" if prec == PRECISION_FP64 else
                                 "mixed policy: fp32 V-cycle, fast multigrid build, fp64 K and Krylov vectors")},
        "p50_ms": r["p50_ms"], "p99_ms": r["p99_ms"], "batch": r,
        "vs_plain_fp64_per_request": r["solves_per_s"] / r["plain_fp64_per_request_solves_per_s"],
        "roofline": None,
    }
    if clk is not None:
        line["clocks"] = clk
    print(json.dumps(line), flush=True)


def _cpu_piece_init():
    import oracle
    oracle.set_threads(1)


def _cpu_piece_run(job) -> int:
    import oracle
    from opus_destruct_2_gb300.graph import PieceOptions, default_fracture_energies, default_materials
    nodes, bonds, f = job
    oracle.piece_rounds(oracle.Port(nodes, bonds, default_materials()), f, np.zeros(6 * len(nodes)), PieceOptions(),
                        default_fracture_energies())
    return 1


def run_pieces(args, rank: int, world: int):
    """A substep's loose pieces through their break rounds (svxg_batch_piece_rounds) on this GPU:
    value = pieces/s; beside it one piece after another on one problem, and the oracle's
    restatement of the rounds on the host's cores over a sample of the same pieces."""
    os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")
    from opus_destruct_2_gb300 import workloads
    clocks = Clocks(int(os.environ.get("LOCAL_RANK", "0")))
    from opus_destruct_2_gb300.graph import PRECISION_FP64, PRECISION_MIXED, PRECISION_MIXED_ALL
    prec = {"fp64": PRECISION_FP64, "mixed": PRECISION_MIXED, "mixed-all": PRECISION_MIXED_ALL}[args.precision]
    r = workloads.pieces(count=args.graphs, workers=args.workers, precision=prec, steps=args.steps,
                         warmup=args.warmup)
    clk = clocks.stop()
    if rank != 0:
        return
    cpu = None
    if not args.no_cpu_baseline:
        # the reference's arrangement for small pieces: one piece per thread, all cores at once
        # (world_pieces.cpp:1460-1463) - here one single-threaded oracle process per core
        import multiprocessing as mp
        from opus_destruct_2_gb300 import synth
        sizes = synth.lognormal_sizes(args.graphs, 300, 10, 20000, seed=5)
        rng = np.random.default_rng(6)
        jobs = []
        for k, sz in enumerate(sizes):
            imp = float(10 ** rng.uniform(4.0, 6.0)) * 20.0
            nodes, bonds, f, _ = synth.piece_graph(int(sz), free=True, seed=5 * 100003 + k, impact=imp)
            jobs.append((nodes, bonds, f))
        cores = os.cpu_count() or 1
        with mp.get_context("spawn").Pool(cores, initializer=_cpu_piece_init) as pool:
            pool.map(_cpu_piece_run, jobs[:cores])  # (workers up)
            t0 = time.perf_counter()
            done = sum(pool.imap_unordered(_cpu_piece_run, jobs, chunksize=1))
            tc = time.perf_counter() - t0
        cpu = {"value": done / tc, "unit": "pieces/s", "cores": cores, "kind": "port",
               "sample": f"all {done} pieces of the same substep, one single-threaded oracle process per core "
                         f"(the reference's one piece per pool thread)"}
    line = {
        "metric": METRIC, "value": r["pieces_per_s"] * world, "unit": "pieces/s", "n_gpus": world,
        "steps": r["substeps"], "warmup": r["warmup_substeps"], "ms_per_step": 1e3 * r["wall_s"] / r["substeps"],
        "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"precision": args.precision,
                   "workload": f"pieces: {args.graphs} free pieces of log-normal size (median 300 fragments, "
                               f"10-20,000), inertial relief plus one impact each, break rounds at the world's "
                               f"settings (rtol 1e-2, 60 iterations, 8 rounds, resting loads)",
                   "workers": args.workers},
        "pieces": r, "vs_plain_per_piece": r["pieces_per_s"] / r["plain_per_piece_pieces_per_s"],
        "roofline": None,
    }
    if cpu is not None:
        line["cpu_baseline"] = cpu
    if clk is not None:
        line["clocks"] = clk
    print(json.dumps(line), flush=True)


def run_cascade(args, rank: int, world: int):
    """The judge's break rounds of the city block (svxg_cascade): one step = assemble + every round
    (solve warm, judge, break, retire what falls) until nothing is over strength, from the same
    intact city each step, through the C ABI with host buffers. value = solves/s inside the
    cascade; the CPU baseline runs the oracle's restatement of the same rounds (bounded: the first
    rounds) on the host's cores and must break the same bonds."""
    import torch
    from opus_destruct_2_gb300 import StressProblem, load_library
    from opus_destruct_2_gb300.graph import CascadeOptions, StressOptions
    if world > 1:
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    L = load_library()
    from opus_destruct_2_gb300 import synth
    nodes, bonds, f, mats = synth.city_graph(lots_x=args.lots, lots_y=args.lots, seed=args.seed + rank)
    opt = StressOptions()
    o = CascadeOptions(rtol=args.rtol, fragility=args.fragility, maxit=args.maxit)

    def step():
        G = StressProblem(nodes, bonds, mats)
        t0 = time.perf_counter()
        if not G.assemble(opt):
            raise RuntimeError("assemble: singular")
        u, res, ex = G.cascade(f, options=o, opt=opt)
        return time.perf_counter() - t0, res, ex

    for _ in range(args.warmup):
        step()
    clocks = Clocks(int(os.environ.get("LOCAL_RANK", "0")))
    launches0 = L.svxg_launch_count()
    walls, last = [], None
    for _ in range(args.steps):
        w, res, ex = step()
        walls.append(w)
        last = (res, ex)
    launches = L.svxg_launch_count() - launches0
    clk = clocks.stop()
    res, ex = last
    wall = max(walls)
    cpu = None
    if not args.no_cpu_baseline and rank == 0:
        import oracle
        oracle.set_threads(os.cpu_count() or 1)
        rounds = 2
        P = oracle.Port(nodes, bonds, mats)
        t0 = time.perf_counter()
        P.assemble(opt)
        ro = oracle.cascade(P, f, np.zeros(6 * len(nodes)), CascadeOptions(rtol=args.rtol, fragility=args.fragility,
                                                                            maxit=args.maxit, max_rounds=rounds), opt)
        tc = time.perf_counter() - t0
        k = len(ro["broken"])
        cpu = {"value": ro["solves"] / tc, "unit": "solves/s", "cores": os.cpu_count(), "kind": "port",
               "sample": f"assemble + the first {rounds} rounds ({ro['solves']} solves, {k} bonds) of the same "
                         f"cascade, oracle restatement (C, OpenMP)",
               "wall_s": tc, "same_breaks_as_device": ex["broken"][:k] == ro["broken"]}
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": world * res.solves / wall, "unit": "solves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * wall, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"cascade: judge break rounds of the {args.lots}x{args.lots} city block (seeded towers "
                               f"of 5-40 storeys, four materials), gravity, fragility {args.fragility:g}, rtol "
                               f"{args.rtol:g}, {args.maxit} iterations a solve, world defaults (band 0.85, 256 "
                               f"breaks a round, rebuild after 60 iterations on a stale preconditioner)",
                   "nodes": int(len(nodes)), "bonds": int(len(bonds)),
                   "step": "assemble + the whole cascade, host buffers in and out"},
        "cascade": {"status": int(res.status), "rounds": int(res.rounds), "bonds_broken": int(res.bonds_broken),
                    "nodes_retired": int(res.nodes_retired), "solves": int(res.solves),
                    "restarts": int(res.restarts), "pcg_iters": int(res.pcg_iters),
                    "ms_per_round": 1e3 * wall / max(1, res.rounds), "walls_s": walls},
        "roofline": None, "gpu_launches": int(launches / max(1, args.steps)),
    }
    if cpu is not None:
        line["cpu_baseline"] = cpu
    if clk is not None:
        line["clocks"] = clk
    print(json.dumps(line), flush=True)


def run_sections(args, rank: int, world: int):
    """Graph construction from voxels: the city block's bonds from its voxel-face interfaces
    (svxg_build_bonds: SecAcc::finish_lattice + section_strengths on the device). One step = every
    bond of the city; value = bonds/s with the interfaces resident (CUDA events on the launching
    stream), e2e = bonds/s through the C ABI with host arrays in and out; the CPU baseline is the
    oracle's restatement (one thread) on the same interfaces, which must give the same bytes."""
    import torch
    from opus_destruct_2_gb300 import build_bonds, load_library, synth
    from opus_destruct_2_gb300.graph import BOND_DTYPE
    L = load_library()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    nodes, _, _, mats = synth.city_graph(lots_x=args.lots, lots_y=args.lots, seed=args.seed + rank)
    secs, faces = synth.last_sections()
    nb, nf = len(secs), len(faces)
    t = {k: torch.from_numpy(np.frombuffer(v.tobytes(), np.uint8).copy()).to(dev)
         for k, v in dict(nodes=nodes, secs=secs, faces=faces, mats=mats).items()}
    out = torch.zeros(nb * BOND_DTYPE.itemsize, dtype=torch.uint8, device=dev)
    flush = torch.empty(2 * L2_BYTES, dtype=torch.uint8, device=dev)
    st = torch.cuda.current_stream(dev)

    def launch():
        rc = L.svxg_build_bonds_device(ctypes.c_void_p(t["nodes"].data_ptr()), len(nodes),
                                       ctypes.c_void_p(t["secs"].data_ptr()), nb, ctypes.c_void_p(t["faces"].data_ptr()),
                                       nf, None, 0, None, 0, 2, ctypes.c_void_p(t["mats"].data_ptr()),
                                       ctypes.c_void_p(out.data_ptr()), None, ctypes.c_void_p(st.cuda_stream))
        if rc:
            raise RuntimeError(L.svxg_last_error().decode())

    for _ in range(args.warmup):
        launch()
    torch.cuda.synchronize()
    clocks = Clocks(local)
    launches0 = L.svxg_launch_count()
    ms = []
    for _ in range(args.steps):
        flush.zero_()  # (L2 flushed between steps)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        launch()
        e1.record(st)
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
    launches = L.svxg_launch_count() - launches0
    clk = clocks.stop()
    kernel_ms = statistics.median(ms)
    got = np.frombuffer(out.cpu().numpy().tobytes(), dtype=BOND_DTYPE)
    # end to end: host arrays in and out
    build_bonds(nodes, secs, faces, mats)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        built = build_bonds(nodes, secs, faces, mats)
    e2e_s = (time.perf_counter() - t0) / args.steps
    cpu = None
    if not args.no_cpu_baseline:
        import oracle
        t0 = time.perf_counter()
        want = oracle.build_bonds(nodes, secs, faces, mats)
        tc = time.perf_counter() - t0
        same = all(np.ascontiguousarray(got[k]).tobytes() == np.ascontiguousarray(want[k]).tobytes()
                   for k in BOND_DTYPE.names)
        cpu = {"value": nb / tc, "unit": "bonds/s", "cores": 1, "kind": "port",
               "sample": "every bond of the same city, oracle restatement (C, one thread)", "same_bytes": bool(same)}
    algo = nb * (64 + BOND_DTYPE.itemsize + 2 * 40) + nf * 20
    peaks = measured_peaks()
    achieved = algo / (kernel_ms / 1e3) / 1e9
    line = {
        "metric": METRIC, "value": nb / (kernel_ms / 1e3), "unit": "bonds/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": kernel_ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"sections: the bonds of the {args.lots}x{args.lots} city block from its voxel-face "
                               f"interfaces (SecAcc::finish, the lattice path: one grid, no junction samples + "
                               f"section_strengths), L2 flushed between steps",
                   "bonds": int(nb), "faces": int(nf)},
        "e2e": {"value": nb / e2e_s, "unit": "bonds/s", "h2d_bytes_per_step": int(nodes.nbytes + secs.nbytes +
                                                                                   faces.nbytes + mats.nbytes),
                "d2h_bytes_per_step": int(built.nbytes)},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peaks.get("hbm_gbs"), "unit": "GB/s",
                     "frac": achieved / peaks["hbm_gbs"] if peaks.get("hbm_gbs") else None, "traffic": None,
                     "algorithmic_bytes": int(algo)},
        "gpu_launches": int(launches / max(1, args.steps)),
    }
    if cpu is not None:
        line["cpu_baseline"] = cpu
    if clk is not None:
        line["clocks"] = clk
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["serve", "city", "tower", "batch", "cascade", "sections", "pieces"],
                    default="serve")
    ap.add_argument("--batch-graphs", type=int, default=None, help="serve: graphs a batch at most (1: no batching)")
    ap.add_argument("--fragility", type=float, default=1.0, help="cascade: strength divisor")
    ap.add_argument("--requests", type=int, default=20000, help="serve: requests in the stream")
    ap.add_argument("--rate", type=float, default=5000.0, help="serve: Poisson arrival rate (requests/s)")
    ap.add_argument("--graphs", type=int, default=512, help="batch: graphs")
    ap.add_argument("--workers", type=int, default=32, help="batch / serve: server slots")
    ap.add_argument("--lots", type=int, default=8)
    ap.add_argument("--seed", type=int, default=2)
    ap.add_argument("--rtol", type=float, default=None, help="default: 1e-6 serving and batch, 1e-8 otherwise")
    ap.add_argument("--maxit", type=int, default=500)
    ap.add_argument("--precision", choices=["fp64", "mixed", "mixed-all"], default=None,
                    help="default: mixed (the policy) serving, fp64 otherwise; mixed-all: the policy with FP32 "
                         "inner sequences")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.rtol is None:
        args.rtol = 1e-6 if args.workload in ("serve", "batch") else 1e-8
    if args.precision is None:
        args.precision = "mixed" if args.workload == "serve" else "fp64"

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if args.workload == "serve":
        run_serve(args, rank, world)
        return
    if args.workload == "batch":
        run_many(args, rank, world)
        return
    if args.workload == "pieces":
        run_pieces(args, rank, world)
        return
    if args.workload == "cascade":
        run_cascade(args, rank, world)
        return
    if args.workload == "sections":
        run_sections(args, rank, world)
        return

    import torch
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl")

    from opus_destruct_2_gb300 import load_library
    from opus_destruct_2_gb300.graph import PcgResult, StressOptions, ptr

    L = load_library()
    L.svxg_launch_count.restype = ctypes.c_int64
    L.svxg_timer_enable.argtypes = [ctypes.c_void_p, ctypes.c_int32]
    L.svxg_timer_read.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int64)]
    L.svxg_time_spmv.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(ctypes.c_double)]
    L.svxg_measure_fp64_rate.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
    L.svxg_phase_timing.argtypes = [ctypes.c_void_p, ctypes.c_int32]
    L.svxg_phase_times.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.POINTER(ctypes.c_int32)]
    L.svxg_utilization_device.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p,
                                          ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32)]

    def check(code):
        if code < 0:
            raise RuntimeError(f"svxg error {code}: {L.svxg_last_error().decode()}")

    nodes, bonds, f, mats, desc = workload(args, rank)
    n, nb = len(nodes), len(bonds)
    dev = torch.device("cuda", local_rank)
    h = ctypes.c_void_p()
    check(L.svxg_problem_create(ctypes.byref(h), local_rank))
    stream = torch.cuda.ExternalStream(L.svxg_problem_stream(h), device=dev)
    opt = StressOptions(amg_min_nodes=160, precision={"fp64": 0, "mixed": 1, "mixed-all": 2}[args.precision])
    fp32_spmv = args.precision == "mixed-all"  # (the FP32 K conjugate-gradient product: inner sequences)
    ok = ctypes.c_int32()
    res = PcgResult()
    n_over = ctypes.c_int32()

    # device-resident inputs and outputs
    f_dev = torch.from_numpy(f).to(dev)
    u_dev = torch.zeros(6 * n, dtype=torch.float64, device=dev)
    phi_dev = torch.zeros(max(nb, 1), dtype=torch.float64, device=dev)
    mode_dev = torch.zeros(max(nb, 1), dtype=torch.uint8, device=dev)
    over_dev = torch.zeros(max(nb, 1), dtype=torch.int32, device=dev)
    torch.cuda.synchronize()
    check(L.svxg_set_graph(h, ptr(nodes), n, ptr(bonds), nb, ptr(mats)))

    phases = {"assemble": [], "solve": [], "judge": []}

    def step_device(record=False):
        t0 = time.perf_counter()
        check(L.svxg_assemble(h, ctypes.byref(opt), ctypes.byref(ok)))
        if not ok.value:
            raise RuntimeError("assemble: singular")
        t1 = time.perf_counter()
        check(L.svxg_solve_device(h, ctypes.c_void_p(f_dev.data_ptr()), ctypes.c_void_p(u_dev.data_ptr()), args.rtol,
                                  args.maxit, 0, ctypes.byref(res)))
        t2 = time.perf_counter()
        check(L.svxg_utilization_device(h, 1.0, ctypes.c_void_p(phi_dev.data_ptr()),
                                        ctypes.c_void_p(mode_dev.data_ptr()), ctypes.c_void_p(over_dev.data_ptr()),
                                        ctypes.byref(n_over)))
        torch.cuda.current_stream(dev).synchronize()
        stream.synchronize()
        t3 = time.perf_counter()
        if record:
            phases["assemble"].append(t1 - t0)
            phases["solve"].append(t2 - t1)
            phases["judge"].append(t3 - t2)
        return t3 - t0

    # host-buffer path (the e2e leg)
    u_host = np.zeros(6 * n)
    phi_host = np.zeros(max(nb, 1))
    mode_host = np.zeros(max(nb, 1), np.uint8)
    over_host = np.zeros(max(nb, 1), np.int32)

    def step_host():
        check(L.svxg_set_graph(h, ptr(nodes), n, ptr(bonds), nb, ptr(mats)))
        check(L.svxg_assemble(h, ctypes.byref(opt), ctypes.byref(ok)))
        check(L.svxg_solve(h, ptr(f), ptr(u_host), args.rtol, args.maxit, 0, ctypes.byref(res)))
        check(L.svxg_utilization(h, 1.0, ptr(phi_host), ptr(mode_host), ptr(over_host), len(over_host),
                                 ctypes.byref(n_over)))

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        step_device()
    # --- timed: device-resident ---
    barrier()
    clocks = Clocks(local_rank)
    launches0 = L.svxg_launch_count()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    lat = []
    for _ in range(args.steps):
        lat.append(step_device(record=True))
    ev1.record(stream)
    barrier()
    elapsed = ev0.elapsed_time(ev1) / 1e3
    launches = L.svxg_launch_count() - launches0
    clk = clocks.stop()
    iters = res.iters
    info_fail = n_over.value
    elapsed = max_over_ranks(elapsed, dist, dev)
    # --- roofline: the same solves again, each CG SpMV launch bracketed by CUDA events on the
    # problem's stream (the library then drives iterations from the host instead of one graph) ---
    tm, tl = ctypes.c_double(), ctypes.c_int64()
    L.svxg_timer_enable(h, 1)
    L.svxg_timer_read(h, ctypes.byref(tm), ctypes.byref(tl))  # (reset)
    for _ in range(args.steps):
        check(L.svxg_solve_device(h, ctypes.c_void_p(f_dev.data_ptr()), ctypes.c_void_p(u_dev.data_ptr()),
                                  args.rtol, args.maxit, 0, ctypes.byref(res)))
    L.svxg_timer_read(h, ctypes.byref(tm), ctypes.byref(tl))
    L.svxg_timer_enable(h, 0)
    # the same kernel in a dedicated loop (every launch does its work) and this GPU's FP64 FMA rate
    prec_code = 1 if fp32_spmv else 0
    loop_ms, fp64_tf = ctypes.c_double(), ctypes.c_double()
    check(L.svxg_time_spmv(h, prec_code, 50, ctypes.byref(loop_ms)))
    check(L.svxg_measure_fp64_rate(local_rank, ctypes.byref(fp64_tf)))
    # the setup's phases: one more assemble with a CUDA event at each phase boundary
    check(L.svxg_phase_timing(h, 1))
    check(L.svxg_assemble(h, ctypes.byref(opt), ctypes.byref(ok)))
    setup_ms = setup_phases(L, h, check)
    check(L.svxg_phase_timing(h, 0))
    # --- timed: end to end through the C ABI with host buffers ---
    step_host()
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step_host()
    barrier()
    e2e_elapsed = time.perf_counter() - t0
    e2e_elapsed = max_over_ranks(e2e_elapsed, dist, dev)

    from opus_destruct_2_gb300 import Info
    info = Info()
    check(L.svxg_get_info(h, ctypes.byref(info)))
    nfree, nnzb = info.nfree, info.matrix_blocks
    vb = 4 if fp32_spmv else 8
    spmv_bytes = nnzb * (36 * vb + 4) + nfree * (4 + 6 * vb + 6 * vb)
    peaks = measured_peaks()
    achieved = (spmv_bytes * tl.value / (tm.value / 1e3) / 1e9) if tm.value > 0 else 0.0
    traffic = None
    tp = os.path.join(ROOT, "profiles", f"spmv_traffic_{'fp32' if fp32_spmv else 'fp64'}.json")
    if os.path.exists(tp):
        with open(tp) as fh:
            tj = json.load(fh)
        if tj.get("nnzb") and tj.get("dram_bytes_per_launch"):
            traffic = float(tj["dram_bytes_per_launch"]) * nnzb / float(tj["nnzb"])

    if rank != 0:
        return
    h2d = nodes.nbytes + bonds.nbytes + mats.nbytes + f.nbytes
    d2h = u_host.nbytes + 8 * nb + nb + 4 * info_fail
    value = world * args.steps / elapsed
    line = {
        "metric": METRIC,
        "value": value,
        "unit": "solves/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1e3 * elapsed / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64" if args.precision == "fp64" else "f32+f64",
        "data": "synthetic",
        "config": {"workload": desc, "nodes": int(n), "bonds": int(nb), "dof": int(6 * nfree), "blocks": int(nnzb),
                   "levels": info.sizes(), "rtol": args.rtol, "pcg_iters": int(iters), "failing_bonds": int(info_fail),
                   "precision": ("fp64 K and CG, f32 V-cycle" if args.precision == "fp64" else
                                 "mixed policy: f32 V-cycle, multigrid built with FMAs and a tree-summed "
                                 "power-iteration norm, fp64 K and Krylov vectors"),
                   "step": "assemble + multigrid build + PCG + judge",
                   "l2": "inputs larger than L2 (K alone is %.0f MB)" % (nnzb * 288 / 1e6),
                   "parallelism": f"replicas x{world}"},
        "roofline": {"kernel": ("conjugate-gradient SpMV (FP32 BSR 6x6, p.q fused in FP64)" if fp32_spmv else
                                "conjugate-gradient SpMV (FP64 BSR 6x6, p.q fused)"), "bound": "hbm",
                     "how": "CUDA events around each SpMV launch that did work (the first `iters` of each "
                            "solve) on the problem's stream, over a timed pass of the same solves; loop_avg_us: "
                            "the same kernel in a dedicated loop of 50 launches",
                     "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": achieved / peaks["hbm_gbs"] if peaks["hbm_gbs"] else None,
                     "peak_source": peaks["source"], "traffic": traffic,
                     "algorithmic_bytes_per_launch": int(spmv_bytes), "launches": int(tl.value),
                     "avg_us": 1e3 * tm.value / max(tl.value, 1),
                     "loop_avg_us": 1e3 * loop_ms.value,
                     "fp64": ({"flops_per_launch": int(72 * nnzb),
                               "achieved_tflops": 72 * nnzb * tl.value / (tm.value / 1e3) / 1e12 if tm.value > 0
                               else 0.0,
                               "peak_tflops": fp64_tf.value,
                               "frac": (72 * nnzb * tl.value / (tm.value / 1e3) / 1e12) / fp64_tf.value
                               if tm.value > 0 and fp64_tf.value > 0 else None,
                               "peak_source": "measured in this run (independent FMA chains on every SM)"}
                              if not fp32_spmv else None)},
        "e2e": {"value": world * args.steps / e2e_elapsed, "unit": "solves/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": int(launches),
        "p50_ms": 1e3 * float(np.percentile(lat, 50)),
        "p99_ms": 1e3 * float(np.percentile(lat, 99)),
        "phase_ms": {k: 1e3 * float(np.mean(v)) for k, v in phases.items() if v},
        "setup_ms": setup_ms,
    }
    if clk is not None:
        line["clocks"] = clk
    if world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args, nodes, bonds, f, mats)
    print(json.dumps(line), flush=True)
    L.svxg_problem_destroy(h)


if __name__ == "__main__":
    main()
