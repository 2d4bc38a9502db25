"""The batched and serving workloads, run through the library's server (include/svxg_server.h).

Batch: independent fragment graphs of log-normal size (median 300 fragments, 10-20,000), half
free pieces pinned at the node nearest their centre of mass with inertial-relief loads, half
ground-supported, gravity plus one seeded impact load each (synth.batch_graphs) - all submitted
at once, solved and judged.

Serving: a Poisson stream of solve requests (sizes log-normal, median 500 fragments, at most
50,000); a share of them repeat a structure solved earlier with 1-5 % of its bonds removed, which
the server solves in place from the structure's last displacement. The graphs come from a pool
of distinct seeded pieces (a new request of a pooled geometry is still a full assemble and solve).

Both report solves/s and latency percentiles, beside the plain FP64 per-request solve: one problem
on one stream, each request assembled and solved cold in arrival order, over a sample of the same
requests.
"""
from __future__ import annotations

import time

import numpy as np

from . import StressProblem, load_library, synth
from .graph import PRECISION_FP64, PRECISION_MIXED, StressOptions, default_materials
from .server import Server


def plain_per_request(reqs, mats, rtol: float, maxit: int, limit: int):
    """solves/s and latencies of the plain FP64 path, one request after another (sample)."""
    opt = StressOptions(precision=PRECISION_FP64)
    lat = []
    t0 = time.perf_counter()
    for nodes, bonds, f in reqs[:limit]:
        a = time.perf_counter()
        G = StressProblem(nodes, bonds, mats)
        G.assemble(opt)
        G.solve(f, rtol=rtol, maxit=maxit)
        G.utilization(1.0)
        del G
        lat.append(time.perf_counter() - a)
    dt = time.perf_counter() - t0
    n = min(limit, len(reqs))
    return n / dt, 1e3 * np.array(lat)


def removable_bonds(nodes, bonds) -> np.ndarray:
    """Bonds outside a spanning tree of the graph (fixed nodes and supports joined to the ground):
    removing any subset of them leaves every fragment connected, as the reference's world keeps
    a structure's graph connected by splitting off detached parts before it solves. The tree is
    Kruskal's in bond order after the fixed nodes' links to the ground: the minimum spanning tree
    with bond k weighing k + 1 and each fixed node's link 0.5 (distinct weights: one tree); of
    bonds joining the same pair only the first can be in it."""
    import scipy.sparse as sp
    from scipy.sparse.csgraph import minimum_spanning_tree
    n, nb = len(nodes), len(bonds)
    if nb == 0:
        return np.zeros(0, np.int32)
    a = bonds["a"].astype(np.int64)
    b = bonds["b"].astype(np.int64)
    b = np.where(b >= 0, b, n)  # (node n: the ground)
    lo, hi = np.minimum(a, b), np.maximum(a, b)
    _, first = np.unique(lo * (n + 1) + hi, return_index=True)
    fixed = np.nonzero(nodes["fixed"])[0]
    rows = np.concatenate([lo[first], fixed])
    cols = np.concatenate([hi[first], np.full(len(fixed), n)])
    w = np.concatenate([first.astype(np.float64) + 1.0, np.full(len(fixed), 0.5)])
    G = sp.coo_matrix((w, (rows, cols)), shape=(n + 1, n + 1)).tocsr()
    G.sum_duplicates()  # (a fixed node's support bond and its ground link: 0.5 + weight, never in the tree)
    T = minimum_spanning_tree(G).tocoo()
    in_tree = np.zeros(nb, bool)
    in_tree[np.round(T.data[T.data >= 1.0] - 1.0).astype(np.int64)] = True
    return np.nonzero(~in_tree)[0].astype(np.int32)


def batch(count: int = 512, workers: int = 16, precision: int = PRECISION_MIXED, rtol: float = 1e-6,
          maxit: int = 2000, seed: int = 3, plain_sample: int = 128, steps: int = 1, warmup: int = 1):
    """`count` graphs submitted at once (svxg_batch_solve: the server takes them in batches), each
    assembled and solved cold to `rtol` under `precision`; `warmup` untimed passes over all of them,
    then `steps` timed ones (fresh problems each time). Reports solves/s beside the plain FP64
    path one graph after another."""
    gs = [(g[0], g[1], g[2]) for g in synth.batch_graphs(count, seed=seed)]
    mats = default_materials()
    opt = StressOptions(precision=precision)
    with Server(workers=workers, budget=40 << 30) as S:
        for _ in range(max(warmup, 1)):
            S.batch_solve(gs, mats, opt=opt, rtol=rtol, maxit=maxit, want_u=False)  # (warm-up passes)
        S.reset_stats()
        t0 = time.perf_counter()
        for _ in range(max(steps, 1)):
            res, _ = S.batch_solve(gs, mats, opt=opt, rtol=rtol, maxit=maxit, want_u=False)
        wall = time.perf_counter() - t0
        st = S.stats()
    plain_rate, _ = plain_per_request(gs, mats, rtol, maxit, plain_sample)
    n = np.array([len(g[0]) for g in gs])
    iters = np.array([r.iters for r in res])
    bad = int(sum(1 for r in res if r.status != 0 or not bool(r.converged)))
    return {
        "solves_per_s": max(steps, 1) * count / wall, "wall_s": wall, "passes": max(steps, 1),
        "warmup_passes": max(warmup, 1), "p50_ms": st.p50_ms, "p99_ms": st.p99_ms,
        "block_row_iterations_per_s": max(steps, 1) * float((n * iters).sum()) / wall, "graphs": count,
        "nodes": int(n.sum()),
        "bonds": int(sum(len(g[1]) for g in gs)), "not_converged": bad, "workers": workers,
        "plain_fp64_per_request_solves_per_s": plain_rate, "plain_sample": min(plain_sample, count),
        "peak_admitted_bytes": int(st.peak_bytes),
    }


def pieces(count: int = 512, workers: int = 16, seed: int = 5, plain_sample: int = 64, impact_scale: float = 20.0,
           precision: int = PRECISION_FP64, steps: int = 1, warmup: int = 1):
    """A substep's loose pieces through their break rounds (svxg_batch_piece_rounds): the batched
    workload's piece sizes (log-normal, median 300 fragments, 10-20,000), every piece free with
    inertial-relief loads and one impact of log-uniform 1e4-1e6 N scaled by `impact_scale` (so
    that most pieces crack), the world's settings (rtol 1e-2, 60 iterations, 8 rounds), resting
    loads (no energy limit), under `precision` (FP64: the bit-exact multigrid; the mixed policy:
    its fast build). `warmup` untimed substeps, then `steps` timed ones (every piece's rounds from
    its original graph each time, on a fresh problem). Reports pieces/s beside one piece after
    another on one problem."""
    from .graph import PieceOptions
    sizes = synth.lognormal_sizes(count, 300, 10, 20000, seed=seed)
    rng = np.random.default_rng(seed + 1)
    ps = []
    for k, sz in enumerate(sizes):
        imp = float(10 ** rng.uniform(4.0, 6.0)) * impact_scale
        nodes, bonds, f, _ = synth.piece_graph(int(sz), free=True, seed=seed * 100003 + k, impact=imp)
        ps.append((nodes, bonds, f))
    mats = default_materials()
    o = PieceOptions()
    so = StressOptions(precision=precision)
    with Server(workers=workers, budget=40 << 30) as S:
        for _ in range(max(warmup, 1)):
            S.batch_piece_rounds(ps, mats, options=o, opt=so)  # (warm-up substeps)
        S.reset_stats()
        t0 = time.perf_counter()
        for _ in range(max(steps, 1)):
            pres, res, _, _, _ = S.batch_piece_rounds(ps, mats, options=o, opt=so)
        wall = time.perf_counter() - t0
        st = S.stats()
    # one piece after another on one problem (the plain per-request path), on a sample
    lim = min(plain_sample, count)
    t0 = time.perf_counter()
    for nodes, bonds, f in ps[:lim]:
        G = StressProblem(nodes, bonds, mats)
        G.piece_rounds(f, options=o, opt=so)
        del G
    plain = lim / (time.perf_counter() - t0)
    return {
        "pieces_per_s": max(steps, 1) * count / wall, "wall_s": wall, "substeps": max(steps, 1),
        "warmup_substeps": max(warmup, 1), "p50_ms": st.p50_ms, "p99_ms": st.p99_ms, "pieces": count,
        "nodes": int(sum(len(p[0]) for p in ps)), "bonds_broken": int(sum(r.bonds_broken for r in pres)),
        "chips": int(sum(r.chips for r in pres)), "rounds": int(sum(r.checks for r in pres)),
        "statuses": {str(s_): int(sum(1 for r in pres if r.status == s_)) for s_ in range(7)},
        "failed_requests": int(sum(1 for r in res if r.status != 0)), "workers": workers,
        "plain_per_piece_pieces_per_s": plain, "plain_sample": lim,
    }


class Stream:
    """A seeded serving stream (the serving configuration): `requests` Poisson arrivals at `rate`,
    a pool of `pool` distinct seeded pieces of log-normal size (median 500 fragments, 10-50,000),
    half free and half ground-supported; a share `repeat_share` of requests repeat one of the 256
    structures submitted most recently with 1-5 % of its bonds removed (bonds outside a spanning
    tree, so the structure stays connected), the rest are new structures of a pool geometry (a new
    structure is a full assemble and solve even when its geometry repeats).

    plan[k] = (kind, structure id, geometry index, bonds to remove); gaps[k]: seconds before
    request k arrives."""

    def __init__(self, requests: int = 20000, rate: float = 5000.0, repeat_share: float = 0.3, pool: int = 1500,
                 seed: int = 11):
        import os
        from concurrent.futures import ThreadPoolExecutor
        rng = np.random.default_rng(seed)
        sizes = synth.lognormal_sizes(pool, 500, 10, 50000, seed=seed)
        free = [bool(rng.integers(0, 2)) for _ in sizes]
        # (the generator is C++ behind ctypes, which lets go of the interpreter: one piece a thread)
        with ThreadPoolExecutor(max_workers=os.cpu_count() or 1) as ex:
            self.geoms = list(ex.map(lambda k: synth.piece_graph(int(sizes[k]), free=free[k], seed=seed * 7919 + k)[:3],
                                     range(pool)))
            spare = list(ex.map(lambda g: removable_bonds(g[0], g[1]), self.geoms))
        self.mats = default_materials()
        plan, recent, plan_geom = [], [], {}
        for _ in range(requests):
            if recent and rng.random() < repeat_share:
                sid = int(recent[rng.integers(0, len(recent))])
                g = plan_geom[sid]
                want = max(1, int(rng.uniform(0.01, 0.05) * len(self.geoms[g][1])))
                pick = spare[g]
                cand = rng.choice(pick, size=min(want, len(pick)), replace=False) if len(pick) else pick
                plan.append(("repeat", sid, g, np.sort(cand).astype(np.int32)))
            else:
                g = int(rng.integers(0, pool))
                sid = len(plan_geom)
                plan_geom[sid] = g
                recent = (recent + [sid])[-256:]
                plan.append(("new", sid, g, None))
        self.plan = plan
        self.gaps = rng.exponential(1.0 / rate, size=requests)
        self.rate = rate
        self.seed = seed

    def dof(self) -> np.ndarray:
        return np.array([6 * len(self.geoms[p[2]][0]) for p in self.plan])

    def subset(self, every: int) -> list[int]:
        """Requests of every `every`-th structure with all their repeats, in arrival order: a sample
        of the stream with its sizes and its repeat share."""
        return [k for k, p in enumerate(self.plan) if p[1] % every == 0]


class DeviceGeometries:
    """The stream's pool geometries, material table and loads staged in device memory (torch
    buffers), for submissions whose inputs are already resident on the device."""

    def __init__(self, stream: Stream, device: int = 0):
        import torch
        dev = torch.device("cuda", device)
        as_dev = lambda a: torch.from_numpy(np.ascontiguousarray(a).view(np.uint8).copy()).to(dev)  # noqa: E731
        self.keep = [(as_dev(n), as_dev(b), as_dev(f)) for n, b, f in stream.geoms]
        self.mats = as_dev(stream.mats)
        torch.cuda.synchronize(dev)

    def ptrs(self, g: int):
        n, b, f = self.keep[g]
        return n.data_ptr(), b.data_ptr(), f.data_ptr()


def serve_stream(stream: Stream, workers: int = 16, precision: int = PRECISION_MIXED, rtol: float = 1e-6,
                 maxit: int = 2000, budget: int = 40 << 30, inputs: str = "host", warmup: int = 64,
                 indices=None, rate: float | None = None, staged: DeviceGeometries | None = None,
                 batching: tuple | None = None):
    """The stream (or the requests `indices` of it) through a fresh server: each request submitted at
    its arrival time (gaps scaled to `rate` when given), results awaited. inputs "host": graphs and
    loads from host arrays (svxg_server_submit); "device": from `staged` device copies
    (svxg_server_submit_device). batching: (max graphs, max nodes a graph, max nodes) or None for
    the server's defaults. Returns solves/s (completed / first submission -> last completion),
    latency percentiles and block-row iterations/s."""
    idx = list(range(len(stream.plan))) if indices is None else list(indices)
    scale = 1.0 if rate is None else stream.rate / rate
    opt = StressOptions(precision=precision)
    mats = stream.mats
    L = load_library()
    with Server(workers=workers, budget=budget) as S:
        if batching is not None:
            S.set_batching(*batching)
        # warm-up: pool geometries as one-shot requests (not kept), then counters reset
        for g in range(min(warmup, len(stream.geoms))):
            S.submit(*stream.geoms[g][:2], mats, stream.geoms[g][2], opt=opt, rtol=rtol, maxit=maxit, want_u=False)
        S.drain()
        S.reset_stats()
        l0, g0 = L.svxg_launch_count(), L.svxg_graph_launch_count()
        tickets = []
        t_start = time.perf_counter()
        t_next = t_start
        for k in idx:
            kind, sid, g, rm = stream.plan[k]
            t_next += stream.gaps[k] * scale
            now = time.perf_counter()
            if t_next > now:
                time.sleep(t_next - now)
            nodes, bonds, f = stream.geoms[g]
            if inputs == "device":
                pn, pb, pf = staged.ptrs(g)
                if kind == "new":
                    t = S.submit_device(pn, len(nodes), pb, len(bonds), staged.mats.data_ptr(), pf, structure=sid,
                                        opt=opt, rtol=rtol, maxit=maxit)
                else:
                    t = S.submit_repeat_device(sid, rm, pf, len(nodes), rtol=rtol, maxit=maxit)
            elif kind == "new":
                t = S.submit(nodes, bonds, mats, f, structure=sid, opt=opt, rtol=rtol, maxit=maxit, want_u=False)
            else:
                t = S.submit_repeat(sid, rm, f, rtol=rtol, maxit=maxit, want_u=False)
            tickets.append(t)
        submit_s = time.perf_counter() - t_start
        res = [S.wait(t)[0] for t in tickets]
        wall = time.perf_counter() - t_start
        launches, in_graphs = L.svxg_launch_count() - l0, L.svxg_graph_launch_count() - g0
        st = S.stats()
    lat = np.array([r.latency_ms for r in res])
    ok = np.array([bool(r.status == 0 and r.converged) for r in res])
    statuses = {}
    for r in res:
        if r.status != 0 or not r.converged:
            key = "unconverged" if r.status == 0 else f"status {r.status}"
            statuses[key] = statuses.get(key, 0) + 1
    rep = np.array([stream.plan[k][0] == "repeat" for k in idx])
    dof = stream.dof()[idx]
    near10k = (dof >= 8000) & (dof <= 12000)
    iters = np.array([r.iters for r in res])
    pct = lambda a, q: float(np.percentile(a, q)) if len(a) else None  # noqa: E731
    return {
        "solves_per_s": float(ok.sum()) / wall, "wall_s": wall, "submit_s": submit_s, "requests": len(idx),
        "offered_rate": stream.rate / scale, "completed": int(ok.sum()), "failed_or_unconverged": int((~ok).sum()),
        "failures": statuses, "p50_ms": pct(lat, 50), "p99_ms": pct(lat, 99),
        "repeat_p50_ms": pct(lat[rep], 50), "repeat_p99_ms": pct(lat[rep], 99),
        "new_p50_ms": pct(lat[~rep], 50), "new_p99_ms": pct(lat[~rep], 99),
        "p99_ms_8k_12k_dof": pct(lat[near10k], 99), "requests_8k_12k_dof": int(near10k.sum()),
        "block_row_iterations_per_s": float((dof / 6 * iters).sum()) / wall,
        "pcg_iters_mean": float(iters.mean()) if len(iters) else 0.0,
        "batches": int(st.batches), "batched_requests": int(st.batched_requests),
        "evictions": int(st.evictions), "admission_waits": int(st.admission_waits),
        "peak_admitted_bytes": int(st.peak_bytes), "workers": workers, "inputs": inputs,
        "launches": int(launches), "launches_in_graphs": int(in_graphs),
        "host_launches_per_s": float(launches - in_graphs) / wall,
    }


def plain_stream(stream: Stream, indices, rtol: float = 1e-6, maxit: int = 2000):
    """The plain FP64 drop-in per request (one StressProblem at a time through the C ABI, FP64 PCG),
    over the requests `indices` in arrival order with no queueing: a new structure is assembled
    and solved cold, a repeat removes its bonds in place on that structure's problem and solves
    warm from its last solution (the reference's remove_bond + warm solve), each judged. Returns
    solves/s (requests / busy time) and service-time percentiles."""
    opt = StressOptions(precision=PRECISION_FP64)
    mats = stream.mats
    kept: dict[int, StressProblem] = {}
    order: list[int] = []
    lat = []
    ok = 0
    t0 = time.perf_counter()
    for k in indices:
        kind, sid, g, rm = stream.plan[k]
        nodes, bonds, f = stream.geoms[g]
        a = time.perf_counter()
        if kind == "new":
            G = StressProblem(nodes, bonds, mats)
            G.assemble(opt)
            u, res = G.solve(f, rtol=rtol, maxit=maxit)
            kept[sid] = G
            order.append(sid)
            if len(order) > 256:
                kept.pop(order.pop(0), None)
        else:
            G = kept.get(sid)
            if G is None:  # (its structure left the last 256: the stream never repeats one)
                continue
            G.remove_bonds(rm)
            u, res = G.solve(f, u=G.current(), rtol=rtol, maxit=maxit, warm=True)
        G.utilization(1.0)
        lat.append(time.perf_counter() - a)
        ok += int(res.converged)
    dt = time.perf_counter() - t0
    lat = 1e3 * np.array(lat)
    return {"solves_per_s": len(lat) / dt, "requests": len(lat), "converged": ok, "wall_s": dt,
            "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99))}


def serve(requests: int = 20000, rate: float = 5000.0, workers: int = 16, precision: int = PRECISION_MIXED,
          rtol: float = 1e-6, maxit: int = 2000, budget: int = 40 << 30, seed: int = 11, plain_every: int = 8):
    """The serving stream through the server (host inputs) beside the plain FP64 per-request path on
    a sample of the same stream (every `plain_every`-th structure with its repeats)."""
    st = Stream(requests=requests, rate=rate, seed=seed)
    r = serve_stream(st, workers=workers, precision=precision, rtol=rtol, maxit=maxit, budget=budget)
    if plain_every > 0:
        p = plain_stream(st, st.subset(plain_every), rtol=rtol, maxit=maxit)
        r.update({"plain_fp64_per_request_solves_per_s": p["solves_per_s"], "plain_sample": p["requests"],
                  "plain_fp64_p50_ms": p["p50_ms"], "plain_fp64_p99_ms": p["p99_ms"]})
    return r


__all__ = ["batch", "serve", "plain_per_request", "removable_bonds", "Stream", "DeviceGeometries", "serve_stream",
           "plain_stream"]
