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

from . import StressProblem, synth
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
    a structure's graph connected by splitting off detached parts before it solves."""
    n = len(nodes)
    parent = np.arange(n + 1)  # (n: the ground)

    def find(a):
        while parent[a] != a:
            parent[a] = parent[parent[a]]
            a = parent[a]
        return a

    for i in np.nonzero(nodes["fixed"])[0]:
        parent[find(int(i))] = find(n)
    keep = []
    for k, (a, b) in enumerate(zip(bonds["a"], bonds["b"])):
        ra, rb = find(int(a)), find(int(b) if b >= 0 else n)
        if ra == rb:
            keep.append(k)
        else:
            parent[ra] = rb
    return np.array(keep, dtype=np.int32)


def batch(count: int = 512, workers: int = 16, precision: int = PRECISION_MIXED, rtol: float = 1e-6,
          maxit: int = 2000, seed: int = 3, plain_sample: int = 128):
    gs = [(g[0], g[1], g[2]) for g in synth.batch_graphs(count, seed=seed)]
    mats = default_materials()
    opt = StressOptions(precision=precision)
    with Server(workers=workers, budget=40 << 30) as S:
        S.batch_solve(gs[:min(32, count)], mats, opt=opt, rtol=rtol, maxit=maxit, want_u=False)  # (warm-up)
        S.reset_stats()
        t0 = time.perf_counter()
        res, _ = S.batch_solve(gs, mats, opt=opt, rtol=rtol, maxit=maxit, want_u=False)
        wall = time.perf_counter() - t0
        st = S.stats()
    plain_rate, _ = plain_per_request(gs, mats, rtol, maxit, plain_sample)
    n = np.array([len(g[0]) for g in gs])
    iters = np.array([r.iters for r in res])
    bad = int(sum(1 for r in res if r.status != 0 or not bool(r.converged)))
    return {
        "solves_per_s": count / wall, "wall_s": wall, "p50_ms": st.p50_ms, "p99_ms": st.p99_ms,
        "block_row_iterations_per_s": float((n * iters).sum()) / wall, "graphs": count, "nodes": int(n.sum()),
        "bonds": int(sum(len(g[1]) for g in gs)), "not_converged": bad, "workers": workers,
        "plain_fp64_per_request_solves_per_s": plain_rate, "plain_sample": min(plain_sample, count),
        "peak_admitted_bytes": int(st.peak_bytes),
    }


def pieces(count: int = 512, workers: int = 16, seed: int = 5, plain_sample: int = 64, impact_scale: float = 20.0):
    """A substep's loose pieces through their break rounds (svxg_batch_piece_rounds): the batched
    workload's piece sizes (log-normal, median 300 fragments, 10-20,000), every piece free with
    inertial-relief loads and one impact of log-uniform 1e4-1e6 N scaled by `impact_scale` (so
    that most pieces crack), the world's settings (rtol 1e-2, 60 iterations, 8 rounds), resting
    loads (no energy limit). Reports pieces/s beside one piece after another on one problem."""
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
    with Server(workers=workers, budget=40 << 30) as S:
        S.batch_piece_rounds(ps[:min(32, count)], mats, options=o)  # (warm-up)
        S.reset_stats()
        t0 = time.perf_counter()
        pres, res, _, _, _ = S.batch_piece_rounds(ps, mats, options=o)
        wall = time.perf_counter() - t0
        st = S.stats()
    # one piece after another on one problem (the plain per-request path), on a sample
    lim = min(plain_sample, count)
    t0 = time.perf_counter()
    for nodes, bonds, f in ps[:lim]:
        G = StressProblem(nodes, bonds, mats)
        G.piece_rounds(f, options=o)
        del G
    plain = lim / (time.perf_counter() - t0)
    return {
        "pieces_per_s": count / wall, "wall_s": wall, "p50_ms": st.p50_ms, "p99_ms": st.p99_ms, "pieces": count,
        "nodes": int(sum(len(p[0]) for p in ps)), "bonds_broken": int(sum(r.bonds_broken for r in pres)),
        "chips": int(sum(r.chips for r in pres)), "rounds": int(sum(r.checks for r in pres)),
        "statuses": {str(s_): int(sum(1 for r in pres if r.status == s_)) for s_ in range(7)},
        "failed_requests": int(sum(1 for r in res if r.status != 0)), "workers": workers,
        "plain_per_piece_pieces_per_s": plain, "plain_sample": lim,
    }


def serve(requests: int = 20000, rate: float = 5000.0, repeat_share: float = 0.3, pool: int = 1500,
          workers: int = 16, precision: int = PRECISION_MIXED, rtol: float = 1e-6, maxit: int = 2000,
          budget: int = 40 << 30, seed: int = 11, plain_sample: int = 300):
    rng = np.random.default_rng(seed)
    sizes = synth.lognormal_sizes(pool, 500, 10, 50000, seed=seed)
    geoms = [synth.piece_graph(int(s), free=bool(rng.integers(0, 2)), seed=seed * 7919 + k)[:3]
             for k, s in enumerate(sizes)]
    mats = default_materials()
    opt = StressOptions(precision=precision)
    spare = [removable_bonds(g[0], g[1]) for g in geoms]
    # the request list: (kind, structure id, geometry index, bonds to remove); a repeat picks one
    # of the 256 structures submitted most recently and removes 1-5 % of its bonds, chosen among
    # the bonds whose removal keeps it connected
    plan, recent, plan_geom = [], [], {}
    for k in range(requests):
        if recent and rng.random() < repeat_share:
            sid = int(recent[rng.integers(0, len(recent))])
            g = plan_geom[sid]
            nb = len(geoms[g][1])
            want = max(1, int(rng.uniform(0.01, 0.05) * nb))
            pick = spare[g]
            cand = rng.choice(pick, size=min(want, len(pick)), replace=False) if len(pick) else pick
            plan.append(("repeat", sid, g, np.sort(cand).astype(np.int32)))
        else:
            g = int(rng.integers(0, pool))
            sid = len(plan_geom)
            plan_geom[sid] = g
            recent = (recent + [sid])[-256:]
            plan.append(("new", sid, g, None))
    gaps = rng.exponential(1.0 / rate, size=requests)
    with Server(workers=workers, budget=budget) as S:
        # warm-up: a few requests of the pool, then counters reset
        for g in range(min(16, pool)):
            S.wait(S.submit(*geoms[g][:2], mats, geoms[g][2], opt=opt, rtol=rtol, maxit=maxit, want_u=False))
        S.reset_stats()
        tickets = []
        t_start = time.perf_counter()
        t_next = t_start
        for (kind, sid, g, rm), gap in zip(plan, gaps):
            t_next += gap
            now = time.perf_counter()
            if t_next > now:
                time.sleep(t_next - now)
            nodes, bonds, f = geoms[g]
            if kind == "new":
                tickets.append(S.submit(nodes, bonds, mats, f, structure=sid, opt=opt, rtol=rtol, maxit=maxit,
                                        want_u=False))
            else:
                tickets.append(S.submit_repeat(sid, rm, f, rtol=rtol, maxit=maxit, want_u=False))
        submit_s = time.perf_counter() - t_start
        res = [S.wait(t)[0] for t in tickets]
        wall = time.perf_counter() - t_start
        st = S.stats()
    lat = np.array([r.latency_ms for r in res])
    ok = np.array([bool(r.status == 0 and r.converged) for r in res])
    statuses = {}
    for r in res:
        key = "unconverged" if r.status == 0 and not r.converged else f"status {r.status}"
        if r.status != 0 or not r.converged:
            statuses[key] = statuses.get(key, 0) + 1
    rep = np.array([p[0] == "repeat" for p in plan])
    dof = np.array([6 * len(geoms[p[2]][0]) for p in plan])
    near10k = (dof >= 8000) & (dof <= 12000)
    plain_reqs = [geoms[p[2]] for p in plan]
    plain_rate, plain_lat = (plain_per_request(plain_reqs, mats, rtol, maxit, plain_sample) if plain_sample > 0
                             else (float("nan"), np.array([np.nan])))
    return {
        "solves_per_s": float(ok.sum()) / wall, "wall_s": wall, "submit_s": submit_s,
        "requests": requests, "offered_rate": rate, "completed": int(ok.sum()),
        "failed_or_unconverged": int((~ok).sum()), "failures": statuses,
        "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
        "repeat_p50_ms": float(np.percentile(lat[rep], 50)) if rep.any() else None,
        "repeat_p99_ms": float(np.percentile(lat[rep], 99)) if rep.any() else None,
        "new_p50_ms": float(np.percentile(lat[~rep], 50)), "new_p99_ms": float(np.percentile(lat[~rep], 99)),
        "p99_ms_8k_12k_dof": float(np.percentile(lat[near10k], 99)) if near10k.any() else None,
        "evictions": int(st.evictions), "admission_waits": int(st.admission_waits),
        "peak_admitted_bytes": int(st.peak_bytes), "workers": workers, "pool": pool,
        "plain_fp64_per_request_solves_per_s": plain_rate, "plain_sample": plain_sample,
        "plain_fp64_p50_ms": float(np.percentile(plain_lat, 50)),
        "plain_fp64_p99_ms": float(np.percentile(plain_lat, 99)),
    }


__all__ = ["batch", "serve", "plain_per_request", "removable_bonds"]
