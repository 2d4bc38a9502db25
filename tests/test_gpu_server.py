"""The serving loop and the batched solve (include/svxg_server.h) on the device.

Bars:
  * each result is the same alone and in the mix: without batching, a graph solved through the
    server, among others running at the same time, gives bit for bit the displacement, iteration
    count and failure list of the same graph solved alone on a fresh problem (FP64 and mixed
    precision); with batching (several new requests as one problem), every graph meets its own
    target and its displacement is within 1e-6 of the graph solved alone (both to 1e-10), its
    failure list the same;
  * a repeat request (bonds removed in place, warm start from the last solution on the device)
    gives the single-problem path's result for the same removals and warm start, bit for bit
    without batching, within 1e-6 for members of a batch kept resident (repeats of several
    members solved together);
  * admission: a budget that holds one structure at a time evicts the least recently used one,
    and a repeat of an evicted structure fails with SVXG_ERR_STATE in its result;
  * latencies are recorded (p50 <= p99 <= max) for every request.
"""
import numpy as np
import pytest

from opus_destruct_2_gb300 import StressProblem, synth
from opus_destruct_2_gb300.graph import StressOptions, default_materials
from opus_destruct_2_gb300.server import Server, estimate_bytes

pytestmark = pytest.mark.gpu

MATS = default_materials()
FP64, MIXED = 0, 1


def graphs(count, seed):
    return [(g[0], g[1], g[2]) for g in synth.batch_graphs(count, median=250, hi=3000, seed=seed)]


def alone(nodes, bonds, f, opt, rtol, fragility):
    G = StressProblem(nodes, bonds, MATS)
    ok = G.assemble(opt)
    assert ok
    u, res = G.solve(f, rtol=rtol, maxit=2000)
    _, _, over = G.utilization(fragility)
    return u, res, over


@pytest.mark.parametrize("precision", [FP64, MIXED])
def test_same_result_alone_and_in_the_mix(precision):
    gs = graphs(24, seed=5)
    opt = StressOptions(precision=precision)
    rtol, frag = 1e-6, 40.0
    ref = [alone(*g, opt, rtol, frag) for g in gs]
    with Server(workers=6, budget=8 << 30) as S:
        S.set_batching(1)
        tickets = [S.submit(*g[:2], MATS, g[2], opt=opt, rtol=rtol, maxit=2000, fragility=frag, want_over=True)
                   for g in gs]
        out = [S.wait(t) for t in tickets]
        st = S.stats()
    for (u0, r0, over0), (r, u, over) in zip(ref, out):
        assert r.status == 0
        assert r.iters == r0.iters and r.converged == r0.converged == 1
        assert np.array_equal(u, u0)
        assert np.array_equal(over, over0)
    assert st.completed == len(gs) and st.failed == 0
    assert 0 < st.p50_ms <= st.p99_ms <= st.max_ms


def relerr(a, b):
    m = np.max(np.abs(b))
    return float(np.max(np.abs(a - b)) / m) if m > 0 else float(np.max(np.abs(a - b)))


def test_batch_solve_matches_alone():
    """svxg_batch_solve: the graphs go into batches, several graphs to a problem."""
    gs = graphs(16, seed=9)
    opt = StressOptions(precision=MIXED)
    ref = [alone(*g, opt, 1e-10, 1.0) for g in gs]
    with Server(workers=4, budget=8 << 30) as S:
        res, us = S.batch_solve(gs, MATS, opt=opt, rtol=1e-10, maxit=5000)
        st = S.stats()
    assert st.batches >= 1 and st.batched_requests >= 2
    for (u0, r0, _), r, u in zip(ref, res, us):
        assert r.status == 0 and r.converged and r.rel_res <= 1e-10
        assert relerr(u, u0) <= 1e-6


def test_batched_requests_same_within_tolerance():
    gs = graphs(24, seed=5)
    opt = StressOptions(precision=MIXED)
    rtol, frag = 1e-10, 40.0
    ref = [alone(*g, opt, rtol, frag) for g in gs]
    with Server(workers=2, budget=8 << 30) as S:
        S.set_batching(8, 20000, 65536)
        S.hold(True)
        tickets = [S.submit(*g[:2], MATS, g[2], opt=opt, rtol=rtol, maxit=5000, fragility=frag, want_over=True)
                   for g in gs]
        S.hold(False)
        out = [S.wait(t) for t in tickets]
        st = S.stats()
    assert st.batches >= 3 and st.completed == len(gs)
    for (u0, r0, over0), (r, u, over) in zip(ref, out):
        assert r.status == 0 and r.converged == 1 and r.rel_res <= rtol
        assert relerr(u, u0) <= 1e-6
        assert np.array_equal(over, over0)


def test_bundle_repeats_match_single_problem_path():
    """Two structures solved in one batch and kept; repeats of both, queued together so that one
    solve of the bundle serves them, against the single-problem path (solve, in-place removal,
    warm solve)."""
    pieces = [synth.piece_graph(400, free=False, seed=21)[:3], synth.piece_graph(300, free=True, seed=23)[:3]]
    rng = np.random.default_rng(4)
    rms = [np.sort(rng.choice(len(b), size=max(1, len(b) // 40), replace=False)).astype(np.int32)
           for _, b, _ in pieces]
    opt = StressOptions(precision=MIXED)
    want = []
    for (nodes, bonds, f), rm in zip(pieces, rms):
        G = StressProblem(nodes, bonds, MATS)
        assert G.assemble(opt)
        u1, _ = G.solve(f, rtol=1e-10, maxit=5000)
        G.remove_bonds(rm)
        u2, _ = G.solve(f, u=u1, rtol=1e-10, maxit=5000, warm=True)
        _, _, over2 = G.utilization(1.0)
        want.append((u1, u2, over2))
    with Server(workers=1, budget=8 << 30) as S:
        S.set_batching(8, 20000, 65536)
        S.hold(True)
        t = [S.submit(n, b, MATS, f, structure=10 + k, opt=opt, rtol=1e-10, maxit=5000)
             for k, (n, b, f) in enumerate(pieces)]
        S.hold(False)
        first = [S.wait(x) for x in t]
        assert S.stats().batches == 1 and S.stats().resident == 2
        S.hold(True)
        t = [S.submit_repeat(10 + k, rm, f, rtol=1e-10, maxit=5000, want_over=True, nb=len(b))
             for k, ((n, b, f), rm) in enumerate(zip(pieces, rms))]
        S.hold(False)
        second = [S.wait(x) for x in t]
    for (r, u, _), (u1, _, _) in zip(first, want):
        assert r.status == 0 and r.converged and relerr(u, u1) <= 1e-6
    for (r, u, over), (_, u2, over2) in zip(second, want):
        assert r.status == 0 and r.warm == 1 and r.converged and r.rel_res <= 1e-10
        assert relerr(u, u2) <= 1e-6
        assert np.array_equal(over, over2)


def test_repeat_warm_start_matches_single_problem_path():
    nodes, bonds, f, _ = synth.piece_graph(400, free=False, seed=21)
    rng = np.random.default_rng(4)
    rm = np.sort(rng.choice(len(bonds), size=max(1, len(bonds) // 40), replace=False)).astype(np.int32)
    opt = StressOptions(precision=MIXED)
    # single-problem path: solve, remove in place, warm solve from the last u
    G = StressProblem(nodes, bonds, MATS)
    assert G.assemble(opt)
    u1, r1 = G.solve(f, rtol=1e-6, maxit=2000)
    for b in rm:
        G.remove_bond(int(b))
    u2, r2 = G.solve(f, u=u1, rtol=1e-6, maxit=2000, warm=True)
    _, _, over2 = G.utilization(1.0)
    with Server(workers=3, budget=8 << 30) as S:
        S.set_batching(1)
        t1 = S.submit(nodes, bonds, MATS, f, structure=7, opt=opt, rtol=1e-6, maxit=2000)
        t2 = S.submit_repeat(7, rm, f, rtol=1e-6, maxit=2000, want_over=True, nb=len(bonds))
        a, ua, _ = S.wait(t1)
        b, ub, overb = S.wait(t2)
        assert S.stats().resident == 1
    assert a.status == 0 and b.status == 0 and b.warm == 1 and a.warm == 0
    assert np.array_equal(ua, u1) and a.iters == r1.iters
    assert b.iters == r2.iters and np.array_equal(ub, u2)
    assert np.array_equal(overb, over2)


def test_admission_evicts_least_recently_used():
    nodes, bonds, f, _ = synth.piece_graph(300, free=False, seed=17)
    est = estimate_bytes(len(nodes), len(bonds))
    # room for one running request and nothing else: each new structure evicts the last one
    with Server(workers=1, budget=est + 1) as S:
        S.set_batching(1)
        for k in range(3):
            r, _, _ = S.wait(S.submit(nodes, bonds, MATS, f, structure=k))
            assert r.status == 0
        st = S.stats()
        assert st.evictions == 2 and st.resident == 1
        r, _, _ = S.wait(S.submit_repeat(0, [], f))
        assert r.status == -4  # SVXG_ERR_STATE: evicted
        r, _, _ = S.wait(S.submit_repeat(2, [], f))
        assert r.status == 0 and r.warm == 1 and r.iters <= 1
    with Server(workers=1, budget=est - 1) as S:
        r, _, _ = S.wait(S.submit(nodes, bonds, MATS, f))
        assert r.status == -3  # SVXG_ERR_NOMEM: larger than the whole budget


def test_admission_evicts_bundles_whole():
    """A batch kept resident frees memory only as a whole: with room for one batch, a second batch
    evicts the first (both its members), whose repeats then fail with SVXG_ERR_STATE."""
    a = synth.piece_graph(300, free=False, seed=17)[:3]
    b = synth.piece_graph(200, free=True, seed=18)[:3]
    est = estimate_bytes(len(a[0]), len(a[1])) + estimate_bytes(len(b[0]), len(b[1]))
    with Server(workers=1, budget=est + 1) as S:
        S.set_batching(8, 20000, 65536)
        for ids in ((1, 2), (3, 4)):
            S.hold(True)
            t = [S.submit(*a[:2], MATS, a[2], structure=ids[0]), S.submit(*b[:2], MATS, b[2], structure=ids[1])]
            S.hold(False)
            assert all(S.wait(x)[0].status == 0 for x in t)
        st = S.stats()
        assert st.batches == 2 and st.evictions == 2 and st.resident == 2
        assert S.wait(S.submit_repeat(1, [], a[2]))[0].status == -4
        r = S.wait(S.submit_repeat(4, [], b[2]))[0]
        assert r.status == 0 and r.warm == 1


def test_shutdown_after_deferred_repeats():
    """Repeats of one structure queued behind its first request are deferred by the slots that
    find it running; after every result is in, closing the server runs nothing more (a slot whose
    last act was a deferral has no request left to run), lifecycle after lifecycle."""
    nodes, bonds, f, _ = synth.piece_graph(300, free=False, seed=17)
    for rep in range(6):
        with Server(workers=8, budget=8 << 30) as S:
            S.set_batching(1)
            S.hold(True)
            t = [S.submit(nodes, bonds, MATS, f, structure=1)]
            t += [S.submit_repeat(1, [], f) for _ in range(12)]
            S.hold(False)
            out = [S.wait(x)[0] for x in t]
            st = S.stats()
        assert all(r.status == 0 for r in out)
        assert st.completed == len(t) and st.failed == 0
