"""A batch of independent graphs as one problem (svxg_set_graphs) against the oracle.

* the batch is one graph to the setup: its level sizes and blocks and the work counters equal the
  oracle's for the same union graph (the reference's algorithm applied to it, with uncoupled
  leftover rows kept single as the batch keeps them);
* one sequence per graph: each graph's iteration count stays near its count alone as the batch
  grows (a shared sequence's would grow with the number of graphs);
* per-graph stopping: at rtol 1e-6 every graph's own residual, recomputed on the host with the
  oracle's K of that graph alone, is within the target (the batch's global residual decides
  nothing), and the per-graph rel. residuals the library reports are those residuals;
* each graph's u within 1e-6 (relative, FP64) of the oracle's solve of the graph alone (both to
  tight tolerances), phi likewise, and the failure set identical away from phi = 1;
* the same graph alone and in the batch (GPU, tight tolerance): within 1e-6.
"""
import numpy as np
import pytest

from opus_destruct_2_gb300 import Batch, StressProblem, synth
from opus_destruct_2_gb300.graph import BOND_DTYPE, StressOptions, default_materials
import oracle
from oracle import Port

pytestmark = pytest.mark.gpu

MATS = default_materials()


def graphs():
    out = []
    for k, (size, free) in enumerate([(12, True), (40, False), (150, True), (300, False), (700, True), (1500, False),
                                      (2500, True), (90, False), (500, True), (4000, False)]):
        n, b, f, _ = synth.piece_graph(size, free=free, seed=900 + k)
        out.append((n, b, f))
    return out


def union(gs):
    nodes = np.concatenate([g[0] for g in gs])
    bl, off = [], 0
    for g in gs:
        b = g[1].copy()
        b["a"] += off
        b["b"] = np.where(b["b"] >= 0, b["b"] + off, b["b"])
        bl.append(b)
        off += len(g[0])
    return nodes, np.concatenate(bl).astype(BOND_DTYPE), np.concatenate([g[2] for g in gs])


def relerr(a, b):
    m = np.max(np.abs(b))
    return float(np.max(np.abs(a - b)) / m) if m > 0 else float(np.max(np.abs(a - b)))


def test_batch_setup_is_the_union_graphs():
    gs = graphs()
    B = Batch([(g[0], g[1]) for g in gs], MATS)
    assert B.assemble(StressOptions())
    n, b, _ = union(gs)
    oracle.set_group_isolated(False)
    try:
        O = Port(n, b, MATS)
        assert O.assemble(StressOptions())
    finally:
        oracle.set_group_isolated(True)
    bi, oi = B.info(), O.info()
    assert bi.sizes() == oi.sizes() and bi.blocks() == oi.blocks()
    for k in ("nfree", "chol_n", "matrix_blocks", "work_per_apply", "build_work", "assembly_work"):
        assert getattr(bi, k) == getattr(oi, k), k


def test_batch_stops_per_graph():
    gs = graphs()
    B = Batch([(g[0], g[1]) for g in gs], MATS)
    assert B.assemble(StressOptions())
    us, res, rel, conv = B.solve([g[2] for g in gs], rtol=1e-6, maxit=2000)
    assert res.converged and conv.all()
    for (n, b, f), u, r in zip(gs, us, rel):
        O = Port(n, b, MATS)
        assert O.assemble(StressOptions())
        # the graph's own residual over its free DOFs, from the oracle's K of that graph alone
        dof = O.matrix()["dof"]
        free = np.nonzero(dof >= 0)[0]
        order = free[np.argsort(dof[free])]
        x = u.reshape(-1, 6)[order].ravel()
        ff = f.reshape(-1, 6)[order].ravel()
        fn = np.linalg.norm(ff)
        own = np.linalg.norm(ff - O.apply_k(x)) / fn if fn > 0 else 0.0
        assert own <= 1e-6 * (1 + 1e-6), own
        assert abs(own - r) <= 1e-9 + 1e-6 * r, (own, r)


def test_batch_matches_each_graph_alone():
    gs = graphs()
    B = Batch([(g[0], g[1]) for g in gs], MATS)
    assert B.assemble(StressOptions())
    us, res, rel, conv = B.solve([g[2] for g in gs], rtol=1e-10, maxit=5000)
    assert res.converged and conv.all() and (rel <= 1e-10).all()
    judged = B.utilization(1.0)
    for (n, b, f), u, (phi, mode, over) in zip(gs, us, judged):
        O = Port(n, b, MATS)
        assert O.assemble(StressOptions())
        uo, ro = O.solve(f, rtol=1e-12, maxit=5000)
        assert ro.converged
        assert relerr(u, uo) <= 1e-6
        _, phio, _ = O.judge(uo)
        assert np.allclose(phi, phio, rtol=1e-6, atol=1e-9 * max(1.0, float(np.max(phio))))
        band = np.nonzero(np.abs(phio - 1.0) <= 1e-6)[0]
        assert np.array_equal(np.setdiff1d(over, band), np.setdiff1d(np.nonzero(phio >= 1.0)[0], band))
        # the same graph alone on the GPU
        G = StressProblem(n, b, MATS)
        assert G.assemble(StressOptions())
        ug, rg = G.solve(f, rtol=1e-10, maxit=5000)
        assert rg.converged and relerr(u, ug) <= 1e-6


def test_batch_of_one_is_the_problem():
    n, b, f = graphs()[5]
    B = Batch([(n, b)], MATS)
    assert B.assemble(StressOptions())
    us, res, rel, conv = B.solve([f], rtol=1e-8, maxit=2000)
    G = StressProblem(n, b, MATS)
    assert G.assemble(StressOptions())
    ug, rg = G.solve(f, rtol=1e-8, maxit=2000)
    assert res.converged and conv[0] and rg.converged
    assert np.array_equal(us[0], ug) and res.iters == rg.iters


def test_batch_iterations_stay_per_graph():
    """64 pieces of the serving sizes in one batch: every graph's own sequence stops near its
    iteration count alone (the batch's multigrid differs from each graph's own, so not exactly)."""
    from opus_destruct_2_gb300 import workloads
    st = workloads.Stream(requests=64, rate=5000.0, pool=64, repeat_share=0.0, seed=29)
    gs = [st.geoms[p[2]] for p in st.plan][:64]
    B = Batch([(g[0], g[1]) for g in gs], MATS)
    assert B.assemble(StressOptions())
    us, res, rel, conv = B.solve([g[2] for g in gs], rtol=1e-6, maxit=2000)
    assert res.converged and conv.all() and (rel <= 1e-6).all()
    alone = []
    for n, b, f in gs:
        G = StressProblem(n, b, MATS)
        assert G.assemble(StressOptions(amg_min_nodes=0))
        alone.append(G.solve(f, rtol=1e-6, maxit=2000)[1].iters)
    assert int(np.max(B.iters)) <= 2 * int(np.max(alone)) + 5, (np.max(B.iters), np.max(alone))
    assert float(np.mean(B.iters)) <= 2.0 * float(np.mean(alone)) + 5.0, (np.mean(B.iters), np.mean(alone))
