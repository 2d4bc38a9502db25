"""StressProblem::reassemble and extend_warm_start (core/src/stress/stress.cpp:178-244) on the
device, through the C ABI.

Bars:
  * extend_warm_start: bit-exact against the oracle's restatement (itself pinned to the
    reference in test_oracle_pin.py);
  * reassemble: after nodes are appended, the solve (cold or warm-started from the extended u)
    converges and agrees with the oracle's solve of the whole graph to 1e-6 (FP64), with the
    appended nodes preconditioned by their own multigrid (>= 24 nodes) or by their block-Jacobi
    inverses (fewer), and the preconditioner reported stale as the reference reports it.
"""
import numpy as np
import pytest

import fixtures as fx
import oracle
from opus_destruct_2_gb300 import StressProblem
from opus_destruct_2_gb300.graph import StressOptions, default_materials, empty_bonds

pytestmark = pytest.mark.gpu
MATS = default_materials()


def relerr(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def appended_case(n: int, top: int):
    """A lattice whose top `top` layers are appended: (old nodes, old bonds, all nodes, all bonds
    with the old ones first, number of old nodes)."""
    nodes, bonds = fx.lattice(n)
    z = np.rint(nodes["c"]["z"] / 0.4 - 0.5).astype(int)
    new = z >= n - top
    order = np.concatenate([np.nonzero(~new)[0], np.nonzero(new)[0]])
    inv = np.empty_like(order)
    inv[order] = np.arange(len(order))
    nodes2 = nodes[order].copy()
    b2 = empty_bonds(len(bonds))
    b2[:] = bonds
    b2["a"] = inv[bonds["a"]]
    b2["b"] = np.where(bonds["b"] >= 0, inv[np.maximum(bonds["b"], 0)], -1)
    n_old = int((~new).sum())
    old = (b2["a"] < n_old) & (b2["b"] < n_old)
    k = int(old.sum())
    allb = empty_bonds(len(b2))
    allb[:k] = b2[old]
    allb[k:] = b2[~old]
    oldb = empty_bonds(k)
    oldb[:] = b2[old]
    return nodes2[:n_old].copy(), oldb, nodes2, allb, n_old


# 64 appended nodes (their own multigrid), 16 (their block-Jacobi inverses)
@pytest.mark.parametrize("n,top,min_nodes", [(8, 1, 160), (4, 1, 16)])
def test_reassemble_appended_nodes(n, top, min_nodes):
    nodes_old, bonds_old, nodes, bonds, n_old = appended_case(n, top)
    opt = StressOptions(amg_min_nodes=min_nodes)
    G = StressProblem(nodes_old, bonds_old, MATS)
    assert G.assemble(opt) and not G.block_jacobi()
    u_old, r_old = G.solve(fx.gravity_live(nodes_old), rtol=1e-10, maxit=2000)
    assert r_old.converged
    # the world appends nodes and bonds, then reassembles
    G.nodes, G.bonds = nodes, bonds
    assert G.reassemble()
    na = len(nodes) - n_old
    assert G.appended() == na
    assert not G.preconditioner_current()
    f = fx.gravity_live(nodes)
    O = oracle.Port(nodes, bonds, MATS)
    O.assemble(opt)
    uo, _ = O.solve(f, rtol=1e-12, maxit=5000)
    # cold
    u1, r1 = G.solve(f, rtol=1e-10, maxit=2000)
    assert r1.converged and relerr(u1, uo) <= 1e-6
    # warm, from the old solution extended to the appended nodes
    u0 = np.zeros(6 * len(nodes))
    u0[:6 * n_old] = u_old
    ug = G.extend_warm_start(u0, n_old)
    ue = oracle.extend_warm_start(nodes, bonds, u0, n_old)
    assert np.array_equal(ug, ue)
    assert np.all(np.isfinite(ug)) and np.any(ug[6 * n_old:] != 0.0)
    u2, r2 = G.solve(f, u=ug, rtol=1e-10, maxit=2000, warm=True)
    assert r2.converged and relerr(u2, uo) <= 1e-6
    # a bond removed in place after the reassemble, then solved again
    G.remove_bond(len(bonds) - 1)
    u3, r3 = G.solve(f, rtol=1e-10, maxit=2000)
    assert r3.converged
    # assemble() makes the preconditioner whole again
    assert G.assemble(opt) and G.appended() == 0 and G.preconditioner_current()


def test_reassemble_without_an_assemble_is_assemble():
    nodes, bonds = fx.lattice(6)
    G = StressProblem(nodes, bonds, MATS)
    assert G.reassemble()
    assert G.appended() == 0 and G.preconditioner_current()
    H = StressProblem(nodes, bonds, MATS)
    assert H.assemble(StressOptions())
    f = fx.gravity_live(nodes)
    ua, ra = G.solve(f, rtol=1e-10, maxit=1000)
    ub, rb = H.solve(f, rtol=1e-10, maxit=1000)
    assert ra.iters == rb.iters and np.array_equal(ua, ub)
