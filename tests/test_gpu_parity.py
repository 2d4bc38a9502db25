"""Parity of the CUDA path (through the C ABI) with the oracle, on the reference's own fixtures and
on seeded synthetic graphs.

Bars (from the task's definition of parity):
  * K, its pattern, the DOF numbering and id_scale: bit-exact (value for value);
  * bond loads, utilizations and failure modes at the same u: bit-exact;
  * displacements and bond loads of a solve: relative error <= 1e-6 (FP64) against the oracle
    solved to rtol 1e-12, error measured as max|a - b| / max|b| over the vector;
  * edge cases: zero load (u = 0, converged), non-finite load (breakdown, rel_res = inf),
    iteration cap and resume, in-place bond removal and node retirement.
"""
import numpy as np
import pytest

import fixtures as fx
from opus_destruct_2_gb300 import StressProblem, synth
from opus_destruct_2_gb300.graph import StressOptions, default_materials
from oracle import Port

pytestmark = pytest.mark.gpu

MATS = default_materials()
JACOBI = dict(amg_min_nodes=1 << 30)

GRAPHS = {
    "cantilever12": lambda: fx.cantilever(12, 0.5, 300.0),
    "lattice8": lambda: fx.lattice(8),
    "lattice10_retired": lambda: fx.lattice(10, keep_z=6, retire_top=True),
    "tower3": lambda: synth.tower_graph(storeys=3, seed=3)[:2],
    "piece_free": lambda: synth.piece_graph(300, free=True, seed=11)[:2],
    "piece_grounded": lambda: synth.piece_graph(200, free=False, seed=12)[:2],
}


def relerr(a, b):
    m = np.max(np.abs(b))
    return float(np.max(np.abs(a - b)) / m) if m > 0 else float(np.max(np.abs(a - b)))


def loads_array(L):
    return np.stack([L[k] for k in ("N", "V1", "V2", "T", "M1", "M2")], axis=-1)


@pytest.mark.parametrize("name", list(GRAPHS))
def test_matrix_bit_exact(name):
    nodes, bonds = GRAPHS[name]()
    G = StressProblem(nodes, bonds, MATS)
    assert G.assemble(StressOptions(**JACOBI))
    O = Port(nodes, bonds, MATS)
    assert O.assemble(StressOptions(**JACOBI))
    a, b = G.debug_matrix(), O.matrix()
    assert a["nfree"] == b["nfree"]
    for k in ("dof", "rowptr", "col", "val"):
        assert np.array_equal(a[k], b[k]), k
    assert a["id_scale"] == b["id_scale"]
    # in_k flags as the reference keeps them
    assert np.array_equal(G.bonds["in_k"], O.bond_flags()[1])


@pytest.mark.parametrize("name", list(GRAPHS))
def test_jacobi_solve_matches_oracle(name):
    nodes, bonds = GRAPHS[name]()
    f = fx.gravity_live(nodes)
    G = StressProblem(nodes, bonds, MATS)
    assert G.assemble(StressOptions(**JACOBI))
    u, res = G.solve(f, rtol=1e-12, maxit=20000)
    assert res.converged and not res.breakdown
    O = Port(nodes, bonds, MATS)
    O.assemble(StressOptions(**JACOBI))
    uo, ro = O.solve(f, rtol=1e-12, maxit=20000)
    assert ro.converged
    assert relerr(u, uo) <= 1e-6
    # the reference's preconditioner and recurrences: the counts agree up to rounding in CG's tail
    assert res.iters <= 1.2 * ro.iters + 4
    lg, lo = loads_array(G.bond_loads(u)), loads_array(O.judge(uo)[0])
    assert relerr(lg, lo) <= 1e-6


@pytest.mark.parametrize("name", ["lattice8", "tower3", "piece_free"])
def test_judge_bit_exact_at_same_u(name):
    nodes, bonds = GRAPHS[name]()
    f = fx.gravity_live(nodes)
    O = Port(nodes, bonds, MATS)
    O.assemble(StressOptions(**JACOBI))
    uo, _ = O.solve(f, rtol=1e-10, maxit=20000)
    G = StressProblem(nodes, bonds, MATS)
    assert G.assemble(StressOptions(**JACOBI))
    for frag in (1.0, 25.0, 400.0):
        lo, po, mo = O.judge(uo, frag)
        assert np.array_equal(G.bond_loads(uo), lo)
        G.begin(f, uo)  # (current() = the warm start: a solve of zero iterations)
        G.iterate(0, 1e-30)
        phi, mode, over = G.utilization(frag)
        assert np.array_equal(phi, po) and np.array_equal(mode, mo)
        assert np.array_equal(over, np.nonzero(po >= 1.0)[0])


def test_zero_and_nonfinite_loads():
    nodes, bonds = fx.cantilever(6, 0.5, 100.0)
    G = StressProblem(nodes, bonds, MATS)
    assert G.assemble()
    f = np.zeros(6 * len(nodes))
    u, r0 = G.solve(f, np.ones(6 * len(nodes)), rtol=1e-9, maxit=100, warm=True)
    assert r0.converged and np.all(u == 0.0)
    f[2] = np.nan
    u, r1 = G.solve(f, rtol=1e-9, maxit=100)
    assert not r1.converged and r1.breakdown and np.isinf(r1.rel_res)


def test_iteration_cap_and_resume():
    nodes, bonds = fx.lattice(6)
    f = fx.gravity(nodes)
    G = StressProblem(nodes, bonds, MATS)
    assert G.assemble(StressOptions(**JACOBI))
    G.begin(f)
    r1 = G.iterate(5, 1e-10)
    assert r1.iters == 5 and not r1.converged
    r2 = G.iterate(10000, 1e-10)
    assert r2.converged
    u_split = G.current()
    u_once, r = G.solve(f, rtol=1e-10, maxit=10000)
    assert r.iters == r1.iters + r2.iters
    assert relerr(u_split, u_once) <= 1e-12


def test_remove_bond_in_place_bit_exact():
    nodes, bonds = fx.cantilever(10, 0.5, 200.0)
    bonds = fx.add_bond(nodes, bonds, 6, -1, (0.0, 0.0, -1.0), (3.25, 0.0, -0.25), 0.5)
    G = StressProblem(nodes, bonds, MATS)
    assert G.assemble(StressOptions(**JACOBI))
    G.remove_bond(3)
    O = Port(nodes, bonds, MATS)
    O.assemble(StressOptions(**JACOBI))
    O.remove_bond(3)
    a, b = G.debug_matrix(), O.matrix()
    assert np.array_equal(a["val"], b["val"])
    assert G.bonds["broken"][3] == 1 and G.bonds["in_k"][3] == 0
    f = fx.gravity(nodes)
    u, _ = G.solve(f, rtol=1e-11, maxit=2000)
    uo, _ = O.solve(f, rtol=1e-11, maxit=2000)
    assert relerr(u, uo) <= 1e-6


def test_retire_nodes_in_place_bit_exact():
    nodes, bonds = fx.cantilever(12, 0.5, 200.0)
    for i in (3, 6, 9):
        c = nodes[i]["c"]
        bonds = fx.add_bond(nodes, bonds, i, -1, (0.0, 0.0, -1.0), (float(c["x"]), 0.0, -0.25), 0.5)
    G = StressProblem(nodes, bonds, MATS)
    O = Port(nodes, bonds, MATS)
    assert G.assemble(StressOptions(**JACOBI)) and O.assemble(StressOptions(**JACOBI))
    G.retire_nodes([10, 11])
    O.retire_nodes([10, 11])
    G.retire_nodes([1])
    O.retire_nodes([1])
    a, b = G.debug_matrix(), O.matrix()
    assert np.array_equal(a["val"], b["val"])
    f = fx.gravity_live(G.nodes)
    u, r = G.solve(f, rtol=1e-11, maxit=2000)
    uo, ro = O.solve(f, rtol=1e-11, maxit=2000)
    assert r.converged and not r.breakdown
    assert relerr(u, uo) <= 1e-6


def test_empty_graph():
    G = StressProblem(fx.cantilever(1, 0.5, 1.0)[0][:0], fx.cantilever(1, 0.5, 1.0)[1][:0], MATS)
    assert G.assemble()
    u, r = G.solve(np.zeros(0), rtol=1e-8, maxit=10)
    assert r.converged and u.size == 0
