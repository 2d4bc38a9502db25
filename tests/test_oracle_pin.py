"""Pins the oracle (the C restatement) to the reference compiled from its own sources.

Runs only where the reference tree is present (it is built into oracle/_ref/ from there); the
committed golden fixtures (tests/test_oracle_golden.py) carry the same pin to machines without
it. Every comparison is bit for bit: the restatement follows the reference's operation order.
"""
import numpy as np
import pytest

import fixtures as fx
from opus_destruct_2_gb300.graph import StressOptions, default_materials
from oracle import Port, Reference, reference_lib
from opus_destruct_2_gb300 import synth

pytestmark = pytest.mark.skipif(reference_lib() is None, reason="the reference is not built on this machine")

MATS = default_materials()

CASES = [
    ("cantilever12", lambda: fx.cantilever(12, 0.5, 300.0), dict(amg_min_nodes=4), 1e-10),
    ("lattice8_amg", lambda: fx.lattice(8), dict(amg_min_nodes=16), 1e-9),
    ("lattice8_jacobi", lambda: fx.lattice(8), dict(amg_min_nodes=1 << 30), 1e-9),
    ("lattice8_unsmoothed", lambda: fx.lattice(8), dict(smoothed=0), 1e-8),
    ("lattice16", lambda: fx.lattice(16), dict(), 1e-8),
    ("lattice16_once", lambda: fx.lattice(16), dict(reaggregate=0), 1e-8),
    ("lattice16_dense_smoothed", lambda: fx.lattice(16), dict(reaggregate=0, coarsen_dense=0), 1e-8),
    ("lattice14_retired", lambda: fx.lattice(14, keep_z=9, retire_top=True), dict(amg_min_nodes=16), 1e-8),
    ("tower_small", lambda: synth.tower_graph(storeys=3, seed=3)[:2], dict(), 1e-8),
    ("piece_free", lambda: synth.piece_graph(300, free=True, seed=11)[:2], dict(amg_min_nodes=0), 1e-8),
]


@pytest.mark.parametrize("name,make,opts,rtol", CASES, ids=[c[0] for c in CASES])
def test_solve_bit_identical(name, make, opts, rtol):
    nodes, bonds = make()
    f = fx.gravity_live(nodes)
    opt = StressOptions(**opts)
    r = Reference(nodes, bonds, MATS).solve(f, opt, rtol=rtol, maxit=2000)
    P = Port(nodes, bonds, MATS)
    assert P.assemble(opt) == r["ok"]
    u, res = P.solve(f, rtol=rtol, maxit=2000)
    assert res.iters == r["res"].iters
    assert res.converged == r["res"].converged and res.breakdown == r["res"].breakdown
    assert res.rel_res == r["res"].rel_res
    assert np.array_equal(u, r["u"])
    a, b = P.info(), r["info"]
    assert a.sizes() == b.sizes() and a.blocks() == b.blocks()
    for k in ("nfree", "chol_n", "matrix_blocks", "work_per_iteration", "assembly_work", "work_per_apply",
              "build_work", "block_jacobi"):
        assert getattr(a, k) == getattr(b, k), k
    # the judge: loads, utilizations and modes of every bond
    la, pa, ma = P.judge(u)
    lb, pb, mb = Reference(nodes, bonds, MATS).judge(u)
    assert np.array_equal(la, lb) and np.array_equal(pa, pb) and np.array_equal(ma, mb)


@pytest.mark.parametrize("name,make,opts,rtol", CASES[:8], ids=[c[0] for c in CASES[:8]])
def test_matrix_and_hierarchy_bit_identical(name, make, opts, rtol):
    nodes, bonds = make()
    opt = StressOptions(**opts)
    R = Reference(nodes, bonds, MATS)
    P = Port(nodes, bonds, MATS)
    P.keep_levels(True)
    ka, kb = P.matrix() if P.assemble(StressOptions(amg_min_nodes=1 << 30)) else None, R.matrix()
    for k in ("dof", "rowptr", "col", "val"):
        assert np.array_equal(ka[k], kb[k]), k
    assert ka["id_scale"] == kb["id_scale"]
    if opt.amg_min_nodes > 4096:
        return
    P2 = Port(nodes, bonds, MATS)
    P2.keep_levels(True)
    assert P2.assemble(StressOptions(**dict(opts, amg_min_nodes=0)))
    la = P2.levels()
    lb, chol = R.levels(StressOptions(**opts))
    assert len(la) == len(lb)
    for A, B in zip(la, lb):
        for k in ("rowptr", "col", "val", "dinv", "parent", "prow", "pcol", "pval", "pos"):
            assert np.array_equal(getattr(A, k), getattr(B, k)), k
        assert A.lmax.value == B.lmax.value
    assert np.array_equal(P2.chol(), chol)


def test_extend_warm_start_bit_identical():
    """The oracle's extend_warm_start (stress.cpp:213-244) against the reference's, on a lattice
    whose top layers were appended, from a seeded displacement of the older nodes."""
    from oracle import extend_warm_start
    from test_gpu_reassemble import appended_case
    for n, top in ((6, 2), (8, 1)):
        _, _, nodes, bonds, n_old = appended_case(n, top)
        rng = np.random.default_rng(n)
        u = np.zeros(6 * len(nodes))
        u[:6 * n_old] = rng.normal(size=6 * n_old) * 1e-3
        bonds = bonds.copy()
        bonds["broken"][rng.choice(len(bonds), size=len(bonds) // 10, replace=False)] = 1
        a = extend_warm_start(nodes, bonds, u, n_old)
        b = Reference(nodes, bonds, MATS).extend_warm_start(u, n_old)
        assert np.array_equal(a, b)
        assert np.any(a[6 * n_old:] != 0.0)


import cascade_cases as cc  # noqa: E402
from oracle import RefProblem, cascade  # noqa: E402

CASCADES = cc.cases()


@pytest.mark.parametrize("name", list(CASCADES), ids=list(CASCADES))
def test_cascade_bit_identical(name):
    """The break rounds (oracle.cascade) on the C restatement and on the reference's own
    StressProblem: the same bonds broken in the same order, the same nodes retired, the same u,
    judged loads and utilizations, bit for bit."""
    nodes, bonds, mats, f, ko, so, judged, has = CASCADES[name]
    out = []
    for cls in (Port, RefProblem):
        P = cls(nodes, bonds, mats)
        out.append(cascade(P, f, np.zeros(6 * len(nodes)), cc.options(ko), cc.stress_options(so), judged, has))
    a, b = out
    assert a["rounds"] > 0 or a["bonds_broken"] == 0
    for k in ("status", "rounds", "bonds_broken", "nodes_retired", "solves", "restarts", "pcg_iters", "broken",
              "retired", "per_round", "max_utilization"):
        assert a[k] == b[k], k
    assert np.array_equal(a["u"], b["u"]) and np.array_equal(a["phi"], b["phi"])
    assert a["judged"].tobytes() == b["judged"].tobytes() and np.array_equal(a["has"], b["has"])


import section_cases as scases  # noqa: E402
from oracle import build_bonds  # noqa: E402

SECTIONS = scases.cases()


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_build_bonds_general_bit_identical(seed):
    """finish_general + section_strengths_general (placed lattices, junction samples) of the C
    restatement against the reference's own header code, bit for bit."""
    nodes, secs, faces, js, lats, mats = scases.general(seed)
    a = build_bonds(nodes, secs, faces, mats, junctions=js, lattices=lats)
    b = build_bonds(nodes, secs, faces, mats, reference=True, junctions=js, lattices=lats)
    assert fx.same_records(a, b)


@pytest.mark.parametrize("name", list(SECTIONS), ids=list(SECTIONS))
def test_build_bonds_bit_identical(name):
    """Section geometry (SecAcc::finish_lattice + section_strengths) of the C restatement against
    the reference's own header code on the same interfaces, bit for bit."""
    nodes, secs, faces, mats = SECTIONS[name]
    a = build_bonds(nodes, secs, faces, mats)
    b = build_bonds(nodes, secs, faces, mats, reference=True)
    assert fx.same_records(a, b)


import piece_cases as pcases  # noqa: E402
from oracle import piece_rounds  # noqa: E402


@pytest.mark.parametrize("name", list(pcases.CASES), ids=list(pcases.CASES))
def test_piece_rounds_bit_identical(name):
    """A piece's break rounds (oracle.piece_rounds) on the C restatement and on the reference's own
    StressProblem: the same bonds broken in order with their modes, the same chips, the same u
    and moved loads, bit for bit."""
    nodes, bonds, mats, f, ko, gf = pcases.case(name)
    out = []
    for cls in (Port, RefProblem):
        P = cls(nodes, bonds, mats)
        out.append(piece_rounds(P, f, np.zeros(6 * len(nodes)), pcases.options(ko), gf))
    a, b = out
    for k in ("status", "checks", "bonds_broken", "chips", "pcg_iters", "rebuilt", "spent", "first_max_utilization",
              "max_utilization", "broken", "modes", "chip_nodes"):
        assert a[k] == b[k], k
    assert np.array_equal(a["u"], b["u"]) and np.array_equal(a["f"], b["f"])
