"""The device multigrid against the oracle (through the C ABI).

* hierarchy: per level A (pattern and values), D^-1, aggregates, prolongation and coarse
  positions bit-exact; level sizes, level blocks and the work counters equal;
* AMG-preconditioned solve: u and bond loads within 1e-6 (relative, FP64) of the oracle's solve
  to rtol 1e-12; failure sets identical.
"""
import numpy as np
import pytest

import fixtures as fx
from opus_destruct_2_gb300 import StressProblem, synth
from opus_destruct_2_gb300.graph import StressOptions, default_materials
from oracle import Port

pytestmark = pytest.mark.gpu

MATS = default_materials()

CASES = {
    "lattice8": (lambda: fx.lattice(8), dict(amg_min_nodes=16)),
    "lattice8_unsmoothed": (lambda: fx.lattice(8), dict(smoothed=0, amg_min_nodes=16)),
    "lattice16": (lambda: fx.lattice(16), dict()),
    "lattice16_once": (lambda: fx.lattice(16), dict(reaggregate=0)),
    "lattice16_dense_smoothed": (lambda: fx.lattice(16), dict(reaggregate=0, coarsen_dense=0)),
    "lattice14_retired": (lambda: fx.lattice(14, keep_z=9, retire_top=True), dict(amg_min_nodes=16)),
    "cantilever12": (lambda: fx.cantilever(12, 0.5, 300.0), dict(amg_min_nodes=4)),
    "tower10": (lambda: synth.tower_graph(storeys=10, seed=1)[:2], dict()),
    "piece_free": (lambda: synth.piece_graph(600, free=True, seed=21)[:2], dict(amg_min_nodes=0)),
    "piece_grounded": (lambda: synth.piece_graph(900, free=False, seed=22)[:2], dict(amg_min_nodes=0)),
    # levels of more than 8192 nodes: aggregation rounds across the grid, then the one-block tail
    "lattice24": (lambda: fx.lattice(24), dict()),
    "city3": (lambda: synth.city_graph(lots_x=3, lots_y=3, seed=2)[:2], dict()),
}


def relerr(a, b):
    m = np.max(np.abs(b))
    return float(np.max(np.abs(a - b)) / m) if m > 0 else float(np.max(np.abs(a - b)))


@pytest.mark.parametrize("name", list(CASES))
def test_hierarchy_bit_exact(name):
    make, opts = CASES[name]
    nodes, bonds = make()
    opt = StressOptions(**opts)
    G = StressProblem(nodes, bonds, MATS)
    assert G.assemble(opt)
    O = Port(nodes, bonds, MATS)
    O.keep_levels(True)
    assert O.assemble(opt)
    gi, oi = G.info(), O.info()
    assert gi.sizes() == oi.sizes()
    assert gi.blocks() == oi.blocks()
    for k in ("nfree", "chol_n", "matrix_blocks", "work_per_iteration", "assembly_work", "work_per_apply",
              "build_work", "block_jacobi"):
        assert getattr(gi, k) == getattr(oi, k), k
    gl, ol = G.debug_levels(), O.levels()
    assert len(gl) == len(ol)
    for l, (a, b) in enumerate(zip(gl, ol)):
        for k in ("rowptr", "col", "val", "dinv", "pos"):
            assert np.array_equal(a[k], getattr(b, k)), (l, k)
        if l + 1 < len(gl):
            for k in ("parent", "prow", "pcol", "pval"):
                assert np.array_equal(a[k], getattr(b, k)), (l, k)
            if opt.amg.smoothed and a["lmax"] > 0:
                assert a["lmax"] == b.lmax.value, l


@pytest.mark.parametrize("name", list(CASES))
def test_amg_solve_matches_oracle(name):
    make, opts = CASES[name]
    nodes, bonds = make()
    f = fx.gravity_live(nodes)
    opt = StressOptions(**opts)
    G = StressProblem(nodes, bonds, MATS)
    assert G.assemble(opt)
    u, res = G.solve(f, rtol=1e-12, maxit=2000)
    assert res.converged and not res.breakdown, res
    O = Port(nodes, bonds, MATS)
    O.assemble(opt)
    uo, ro = O.solve(f, rtol=1e-12, maxit=5000)
    assert ro.converged
    assert relerr(u, uo) <= 1e-6
    lg = G.bond_loads(u)
    lo = O.judge(uo)[0]
    for k in ("N", "V1", "V2", "T", "M1", "M2"):
        assert relerr(lg[k], lo[k]) <= 1e-6 * max(1.0, np.max(np.abs(np.stack([lo[q] for q in ("N", "V1", "V2")])))
                                                  / max(np.max(np.abs(lo[k])), 1e-300)), k


@pytest.mark.parametrize("name", ["tower10", "lattice16", "piece_free"])
def test_failure_set_identical(name):
    make, opts = CASES[name]
    nodes, bonds = make()
    f = fx.gravity_live(nodes)
    opt = StressOptions(**opts)
    G = StressProblem(nodes, bonds, MATS)
    assert G.assemble(opt)
    u, res = G.solve(f, rtol=1e-10, maxit=2000)
    O = Port(nodes, bonds, MATS)
    O.assemble(opt)
    uo, ro = O.solve(f, rtol=1e-12, maxit=5000)
    _, po, _ = O.judge(uo)
    # a fragility that puts the failure threshold inside the utilization range
    frag = 1.0 / float(np.quantile(po[po > 0], 0.9)) if np.any(po > 0) else 1.0
    _, po, mo = O.judge(uo, frag)
    phi, mode, over = G.utilization(frag)
    margin = np.min(np.abs(po - 1.0))
    band = 1e-6 * np.max(po)
    # bonds within the solve's error of phi = 1 are listed, not dropped: every bond judged
    # differently must be one of them
    in_band = np.nonzero(np.abs(po - 1.0) <= band)[0]
    differ = np.nonzero((phi >= 1.0) != (po >= 1.0))[0]
    assert np.isin(differ, in_band).all(), (f"min margin {margin:.3e}", differ.tolist(), in_band.tolist())
    if len(in_band) == 0:
        assert np.array_equal(over, np.nonzero(po >= 1.0)[0])
        assert np.array_equal(mode, mo)
