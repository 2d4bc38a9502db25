"""The judge's break rounds on the device (svxg_cascade, through the C ABI) against the oracle's
restatement (oracle.cascade on the C restatement, itself pinned to the same rounds run on the
reference's StressProblem by test_oracle_golden.py / test_oracle_pin.py).

Bars:
  * the same bonds broken in the same order, the same nodes retired in the same order, the same
    number of rounds and the same final status (both sides solve to rtol 1e-10, far inside the
    cases' margins between a utilization and the thresholds it is compared with);
  * u, the judged loads and the last utilizations within 1e-6 relative (FP64);
  * the problem's bond flags and retired nodes as the oracle's;
  * with no preconditioner rebuild on either side (rebuild_after and maxit large), K after the
    rounds bit for bit the oracle's: the parallel in-order downdates and identity rows are the
    reference's own arithmetic in the reference's order.
"""
import numpy as np
import pytest

import cascade_cases as cc
import fixtures as fx
import oracle
from opus_destruct_2_gb300 import StressProblem, synth
from opus_destruct_2_gb300.graph import LOAD_DTYPE, CascadeOptions, StressOptions, default_materials

pytestmark = pytest.mark.gpu
CASES = cc.cases()
TIGHT = dict(rtol=1e-10, maxit=4000, rebuild_after=1 << 30)


def relerr(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    s = float(np.max(np.abs(b))) if b.size else 0.0
    return float(np.max(np.abs(a - b)) / s) if s > 0 else float(np.max(np.abs(a - b), initial=0.0))


def loads_array(rec):
    return np.stack([np.asarray(rec[k], float) for k in oracle.LOAD_FIELDS], axis=1)


def run_both(name, **over):
    nodes, bonds, mats, f, ko, so, judged, has = CASES[name]
    kw = dict(ko, **TIGHT)
    kw.update(over)
    O = oracle.Port(nodes, bonds, mats)
    ro = oracle.cascade(O, f, np.zeros(6 * len(nodes)), CascadeOptions(**kw), StressOptions(**so), judged, has)
    G = StressProblem(nodes, bonds, mats)
    assert G.assemble(StressOptions(**so))
    u, res, ex = G.cascade(f, options=CascadeOptions(**kw), opt=StressOptions(**so), judged=judged, has=has)
    return G, O, ro, u, res, ex


# cases whose over-strength bonds tie in exact arithmetic (a symmetric lattice's supports): their
# utilizations differ in the last bits only, by rounding that differs between any two solvers, so
# the order within a round is compared as a set there
TIES = {"lattice_shock"}


def same_rounds(broken, ref, per_round):
    k = 0
    for c in per_round:
        if sorted(broken[k:k + c]) != sorted(ref[k:k + c]):
            return False
        k += c
    return k == len(broken) == len(ref)


@pytest.mark.parametrize("name", list(CASES), ids=list(CASES))
def test_cascade_matches_oracle(name):
    G, O, ro, u, res, ex = run_both(name)
    assert res.status == ro["status"]
    assert res.rounds == ro["rounds"] and res.bonds_broken == ro["bonds_broken"]
    if name in TIES:
        assert same_rounds(ex["broken"], ro["broken"], ro["per_round"])
    else:
        assert ex["broken"] == ro["broken"]
    assert ex["retired"] == ro["retired"] and res.nodes_retired == ro["nodes_retired"]
    assert relerr(u, ro["u"]) <= 1e-6
    assert relerr(ex["phi"], ro["phi"]) <= 1e-6
    assert abs(res.max_utilization - ro["max_utilization"]) <= 1e-6 * max(1.0, ro["max_utilization"])
    assert np.array_equal(ex["has"], ro["has"])
    assert relerr(loads_array(ex["judged"]), loads_array(ro["judged"])) <= 1e-6
    br, ik = O.bond_flags()
    assert np.array_equal(G.bonds["broken"], br) and np.array_equal(G.bonds["in_k"], ik)
    gone = np.array(CASES[name][0]["gone"], np.uint8)
    gone[ro["retired"]] = 1
    assert np.array_equal(G.nodes["gone"], gone)
    # no rebuild on either side: the downdated K is the oracle's, bit for bit
    a, b = G.debug_matrix(), O.matrix()
    assert np.array_equal(a["rowptr"], b["rowptr"]) and np.array_equal(a["col"], b["col"])
    assert np.array_equal(a["val"], b["val"])


def test_cascade_with_the_worlds_solve_policy():
    """rtol 1e-8, 200 iterations a solve, rebuild after 60 (restarts and rebuilds happen): the same
    rounds as the oracle's; the rebuild decisions may fall at other rounds (iteration counts
    differ), which moves u by the solve tolerance only."""
    nodes, bonds, mats, f, ko, so, judged, has = CASES["tower_f20"]
    O = oracle.Port(nodes, bonds, mats)
    o = CascadeOptions(**dict(ko, rtol=1e-10, maxit=400))
    ro = oracle.cascade(O, f, np.zeros(6 * len(nodes)), o, StressOptions(**so), judged, has)
    G = StressProblem(nodes, bonds, mats)
    u, res, ex = G.cascade(f, options=o, opt=StressOptions(**so))
    assert ex["broken"] == ro["broken"] and ex["retired"] == ro["retired"]
    assert res.status == ro["status"] == 0
    assert relerr(u, ro["u"]) <= 1e-6


def test_cascade_many_breaks_a_round():
    """A round that breaks more bonds than the selection sorts in shared memory (2048): the
    global-memory sort, with ties in phi (a symmetric tower)."""
    nodes, bonds, f, mats = synth.tower_graph(10)
    o = CascadeOptions(rtol=1e-10, maxit=4000, rebuild_after=1 << 30, fragility=400.0, max_breaks_per_round=3000,
                       max_rounds=1, break_band=0.0)
    O = oracle.Port(nodes, bonds, mats)
    ro = oracle.cascade(O, f, np.zeros(6 * len(nodes)), o)
    assert ro["per_round"][0] > 2048
    G = StressProblem(nodes, bonds, mats)
    u, res, ex = G.cascade(f, options=o)
    assert ex["broken"] == ro["broken"] and ex["retired"] == ro["retired"]
    assert res.status == ro["status"] and res.rounds == 1


def test_cascade_nothing_over():
    nodes, bonds = fx.lattice(5)
    G = StressProblem(nodes, bonds, default_materials())
    f = fx.gravity_live(nodes)
    u, res, ex = G.cascade(f, options=CascadeOptions(rtol=1e-10))
    assert res.status == 0 and res.rounds == 0 and res.solves == 1 and ex["broken"] == []
    assert 0.0 < res.max_utilization < 1.0
    u2, r2 = G.solve(f, rtol=1e-10, maxit=1000)
    assert relerr(u, u2) <= 1e-6


def test_cascade_max_rounds_zero_is_a_judgement():
    """max_rounds = 0: one solve and one judgement; phi and the judged loads are the oracle's
    judgement of the same u, bit for bit (lerp from given judged loads, shock on)."""
    nodes, bonds, mats, f, ko, so, judged, has = CASES["tower_f7_shock"]
    o = CascadeOptions(**dict(ko, **TIGHT, max_rounds=0))
    G = StressProblem(nodes, bonds, mats)
    u, res, ex = G.cascade(f, options=o, judged=judged, has=has)
    assert res.status == 1 and res.rounds == 0
    O = oracle.Port(nodes, bonds, mats)
    loads, _, _ = O.judge(u, o.fragility)
    le = loads.copy()
    for k in oracle.LOAD_FIELDS:
        le[k] = judged[k] + o.dif * (loads[k] - judged[k])
    phi, _ = O.utilization_many(le, o.fragility)
    assert np.array_equal(ex["phi"], phi)
    assert ex["judged"].tobytes() == loads.tobytes()


@pytest.mark.parametrize("jacobi", [False, True], ids=["amg", "jacobi"])
def test_retire_many_nodes_bit_exact(jacobi):
    """retire_nodes of a whole block of a lattice (hundreds of bonds: the parallel in-order
    downdate): K and the solve after it as the oracle's."""
    nodes, bonds = fx.lattice(8)
    mats = default_materials()
    opt = StressOptions(amg_min_nodes=1 << 30 if jacobi else 16)
    G = StressProblem(nodes, bonds, mats)
    O = oracle.Port(nodes, bonds, mats)
    assert G.assemble(opt) and O.assemble(opt)
    z = np.rint(nodes["c"]["z"] / 0.4 - 0.5).astype(int)
    x = np.rint(nodes["c"]["x"] / 0.4 - 0.5).astype(int)
    lst = np.nonzero((z >= 5) & (x >= 3))[0].astype(np.int32)
    G.retire_nodes(lst)
    O.retire_nodes(lst)
    a, b = G.debug_matrix(), O.matrix()
    assert np.array_equal(a["val"], b["val"])
    br, ik = O.bond_flags()
    assert np.array_equal(G.bonds["broken"], br) and np.array_equal(G.bonds["in_k"], ik)
    f = fx.gravity_live(G.nodes)
    u, r = G.solve(f, rtol=1e-11, maxit=4000)
    uo, _ = O.solve(f, rtol=1e-11, maxit=4000)
    assert r.converged and relerr(u, uo) <= 1e-6


# (detach = 0 is left out: the parts the rounds cut off then float, K is singular and where a solve
# of an inconsistent singular system breaks down depends on rounding, not on the reference's rules)
@pytest.mark.parametrize("over", [dict(max_breaks_per_round=1, max_rounds=12), dict(break_band=1.0),
                                  dict(max_rounds=3), dict(dif=1.0, shock=1)],
                         ids=["one_a_round", "band_1", "three_rounds", "no_blend"])
def test_cascade_options_match_oracle(over):
    """The rounds' options as the reference's world config varies them: the same bonds broken in
    order, the same nodes retired, the same ending."""
    name = "tower_f9" if "dif" not in over else "tower_f7_shock"
    G, O, ro, u, res, ex = run_both(name, **over)
    assert res.status == ro["status"] and res.rounds == ro["rounds"]
    assert ex["broken"] == ro["broken"] and ex["retired"] == ro["retired"]
    assert relerr(u, ro["u"]) <= 1e-6


def test_cascade_mixed_precision_problem():
    """A problem assembled for mixed precision at every size: its solves (FP32 inner sequences,
    FP64 refinement, K downdated in FP64 only) reach the same tight tolerance, so the rounds are
    the oracle's."""
    nodes, bonds, mats, f, ko, so, judged, has = CASES["tower_f9"]
    kw = dict(ko, **TIGHT)
    O = oracle.Port(nodes, bonds, mats)
    ro = oracle.cascade(O, f, np.zeros(6 * len(nodes)), CascadeOptions(**kw), StressOptions(**so))
    G = StressProblem(nodes, bonds, mats)
    mixed = StressOptions(precision=2, **so)
    assert G.assemble(mixed)
    u, res, ex = G.cascade(f, options=CascadeOptions(**kw), opt=mixed)
    assert res.status == ro["status"] and ex["broken"] == ro["broken"] and ex["retired"] == ro["retired"]
    assert relerr(u, ro["u"]) <= 1e-6


@pytest.mark.parametrize("jacobi", [False, True], ids=["amg", "jacobi"])
def test_remove_bonds_list_bit_exact(jacobi):
    """remove_bonds (one device pass) of a list with repeats and bonds sharing nodes: K and the
    flags as the oracle's remove_bond calls in the same order."""
    nodes, bonds = fx.lattice(7)
    mats = default_materials()
    opt = StressOptions(amg_min_nodes=1 << 30 if jacobi else 16)
    G = StressProblem(nodes, bonds, mats)
    O = oracle.Port(nodes, bonds, mats)
    assert G.assemble(opt) and O.assemble(opt)
    rng = np.random.default_rng(5)
    lst = rng.choice(len(bonds), size=60, replace=False).astype(np.int32)
    lst = np.concatenate([lst, lst[:5]])  # (repeats: no-ops)
    G.remove_bonds(lst)
    for b in lst:
        O.remove_bond(int(b))
    a, b = G.debug_matrix(), O.matrix()
    assert np.array_equal(a["val"], b["val"])
    br, ik = O.bond_flags()
    assert np.array_equal(G.bonds["broken"], br) and np.array_equal(G.bonds["in_k"], ik)
    assert G.preconditioner_current() == O.preconditioner_current()
