"""A loose piece's break rounds on the device (svxg_piece_rounds, through the C ABI) against the
oracle's restatement (oracle.piece_rounds on the C restatement, itself pinned to the same rounds
run on the reference's StressProblem by test_oracle_pin.py / test_oracle_golden.py).

Bars: the same bonds broken in the same order with the same failure modes, the same chips, the
same ending (status, rounds), the same fracture energy spent and the same moved loads bit for bit
(the same bonds' costs and the same chip arithmetic in the same order); u and the rounds' largest
utilizations within 1e-6 (both sides solve to rtol 1e-10, far inside the cases' margins)."""
import numpy as np
import pytest

import oracle
import piece_cases as pc
from opus_destruct_2_gb300 import StressProblem
from opus_destruct_2_gb300.graph import PieceOptions

pytestmark = pytest.mark.gpu


def relerr(a, b):
    s = float(np.max(np.abs(b)))
    return float(np.max(np.abs(a - b)) / s) if s > 0 else float(np.max(np.abs(a - b), initial=0.0))


@pytest.mark.parametrize("name", list(pc.CASES), ids=list(pc.CASES))
def test_piece_rounds_match_oracle(name):
    nodes, bonds, mats, f, ko, gf = pc.case(name)
    o = pc.options(ko)
    ro = oracle.piece_rounds(oracle.Port(nodes, bonds, mats), f, np.zeros(6 * len(nodes)), o, gf)
    G = StressProblem(nodes, bonds, mats)
    u, f_out, res, ex = G.piece_rounds(f, options=o, gf=gf)
    assert res.status == ro["status"] and res.checks == ro["checks"]
    assert ex["broken"] == ro["broken"] and ex["modes"] == ro["modes"]
    assert ex["chips"] == ro["chip_nodes"] and res.chips == ro["chips"]
    assert res.spent == ro["spent"]
    assert np.array_equal(f_out, ro["f"])
    assert relerr(u, ro["u"]) <= 1e-6
    for a, b in ((res.first_max_utilization, ro["first_max_utilization"]), (res.max_utilization, ro["max_utilization"])):
        assert abs(a - b) <= 1e-6 * max(1.0, b)
    gone = np.array(nodes["gone"], np.uint8)
    gone[ro["chip_nodes"]] = 1
    assert np.array_equal(G.nodes["gone"], gone)


def test_piece_rounds_with_the_worlds_tolerance():
    """rtol 1e-2 and 60 iterations a solve, as the world runs pieces: the rounds complete and break
    bonds of the same piece; u matches the oracle's only to the solve tolerance, so the sequences
    are not compared."""
    nodes, bonds, mats, f, ko, gf = pc.case("chips_last_round")
    G = StressProblem(nodes, bonds, mats)
    u, f_out, res, ex = G.piece_rounds(f, options=PieceOptions(energy=-1.0), gf=gf)
    assert res.checks >= 1 and res.bonds_broken >= 1 and res.status in (0, 2, 3, 4)
    assert np.all(np.isfinite(u))


def test_piece_nothing_over():
    nodes, bonds, mats, f, ko, gf = pc.case("chips_settled")
    G = StressProblem(nodes, bonds, mats)
    u, f_out, res, ex = G.piece_rounds(f * 1e-3, options=pc.options(ko), gf=gf)
    assert res.status == 0 and res.checks == 1 and ex["broken"] == [] and res.spent == 0.0
    assert np.array_equal(f_out, f * 1e-3)


def test_batch_piece_rounds_match_one_by_one():
    """The same pieces through the server, all in flight at once: each piece's rounds as when it
    runs alone (tight solves: the same bonds, chips and moved loads)."""
    from opus_destruct_2_gb300.server import Server
    names = list(pc.CASES)
    cases = [pc.case(nm) for nm in names]
    o = pc.options(cases[0][4])
    with Server(workers=4) as S:
        pres, res, us, fs, lists = S.batch_piece_rounds([(c[0], c[1], c[3]) for c in cases], cases[0][2], options=o,
                                                        gf=cases[0][5], want_lists=True)
    for i, (nodes, bonds, mats, f, ko, gf) in enumerate(cases):
        assert res[i].status == 0
        G = StressProblem(nodes, bonds, mats)
        u, f_out, r1, ex = G.piece_rounds(f, options=o, gf=gf)
        assert pres[i].status == r1.status and pres[i].bonds_broken == r1.bonds_broken
        assert lists[i]["broken"] == ex["broken"] and lists[i]["chips"] == ex["chips"]
        assert np.array_equal(fs[i], f_out)
        assert relerr(us[i], u) <= 1e-8


@pytest.mark.parametrize("over", [dict(rounds=1), dict(max_breaks_per_round=1), dict(energy=0.0),
                                  dict(round_fraction=1.0), dict(break_band=1.0, energy=5000.0)],
                         ids=["one_round", "one_a_round", "no_energy", "all_over", "band_energy"])
def test_piece_options_match_oracle(over):
    nodes, bonds, mats, f, ko, gf = pc.case("many_chips")
    o = pc.options(dict(ko, **over))
    ro = oracle.piece_rounds(oracle.Port(nodes, bonds, mats), f, np.zeros(6 * len(nodes)), o, gf)
    G = StressProblem(nodes, bonds, mats)
    u, f_out, res, ex = G.piece_rounds(f, options=o, gf=gf)
    assert res.status == ro["status"] and res.checks == ro["checks"]
    assert ex["broken"] == ro["broken"] and ex["modes"] == ro["modes"] and ex["chips"] == ro["chip_nodes"]
    assert res.spent == ro["spent"] and np.array_equal(f_out, ro["f"])
    assert relerr(u, ro["u"]) <= 1e-6
