"""The oracle against the golden fixtures written from the reference itself
(tests/golden/make_golden.py): bit for bit, on any machine (the restatement evaluates every
expression as the reference does, -ffp-contract=off, so x86 and Arm agree)."""
import glob
import os

import numpy as np
import pytest

from opus_destruct_2_gb300.graph import StressOptions
from oracle import Port

FILES = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))


@pytest.mark.parametrize("path", FILES, ids=[os.path.basename(p)[:-4] for p in FILES])
def test_oracle_matches_reference_golden(path):
    g = np.load(path)
    amg_min, smoothed, reagg, cdense = (int(x) for x in g["opts"])
    opt = StressOptions(amg_min_nodes=amg_min, smoothed=smoothed, reaggregate=reagg, coarsen_dense=cdense)
    P = Port(g["nodes"], g["bonds"], g["mats"])
    assert P.assemble(opt)
    u, r = P.solve(g["f"], rtol=1e-12, maxit=5000)
    assert r.iters == int(g["iters"]) and r.rel_res == float(g["rel_res"]) and r.converged == int(g["converged"])
    assert np.array_equal(u, g["u"])
    i = P.info()
    assert i.sizes() == list(g["level_sizes"]) and i.blocks() == list(g["level_blocks"])
    assert [i.nfree, i.chol_n, i.matrix_blocks, i.work_per_iteration, i.assembly_work, i.work_per_apply,
            i.build_work] == list(g["counters"])
    loads, phi, mode = P.judge(g["u"])
    assert np.array_equal(loads, g["loads"]) and np.array_equal(phi, g["phi"]) and np.array_equal(mode, g["mode"])


import cascade_cases as cc  # noqa: E402
import fixtures as fx  # noqa: E402
from oracle import cascade  # noqa: E402

CASCADE_FILES = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "cascade", "*.npz")))


@pytest.mark.parametrize("path", CASCADE_FILES, ids=[os.path.basename(p)[:-4] for p in CASCADE_FILES])
def test_oracle_cascade_matches_reference_golden(path):
    """The break rounds on the C restatement against the same rounds run on the reference's own
    StressProblem (golden/make_golden.py): bit for bit."""
    nodes, bonds, mats, f, ko, so, judged, has, exp = cc.load_golden(path)
    P = Port(nodes, bonds, mats)
    r = cascade(P, f, np.zeros(6 * len(nodes)), cc.options(ko), cc.stress_options(so), judged, has)
    for k in ("status", "rounds", "bonds_broken", "nodes_retired", "solves", "restarts", "pcg_iters", "broken",
              "retired", "per_round", "max_utilization"):
        assert r[k] == exp[k], k
    assert np.array_equal(r["u"], exp["u"]) and np.array_equal(r["phi"], exp["phi"])
    assert r["judged"].tobytes() == exp["judged"].tobytes() and np.array_equal(r["has"], exp["has"])


def test_select_breaks_rules():
    """The round's selection (world.cpp:1219-1271) on hand-made over-strength lists: phi
    descending, index ascending on ties; everything at or over max(1, band x max); at least the
    worst quarter; at most max_breaks."""
    from oracle import select_breaks
    b = np.array([3, 7, 9, 12, 20, 21, 30, 31], np.int64)
    phi = np.array([1.2, 2.0, 1.0, 2.0, 1.9, 1.05, 1.1, 1.71])
    # thr = max(1, 0.85 x 2.0) = 1.7: 7, 12 (ties by index), 20, 31
    assert select_breaks(b, phi, 0.85, 256) == [7, 12, 20, 31]
    assert select_breaks(b, phi, 0.85, 3) == [7, 12, 20]
    # band 0.99: thr 1.98 -> 2 bonds, but the quota is (8 + 3) / 4 = 2
    assert select_breaks(b, phi, 0.99, 256) == [7, 12]
    # band 0.5: thr max(1, 1.0) = 1 -> every one
    assert select_breaks(b, phi, 0.5, 256) == [7, 12, 20, 31, 3, 30, 21, 9]
    # one over: one break
    assert select_breaks(np.array([5]), np.array([1.0]), 0.85, 256) == [5]
    # quota above the band: 9 over, thr picks 1, quota (9 + 3) / 4 = 3
    b9 = np.arange(9)
    p9 = np.array([1.0, 1.0, 5.0, 1.1, 1.2, 1.0, 1.0, 1.0, 1.3])
    assert select_breaks(b9, p9, 0.85, 256) == [2, 8, 4]


SECTION_FILES = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "sections", "*.npz")))


@pytest.mark.parametrize("path", SECTION_FILES, ids=[os.path.basename(p)[:-4] for p in SECTION_FILES])
def test_oracle_sections_match_reference_golden(path):
    """Section geometry of the C restatement against the bonds the reference's own
    SecAcc::finish_lattice + section_strengths made of the same interfaces: bit for bit."""
    from oracle import build_bonds
    g = np.load(path)
    js, lats = g["junctions"], g["lattices"]
    out = build_bonds(g["nodes"], g["secs"], g["faces"], g["mats"], junctions=js if len(js) else None,
                      lattices=lats if len(lats) else None)
    assert fx.same_records(out, g["bonds"])


import piece_cases as pc  # noqa: E402
from oracle import piece_rounds  # noqa: E402

PIECE_FILES = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "pieces", "*.npz")))


@pytest.mark.parametrize("path", PIECE_FILES, ids=[os.path.basename(p)[:-4] for p in PIECE_FILES])
def test_oracle_piece_rounds_match_reference_golden(path):
    """A piece's break rounds on the C restatement against the same rounds run on the reference's
    own StressProblem (golden/make_golden.py): bit for bit."""
    nodes, bonds, mats, f, ko, gf, exp = pc.load_golden(path)
    r = piece_rounds(Port(nodes, bonds, mats), f, np.zeros(6 * len(nodes)), pc.options(ko), gf)
    for k in ("status", "checks", "bonds_broken", "chips", "pcg_iters", "rebuilt", "spent", "first_max_utilization",
              "max_utilization", "broken", "modes", "chip_nodes"):
        assert r[k] == exp[k], k
    assert np.array_equal(r["u"], exp["u"]) and np.array_equal(r["f"], exp["f"])
