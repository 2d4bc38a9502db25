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
