"""A batch's iteration bodies skip the rows of graphs whose sequence has stopped (the SpMV and every
level of the V-cycle; solve.cu seg_body, vcycle.cu): the running graphs' results must be the same
bits as without the skipping (SVXG_NO_ROW_SKIP=1, read once per process, so each side runs in a
process of its own).

Cases: a batch of ten graphs of 12-4,000 fragments solved cold (FP64 and the mixed-precision
policy), its graphs stopping one after another; and bundle repeats through the server - one
member's bonds removed and solved warm while the other members stay stopped, then two members at
once. Compared bit for bit: every graph's u, iterations, rel. residual and failure list.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCRIPT = r'''
import sys
import numpy as np
from opus_destruct_2_gb300 import Batch, synth
from opus_destruct_2_gb300.graph import PRECISION_MIXED, StressOptions, default_materials
from opus_destruct_2_gb300.server import Server

MATS = default_materials()
out = {}
gs = []
for k, (size, free) in enumerate([(12, True), (40, False), (150, True), (300, False), (700, True), (1500, False),
                                  (2500, True), (90, False), (500, True), (4000, False)]):
    n, b, f, _ = synth.piece_graph(size, free=free, seed=900 + k)
    gs.append((n, b, f))
for name, opt in (("fp64", StressOptions()), ("mixed", StressOptions(precision=PRECISION_MIXED))):
    B = Batch([(g[0], g[1]) for g in gs], MATS)
    assert B.assemble(opt)
    us, res, rel, conv = B.solve([g[2] for g in gs], rtol=1e-8, maxit=3000)
    out[name + "_u"] = np.concatenate(us)
    out[name + "_iters"] = B.iters.copy()
    out[name + "_rel"] = rel
    out[name + "_conv"] = conv
    judged = B.utilization(1.0)
    out[name + "_over"] = np.concatenate([j[2] for j in judged])

pieces = [synth.piece_graph(s, free=bool(k % 2), seed=31 + k)[:3] for k, s in enumerate((400, 250, 900, 120, 600, 300))]
rng = np.random.default_rng(5)
rms = [np.sort(rng.choice(len(b), size=max(1, len(b) // 30), replace=False)).astype(np.int32) for _, b, _ in pieces]
opt = StressOptions(precision=PRECISION_MIXED)
with Server(workers=1, budget=8 << 30) as S:
    S.set_batching(8, 20000, 65536)
    S.hold(True)
    t = [S.submit(n, b, MATS, f, structure=20 + k, opt=opt, rtol=1e-8, maxit=3000)
         for k, (n, b, f) in enumerate(pieces)]
    S.hold(False)
    first = [S.wait(x) for x in t]
    assert S.stats().batches == 1
    # one member changes while the other five stay stopped
    r, u, over = S.wait(S.submit_repeat(22, rms[2], pieces[2][2], rtol=1e-8, maxit=3000, want_over=True,
                                        nb=len(pieces[2][1])))
    assert r.status == 0 and r.converged
    out["rep1_u"], out["rep1_over"], out["rep1_iters"] = u, over, np.array([r.iters])
    # two members together
    S.hold(True)
    t = [S.submit_repeat(20 + k, rms[k], pieces[k][2], rtol=1e-8, maxit=3000, want_over=True, nb=len(pieces[k][1]))
         for k in (0, 4)]
    S.hold(False)
    for k, x in zip((0, 4), t):
        r, u, over = S.wait(x)
        assert r.status == 0 and r.converged
        out[f"rep2_{k}_u"], out[f"rep2_{k}_over"], out[f"rep2_{k}_iters"] = u, over, np.array([r.iters])
    for k, (r, u, _) in enumerate(first):
        out[f"first_{k}_u"] = u
np.savez(sys.argv[1], **out)
'''


def run(tmp_path, name, skip_off):
    script = tmp_path / "row_skip_case.py"
    script.write_text(SCRIPT)
    out = tmp_path / f"{name}.npz"
    env = dict(os.environ)
    env["PYTHONPATH"] = ROOT + os.pathsep + env.get("PYTHONPATH", "")
    env.pop("SVXG_NO_ROW_SKIP", None)
    if skip_off:
        env["SVXG_NO_ROW_SKIP"] = "1"
    r = subprocess.run([sys.executable, str(script), str(out)], cwd=ROOT, env=env, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    return dict(np.load(out))


def test_row_skip_changes_no_bits(tmp_path):
    on = run(tmp_path, "on", False)
    off = run(tmp_path, "off", True)
    assert on.keys() == off.keys()
    for k in sorted(on):
        assert on[k].shape == off[k].shape, k
        assert np.array_equal(on[k], off[k]), k
    # the batches' graphs stopped at different iterations (so rows were skipped on the way)
    assert len(set(on["fp64_iters"].tolist())) > 1
