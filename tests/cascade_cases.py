"""Graphs and options of the break-round (cascade) tests: shared by the oracle pin
(test_oracle_pin.py), the golden writer (golden/make_golden.py) and the device parity tests
(test_gpu_cascade.py)."""
from __future__ import annotations

import numpy as np

import fixtures as fx
from opus_destruct_2_gb300 import synth
from opus_destruct_2_gb300.graph import LOAD_DTYPE, CascadeOptions, StressOptions, default_materials


def _tower():
    nodes, bonds, f, mats = synth.tower_graph(6, 8, 8)
    return nodes, bonds, mats, f


def _lattice_shock():
    """A lattice loaded at 140 g whose bonds were judged at a third of that: the dynamic
    increase factor carries some over strength."""
    import oracle
    nodes, bonds = fx.lattice(6)
    mats = default_materials()
    f = fx.gravity_live(nodes) * 140.0
    P = oracle.Port(nodes, bonds, mats)
    P.assemble(StressOptions(amg_min_nodes=16))
    u, _ = P.solve(f / 3.0, rtol=1e-12, maxit=1000)
    loads, _, _ = P.judge(u)
    return nodes, bonds, mats, f, loads


def _tower_judged(nodes, bonds, mats, f):
    """The tower's bond loads under a third of its load (the steady state before a change)."""
    import oracle
    P = oracle.Port(nodes, bonds, mats)
    P.assemble(StressOptions())
    u, _ = P.solve(f / 3.0, rtol=1e-12, maxit=1000)
    loads, _, _ = P.judge(u)
    return loads


def cases():
    """name -> (nodes, bonds, mats, f, CascadeOptions kwargs, StressOptions kwargs, judged, has)."""
    out = {}
    nodes, bonds, mats, f = _tower()
    base = dict(rtol=1e-8, maxit=200)
    out["tower_f9"] = (nodes, bonds, mats, f, dict(base, fragility=9.0), {}, None, None)
    out["tower_f20"] = (nodes, bonds, mats, f, dict(base, fragility=20.0), {}, None, None)
    out["tower_f9_jacobi"] = (nodes, bonds, mats, f, dict(base, fragility=9.0), dict(amg_min_nodes=1 << 30), None, None)
    out["tower_f20_band"] = (nodes, bonds, mats, f, dict(base, fragility=20.0, max_breaks_per_round=4, break_band=0.95),
                             {}, None, None)
    out["tower_f7_shock"] = (nodes, bonds, mats, f, dict(base, fragility=7.0, shock=1), {},
                             _tower_judged(nodes, bonds, mats, f), np.ones(len(bonds), np.uint8))
    ln, lb, lm, lf, loads = _lattice_shock()
    out["lattice_shock"] = (ln, lb, lm, lf, dict(base, shock=1), dict(amg_min_nodes=16), loads,
                            np.ones(len(lb), np.uint8))
    return out


def options(kw) -> CascadeOptions:
    return CascadeOptions(**kw)


def stress_options(kw) -> StressOptions:
    return StressOptions(**kw)


def empty_judged(nb: int):
    return np.zeros(nb, LOAD_DTYPE), np.zeros(nb, np.uint8)


def load_golden(path):
    """A tests/golden/cascade/*.npz: (nodes, bonds, mats, f, CascadeOptions kwargs, StressOptions
    kwargs, judged, has, expected outputs)."""
    g = np.load(path)
    ko = {str(k): (int(v) if str(k) not in ("rtol", "fragility", "dif", "break_band") else float(v))
          for k, v in zip(g["okeys"], g["ovals"])}
    so = {str(k): int(v) for k, v in zip(g["skeys"], g["svals"])}
    judged = g["judged_in"] if g["judged_in"].size else None
    has = g["has_in"] if g["has_in"].size else None
    c = [int(x) for x in g["counts"]]
    exp = dict(status=c[0], rounds=c[1], bonds_broken=c[2], nodes_retired=c[3], solves=c[4], restarts=c[5],
               pcg_iters=c[6], u=g["u"], phi=g["phi"], judged=g["judged"], has=g["has"], broken=g["broken"].tolist(),
               retired=g["retired"].tolist(), per_round=g["per_round"].tolist(),
               max_utilization=float(g["max_utilization"]))
    return g["nodes"], g["bonds"], g["mats"], g["f"], ko, so, judged, has, exp
