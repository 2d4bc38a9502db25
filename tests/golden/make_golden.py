"""Writes the golden fixtures under tests/golden/ from the reference itself.

Runs only where the reference tree is present (the reference is compiled from its own sources by
oracle/build_oracle.py into oracle/_ref/). For each case it stores the input graph and the
reference StressProblem's outputs: u (solved to rtol 1e-12), the PCG result, the hierarchy and
work counters, and every bond's load, utilization and mode. tests/test_oracle_golden.py checks the
oracle against them on any machine, bit for bit.

    python tests/golden/make_golden.py

It also writes tests/golden/cascade/*.npz: the judge's break rounds of tests/cascade_cases.py
run on the reference's own StressProblem (tests/test_oracle_golden.py checks the oracle's
cascade against them bit for bit), and tests/golden/sections/*.npz: voxel-face interfaces and the
bonds the reference's section geometry makes of them, and tests/golden/pieces/*.npz: loose pieces'
break rounds run on the reference's own StressProblem.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)

import fixtures as fx  # noqa: E402
from opus_destruct_2_gb300 import synth  # noqa: E402
from opus_destruct_2_gb300.graph import StressOptions, default_materials  # noqa: E402
from oracle import Reference, reference_lib  # noqa: E402

CASES = {
    "cantilever12": (lambda: fx.cantilever(12, 0.5, 300.0), dict(amg_min_nodes=4)),
    "lattice8_amg": (lambda: fx.lattice(8), dict(amg_min_nodes=16)),
    "lattice8_jacobi": (lambda: fx.lattice(8), dict(amg_min_nodes=1 << 30)),
    "lattice12_retired": (lambda: fx.lattice(12, keep_z=8, retire_top=True), dict(amg_min_nodes=16)),
    "tower3": (lambda: synth.tower_graph(storeys=3, seed=3)[:2], dict()),
    "piece_free": (lambda: synth.piece_graph(400, free=True, seed=31)[:2], dict(amg_min_nodes=0)),
}


def main():
    if reference_lib() is None:
        raise SystemExit("the reference is not built here")
    mats = default_materials()
    for name, (make, opts) in CASES.items():
        nodes, bonds = make()
        f = fx.gravity_live(nodes)
        opt = StressOptions(**opts)
        R = Reference(nodes, bonds, mats)
        r = R.solve(f, opt, rtol=1e-12, maxit=5000)
        loads, phi, mode = R.judge(r["u"])
        info = r["info"]
        np.savez_compressed(
            os.path.join(HERE, f"{name}.npz"),
            nodes=nodes, bonds=bonds, mats=mats, f=f, u=r["u"], loads=loads, phi=phi, mode=mode,
            iters=r["res"].iters, rel_res=r["res"].rel_res, converged=r["res"].converged,
            level_sizes=np.array(info.sizes(), np.int64), level_blocks=np.array(info.blocks(), np.int64),
            counters=np.array([info.nfree, info.chol_n, info.matrix_blocks, info.work_per_iteration,
                               info.assembly_work, info.work_per_apply, info.build_work], np.int64),
            opts=np.array([opt.amg_min_nodes, opt.amg.smoothed, opt.amg.reaggregate, opt.amg.coarsen_dense],
                          np.int64))
        print(name, len(nodes), len(bonds), r["res"], info.sizes())


def cascades():
    """tests/golden/cascade/<case>.npz: the break rounds of tests/cascade_cases.py run on the
    reference's own StressProblem (oracle.RefProblem): inputs and every output."""
    import cascade_cases as cc
    from oracle import RefProblem, cascade
    out_dir = os.path.join(HERE, "cascade")
    os.makedirs(out_dir, exist_ok=True)
    for name, (nodes, bonds, mats, f, ko, so, judged, has) in cc.cases().items():
        R = RefProblem(nodes, bonds, mats)
        o = cc.options(ko)
        r = cascade(R, f, np.zeros(6 * len(nodes)), o, cc.stress_options(so), judged, has)
        okeys = sorted(ko)
        skeys = sorted(so)
        np.savez_compressed(
            os.path.join(out_dir, f"{name}.npz"), nodes=nodes, bonds=bonds, mats=mats, f=f,
            judged_in=judged if judged is not None else np.zeros(0), has_in=has if has is not None else np.zeros(0),
            okeys=np.array(okeys), ovals=np.array([float(ko[k]) for k in okeys]),
            skeys=np.array(skeys, dtype=str), svals=np.array([float(so[k]) for k in skeys]),
            u=r["u"], phi=r["phi"], judged=r["judged"], has=r["has"], broken=np.array(r["broken"], np.int32),
            retired=np.array(r["retired"], np.int32), per_round=np.array(r["per_round"], np.int32),
            counts=np.array([r["status"], r["rounds"], r["bonds_broken"], r["nodes_retired"], r["solves"],
                             r["restarts"], r["pcg_iters"]], np.int64),
            max_utilization=r["max_utilization"])
        print("cascade", name, r["status"], r["rounds"], r["bonds_broken"], r["nodes_retired"])


def sections():
    """tests/golden/sections/<case>.npz: interfaces of tests/section_cases.py (the small ones) and
    the bonds the reference's own SecAcc::finish_lattice + section_strengths make of them."""
    import section_cases as sc
    from oracle import build_bonds
    out_dir = os.path.join(HERE, "sections")
    os.makedirs(out_dir, exist_ok=True)
    from opus_destruct_2_gb300.graph import JUNCTION_DTYPE, LATTICE_DTYPE
    for name in ("tower2", "piece", "handmade", "general"):
        js, lats = np.zeros(0, JUNCTION_DTYPE), np.zeros(0, LATTICE_DTYPE)
        if name == "tower2":
            nodes, _, _, mats = synth.tower_graph(2, seed=5)
            secs, faces = synth.last_sections()
        elif name == "piece":
            nodes, secs, faces, mats = sc.generated("piece")
        elif name == "handmade":
            nodes, secs, faces, mats = sc.handmade()
        else:
            nodes, secs, faces, js, lats, mats = sc.general(4, count=120)
        bonds = build_bonds(nodes, secs, faces, mats, reference=True, junctions=js if len(js) else None,
                            lattices=lats if len(lats) else None)
        np.savez_compressed(os.path.join(out_dir, f"{name}.npz"), nodes=nodes, secs=secs, faces=faces, mats=mats,
                            junctions=js, lattices=lats, bonds=bonds)
        print("sections", name, len(secs), len(faces), len(js))


def pieces():
    """tests/golden/pieces/<case>.npz: the break rounds of tests/piece_cases.py run on the
    reference's own StressProblem (oracle.RefProblem): inputs and outputs."""
    import piece_cases as pc
    from oracle import RefProblem, piece_rounds
    out_dir = os.path.join(HERE, "pieces")
    os.makedirs(out_dir, exist_ok=True)
    for name in pc.CASES:
        nodes, bonds, mats, f, ko, gf = pc.case(name)
        r = piece_rounds(RefProblem(nodes, bonds, mats), f, np.zeros(6 * len(nodes)), pc.options(ko), gf)
        okeys = sorted(ko)
        np.savez_compressed(
            os.path.join(out_dir, f"{name}.npz"), nodes=nodes, bonds=bonds, mats=mats, f=f, gf=gf,
            okeys=np.array(okeys), ovals=np.array([float(ko[k]) for k in okeys]), u=r["u"], f_out=r["f"],
            broken=np.array(r["broken"], np.int32), modes=np.array(r["modes"], np.int32),
            chip_nodes=np.array(r["chip_nodes"], np.int32),
            counts=np.array([r["status"], r["checks"], r["bonds_broken"], r["chips"], r["pcg_iters"], r["rebuilt"]],
                            np.int64),
            reals=np.array([r["spent"], r["first_max_utilization"], r["max_utilization"]]))
        print("piece", name, r["status"], r["checks"], r["bonds_broken"], r["chips"])


if __name__ == "__main__":
    main()
    cascades()
    sections()
    pieces()
