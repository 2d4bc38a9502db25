"""Loose pieces of the break-round tests (World::Impl::body_stress_run's rounds,
core/src/world/world_pieces.cpp:614-808): seeded free pieces of about 300 fragments with one impact
load, solved tight (rtol 1e-10) so that the device and the oracle see the same utilizations.
Between them the cases end in every way the rounds end: nothing over strength, the impact's
energy spent, the piece apart, the last round; several retire chips. Shared by
test_oracle_pin.py, golden/make_golden.py and test_gpu_pieces.py."""
from __future__ import annotations

from opus_destruct_2_gb300 import synth
from opus_destruct_2_gb300.graph import PieceOptions, default_fracture_energies

# (seed, impact N, energy J (< 0: a resting load), chip fraction)
CASES = {
    "chips_settled": (3, 3e6, -1.0, 0.04),
    "chips_last_round": (6, 3e6, -1.0, 0.04),
    "energy_spent": (6, 3e6, 2000.0, 0.04),
    "apart": (1, 1e7, -1.0, 0.01),
    "many_chips": (5, 1e7, -1.0, 0.01),
    "heavy": (2, 2e7, -1.0, 0.04),
}


def case(name: str):
    """(nodes, bonds, mats, f, PieceOptions kwargs, Gf per material)."""
    seed, impact, energy, chip = CASES[name]
    nodes, bonds, f, mats = synth.piece_graph(300, free=True, seed=seed, impact=impact)
    return nodes, bonds, mats, f, dict(energy=energy, chip_fraction=chip, rtol=1e-10, maxit=3000), \
        default_fracture_energies()


def options(kw) -> PieceOptions:
    return PieceOptions(**kw)


def load_golden(path):
    """A tests/golden/pieces/*.npz: (nodes, bonds, mats, f, PieceOptions kwargs, gf, expected)."""
    import numpy as np
    g = np.load(path)
    ints = ("maxit", "rounds", "max_breaks_per_round")
    ko = {str(k): (int(v) if str(k) in ints else float(v)) for k, v in zip(g["okeys"], g["ovals"])}
    c = [int(x) for x in g["counts"]]
    r = [float(x) for x in g["reals"]]
    exp = dict(status=c[0], checks=c[1], bonds_broken=c[2], chips=c[3], pcg_iters=c[4], rebuilt=c[5], spent=r[0],
               first_max_utilization=r[1], max_utilization=r[2], broken=g["broken"].tolist(),
               modes=g["modes"].tolist(), chip_nodes=g["chip_nodes"].tolist(), u=g["u"], f=g["f_out"])
    return g["nodes"], g["bonds"], g["mats"], g["f"], ko, g["gf"], exp
