"""World::Impl::probe_utilization (core/src/world/world.cpp:1907-1940) through the product API on
the device, against the oracle: the structure's load vector (svxg_structure_loads), assemble,
solve to rel. residual 1e-8 (warm, up to 5000 iterations), every intact bond's utilization from
its load (svxg_bond_utilization on the device's bond loads), the worst one and the count over
strength; then a bond removed in place and the probe again (the assembled operator kept, as the
reference keeps it).

Bars: the worst utilization within 1e-6 (relative) of the oracle's, the count over strength the
same, and every bond's phi within 1e-6 of the largest."""
import numpy as np
import pytest

import oracle
import opus_destruct_2_gb300 as lib
from opus_destruct_2_gb300 import StressProblem, synth
from opus_destruct_2_gb300.graph import StressOptions

pytestmark = pytest.mark.gpu


def probe(P, bonds, f, u, fragility, mats, loads, removed=()):
    """solve (1e-8, warm, 5000) and every intact bond's phi from its load (world.cpp:1920-1933)."""
    u, res = P.solve(f, u=u, rtol=1e-8, maxit=5000, warm=True)
    assert res.converged
    L = loads(P, u)
    phi = np.array([0.0 if b in removed else lib.bond_utilization(bonds[b], L[b], fragility, mats)[0]
                    for b in range(len(L))])
    return u, phi


@pytest.mark.parametrize("name", ["tower10", "piece"])
def test_probe_utilization_matches_oracle(name):
    if name == "tower10":
        nodes, bonds, _, mats = synth.tower_graph(storeys=10, seed=1)
    else:
        nodes, bonds, _, mats = synth.piece_graph(1200, free=False, seed=5)
    weight = nodes["mass"] * 9.81 * (nodes["fixed"] == 0)
    f = lib.structure_loads(weight, np.zeros(6 * len(nodes)))
    so = StressOptions(rtol=2e-3)
    G = StressProblem(nodes, bonds, mats)
    assert G.assemble(so)
    O = oracle.Port(nodes, bonds, mats)
    assert O.assemble(so)
    b = G.bonds.copy()
    ug, ph_g = probe(G, b, f, np.zeros(6 * len(nodes)), 1.0, mats, lambda P, u: P.bond_loads(u))
    uo, ph_o = probe(O, b, f, np.zeros(6 * len(nodes)), 1.0, mats, lambda P, u: P.judge(u)[0])
    frag = 1.0 / float(np.quantile(ph_o[ph_o > 0], 0.95))  # (about 5 % of the bonds over strength)
    ph_g, ph_o = ph_g * frag, ph_o * frag
    assert abs(ph_g.max() - ph_o.max()) <= 1e-6 * ph_o.max()
    assert np.max(np.abs(ph_g - ph_o)) <= 1e-6 * ph_o.max()
    band = np.abs(ph_o - 1.0) <= np.max(np.abs(ph_g - ph_o))
    assert np.count_nonzero(ph_g >= 1.0) == np.count_nonzero(ph_o >= 1.0) or band.any()
    # a bond removed in place, the probe again from the last u (warm)
    k = int(np.argmax(ph_o))
    G.remove_bond(k)
    O.remove_bond(k)
    ug, ph_g = probe(G, b, f, ug, frag, mats, lambda P, u: P.bond_loads(u), removed={k})
    uo, ph_o = probe(O, b, f, uo, frag, mats, lambda P, u: P.judge(u)[0], removed={k})
    assert ph_g[k] == 0.0 and ph_o[k] == 0.0
    assert abs(ph_g.max() - ph_o.max()) <= 1e-6 * ph_o.max()
    assert np.count_nonzero(ph_g >= 1.0) == np.count_nonzero(ph_o >= 1.0)
