"""The load builders and the judge's free functions of the product API, on the host (no GPU):
svxg_structure_loads, svxg_pin_reference, svxg_body_loads, svxg_bond_strength and
svxg_bond_utilization against the oracle.

Bars, all bit for bit:
  * structure loads (World::Impl::load_vector, core/src/world/world.cpp:966-974) and the pinned
    node (pin_reference, core/src/world/world_pieces.cpp:313-326) equal the C restatement's;
  * a loose piece's loads (inertial relief + point forces, world_pieces.cpp:566-603) equal the C
    restatement's and, where the reference tree is here, the same lines computed with the
    reference's own vector operators and StressProblem::add_force;
  * bond_utilization / bond_strength (core/src/stress/stress.cpp:14-57) equal the reference's
    compiled function (where present) and the oracle's on random bonds and loads, every failure
    mode and a bad material id.
"""
import ctypes

import numpy as np
import pytest

import fixtures as fx
import oracle
import opus_destruct_2_gb300 as lib
from opus_destruct_2_gb300.graph import (BOND_DTYPE, LOAD_DTYPE, NODE_DTYPE, POINT_FORCE_DTYPE, BodyState,
                                         default_materials, ptr)

MATS = default_materials()


def random_spd(rng, scale):
    a = rng.normal(size=(3, 3))
    return (a @ a.T + 3.0 * np.eye(3)) * scale


def with_centres(c):
    nodes = np.zeros(len(c), NODE_DTYPE)
    for i, k in enumerate("xyz"):
        nodes["c"][k] = c[:, i]
    return nodes


def random_body(rng, n, nforces):
    """A moving piece: state, nodes, per-node centre / mass / inertia, point forces (two of which
    name no node: they move the piece but load none)."""
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    I = random_spd(rng, 50.0)
    s = BodyState()
    s.x[:] = rng.normal(size=3) * 5.0
    s.q[:] = q
    s.com[:] = rng.normal(size=3)
    s.w[:] = rng.normal(size=3)
    s.inertia[:] = I.ravel()
    s.inv_inertia[:] = np.linalg.inv(I).ravel()
    s.inv_mass = 1.0 / 800.0
    s.gravity = 9.81
    c = rng.normal(size=(n, 3)) * 2.0
    nodes = with_centres(c)
    nodes["mass"] = rng.uniform(1.0, 40.0, n)
    node_com = c + rng.normal(size=(n, 3)) * 0.05
    node_mass = nodes["mass"].copy()
    node_inertia = np.stack([random_spd(rng, 0.5).ravel() for _ in range(n)])
    forces = np.zeros(nforces, POINT_FORCE_DTYPE)
    forces["F"] = rng.normal(size=(nforces, 3)) * 1e4
    forces["p"] = rng.normal(size=(nforces, 3)) * 3.0
    forces["node"] = rng.integers(0, n, nforces)
    forces["node"][:2] = [-1, n]
    return s, nodes, node_com, node_mass, node_inertia, forces


def test_structure_loads():
    rng = np.random.default_rng(3)
    w = rng.uniform(0.0, 1e4, 257)
    w[[0, 5]] = 0.0
    ext = rng.normal(size=6 * 257) * 1e3
    for e in (ext, None):
        a, b = lib.structure_loads(w, e), oracle.structure_loads(w, e)
        assert np.array_equal(a, b) and np.array_equal(np.signbit(a), np.signbit(b))
    assert np.array_equal(lib.structure_loads(w)[2::6], -w + 0.0)


def test_pin_reference():
    nodes, _ = fx.lattice(6)
    for com in ((0.0, 0.0, 0.0), (1.3, 2.2, 0.7), (1e3, -4.0, 2.0)):
        a, b = nodes.copy(), nodes.copy()
        a["fixed"], b["fixed"] = 1, 1
        ia, ib = lib.pin_reference(a, com), oracle.pin_reference(b, com)
        assert ia == ib and np.array_equal(a, b)
        assert np.count_nonzero(a["fixed"]) == 1 and a["fixed"][ia] == 1
    # equal distances: the first node wins
    eq = with_centres(np.array([[1.0, 0.0, 0.0], [-1.0, 0.0, 0.0]]))
    assert lib.pin_reference(eq, (0.0, 0.0, 0.0)) == 0 and list(eq["fixed"]) == [1, 0]
    assert lib.pin_reference(np.zeros(0, NODE_DTYPE), (0.0, 0.0, 0.0)) == -1


@pytest.mark.parametrize("seed", [0, 1, 2])
@pytest.mark.parametrize("inertia", [True, False])
def test_body_loads(seed, inertia):
    rng = np.random.default_rng(100 + seed)
    s, nodes, ncom, nmass, ninert, forces = random_body(rng, 64, 9)
    a = lib.body_loads(s, nodes, forces, ncom, nmass, ninert, inertia=inertia)
    b = oracle.body_loads(s, nodes, forces, ncom, nmass, ninert, inertia=inertia)
    assert np.array_equal(a, b)
    r = oracle.body_loads(s, nodes, forces, ncom, nmass, ninert, inertia=inertia, reference=True)
    if r is not None:
        assert np.array_equal(a, r)
    # the loads balance: without point forces the relief of a free piece under gravity alone is
    # zero force (every node accelerates with g)
    if inertia:
        s.w[:] = [0.0, 0.0, 0.0]
        z = lib.body_loads(s, nodes, forces[:0], ncom, nmass, ninert)
        assert np.max(np.abs(z)) <= 1e-9 * np.max(nmass) * 9.81


def test_body_loads_arguments():
    rng = np.random.default_rng(7)
    s, nodes, ncom, nmass, ninert, forces = random_body(rng, 4, 3)
    L = lib.load_library()
    f = np.zeros(24)
    # inertia without the per-node mass properties is an argument error
    rc = L.svxg_body_loads(ctypes.byref(s), ptr(nodes), 4, None, None, None, ptr(forces), 3, 1, ptr(f))
    assert rc == -1
    # forces only: no mass properties needed
    rc = L.svxg_body_loads(ctypes.byref(s), ptr(nodes), 4, None, None, None, ptr(forces), 3, 0, ptr(f))
    assert rc == 0


def random_bonds_and_loads(rng, count):
    nodes, bonds = fx.lattice(4)
    b = np.resize(bonds, count).astype(BOND_DTYPE)
    b["ma"] = rng.integers(0, 4, count)
    b["mb"] = rng.integers(0, 4, count)
    b["strength"] = rng.uniform(0.5, 1.5, count)
    L = np.zeros(count, LOAD_DTYPE)
    for k in ("N", "V1", "V2", "T", "M1", "M2"):
        L[k] = rng.normal(size=count) * 10.0 ** rng.uniform(1, 6, count)
    L["N"][: count // 4] = np.abs(L["N"][: count // 4])   # tension
    L["N"][count // 4: count // 2] = -np.abs(L["N"][count // 4: count // 2])   # compression
    L[-4:] = np.zeros(4, LOAD_DTYPE)   # unloaded: no failure mode
    return b, L


def test_bond_utilization_matches_reference_and_oracle():
    rng = np.random.default_rng(11)
    b, L = random_bonds_and_loads(rng, 4000)
    ref = oracle.reference_lib()
    port = oracle.port_lib()
    modes = set()
    for k in range(len(b)):
        frag = float(rng.uniform(0.2, 3.0))
        phi, mode = lib.bond_utilization(b[k], L[k], frag, MATS)
        bk, lk = b[k:k + 1].copy(), L[k:k + 1].copy()
        mo = np.zeros(1, np.uint8)
        po = port.svxo_utilization(ptr(bk), ptr(lk), frag, ptr(MATS), ptr(mo))
        assert phi == po and mode == mo[0], k
        if ref is not None:
            mr = np.zeros(1, np.uint8)
            pr = ref.svxr_utilization(ptr(bk), ptr(lk), frag, ptr(MATS), ptr(mr))
            assert phi == pr and mode == mr[0], k
        modes.add(mode)
    assert modes == {0, 1, 2, 3}, modes  # (none, tension, crush, shear)


def test_bond_strength_and_bad_material():
    rng = np.random.default_rng(12)
    b, L = random_bonds_and_loads(rng, 8)
    Lb = lib.load_library()
    out = np.zeros(5)
    for frag in (0.5, 1.0, 2.0):
        assert Lb.svxg_bond_strength(ptr(b[:1]), frag, ptr(MATS), ptr(out)) == 0
        assert np.all(out[:3] > 0.0)
        # phi scales as 1 / strength: halving the fragility's multiplier doubles phi
        p1, _ = lib.bond_utilization(b[0], L[0], frag, MATS)
        p2, _ = lib.bond_utilization(b[0], L[0], 2.0 * frag, MATS)
        assert p2 == pytest.approx(2.0 * p1, rel=1e-12)
    bad = b[:1].copy()
    bad["ma"] = 255
    assert lib.bond_utilization(bad[0], L[0], 1.0, MATS) == (-1.0, 0)
    assert Lb.svxg_bond_strength(ptr(bad), 1.0, ptr(MATS), ptr(out)) == -1
