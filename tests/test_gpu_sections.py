"""Bonds from voxel-face interfaces on the device (svxg_build_bonds, through the C ABI) against
the oracle's restatement of SecAcc::finish (finish_lattice / finish_general) + section_strengths
(_general) (core/src/world/world_internal.hpp:130-441), itself pinned bit for bit to the
reference's own header code (test_oracle_pin.py, golden/sections/). Bar: bit for bit, every field
of every bond (integer and floating point: the same operations in the same order, no
contraction)."""
import ctypes

import numpy as np
import pytest

import fixtures as fx
import oracle
import section_cases as sc
from opus_destruct_2_gb300 import SvxgError, StressProblem, build_bonds, load_library, synth
from opus_destruct_2_gb300.graph import StressOptions, ptr

pytestmark = pytest.mark.gpu
CASES = sc.cases()


@pytest.mark.parametrize("name", list(CASES), ids=list(CASES))
def test_build_bonds_bit_exact(name):
    nodes, secs, faces, mats = CASES[name]
    got = build_bonds(nodes, secs, faces, mats)
    want = oracle.build_bonds(nodes, secs, faces, mats)
    assert fx.same_records(got, want)


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_build_bonds_general_bit_exact(seed):
    """Placed lattices and junction samples between lattices (finish_general,
    section_strengths_general), mixed with lattice sections: bit for bit the oracle's."""
    nodes, secs, faces, js, lats, mats = sc.general(seed)
    got = build_bonds(nodes, secs, faces, mats, junctions=js, lattices=lats)
    want = oracle.build_bonds(nodes, secs, faces, mats, junctions=js, lattices=lats)
    assert fx.same_records(got, want)


def test_build_bonds_rejects_out_of_range():
    nodes, secs, faces, mats = sc.handmade(seed=3, count=20)
    bad = secs.copy()
    bad[5]["first_face"] = len(faces) - 1
    bad[5]["faces"] = 5
    with pytest.raises(SvxgError):
        build_bonds(nodes, bad, faces, mats)
    bad = secs.copy()
    bad[2]["a"] = len(nodes)
    with pytest.raises(SvxgError):
        build_bonds(nodes, bad, faces, mats)


def test_build_bonds_device_counts_bad_sections():
    """The device entry point checks every section on the device: a bad one becomes a broken,
    empty bond and is counted; the others are built as usual."""
    import torch
    nodes, secs, faces, mats = sc.handmade(seed=4, count=30)
    secs = secs.copy()
    secs[7]["b"] = len(nodes) + 3
    dev = torch.device("cuda", 0)
    t = {k: torch.from_numpy(np.frombuffer(v.tobytes(), np.uint8).copy()).to(dev)
         for k, v in dict(nodes=nodes, secs=secs, faces=faces, mats=mats).items()}
    out = torch.zeros(len(secs) * 216, dtype=torch.uint8, device=dev)
    nbad = torch.zeros(1, dtype=torch.int32, device=dev)
    L = load_library()
    rc = L.svxg_build_bonds_device(ctypes.c_void_p(t["nodes"].data_ptr()), len(nodes),
                                   ctypes.c_void_p(t["secs"].data_ptr()), len(secs),
                                   ctypes.c_void_p(t["faces"].data_ptr()), len(faces), None, 0, None, 0, 2,
                                   ctypes.c_void_p(t["mats"].data_ptr()), ctypes.c_void_p(out.data_ptr()),
                                   ctypes.c_void_p(nbad.data_ptr()), None)
    assert rc == 0
    torch.cuda.synchronize()
    assert int(nbad.item()) == 1
    got = np.frombuffer(out.cpu().numpy().tobytes(), dtype=oracle.BOND_DTYPE)
    assert got[7]["broken"] == 1 and got[7]["faces"] == 0
    keep = np.ones(len(secs), bool)
    keep[7] = False
    good = secs.copy()
    good[7]["b"] = -1
    want = oracle.build_bonds(nodes, good, faces, mats)
    assert fx.same_records(got[keep], want[keep])


def test_solve_on_built_bonds():
    """A tower whose bonds the device built from its voxel faces: assembled and solved on the GPU,
    the same u as the oracle's solve of the same bonds."""
    nodes, _, f, mats = synth.tower_graph(4, seed=5)
    secs, faces = synth.last_sections()
    bonds = build_bonds(nodes, secs, faces, mats)
    G = StressProblem(nodes, bonds, mats)
    assert G.assemble(StressOptions())
    u, r = G.solve(f, rtol=1e-10, maxit=2000)
    O = oracle.Port(nodes, bonds, mats)
    assert O.assemble(StressOptions())
    uo, ro = O.solve(f, rtol=1e-12, maxit=5000)
    assert r.converged
    assert float(np.max(np.abs(u - uo)) / np.max(np.abs(uo))) <= 1e-6
