"""svxg_utilization_noalloc - the judge for hosts that cannot let the library allocate device
memory - against the problem's own judge (svxg_utilization_device) through the C ABI.

Bar: bit-exact phi, mode and failure list (the judge's bar), on two calls in a row of different
sizes (the second smaller, so anything left in the shared scratch by the first would show), with
no change in the device's free memory across a call. Collected last: it must pass in a fresh
process and after every other test.
"""
import ctypes

import numpy as np
import pytest

import fixtures as fx
from opus_destruct_2_gb300 import StressProblem, load_library
from opus_destruct_2_gb300.graph import StressOptions, default_materials

pytestmark = pytest.mark.gpu

MATS = default_materials()
MAX_BONDS = 16_777_216
c_vp, c_i32 = ctypes.c_void_p, ctypes.c_int32


def noalloc_fn():
    L = load_library()
    f = L.svxg_utilization_noalloc
    f.restype = c_i32
    f.argtypes = [c_vp, c_i32, c_vp, c_i32, c_vp, c_vp, ctypes.c_double, c_vp, c_vp, c_vp, ctypes.POINTER(c_i32),
                  c_vp]
    return f


def solved(nodes, bonds):
    G = StressProblem(nodes, bonds, MATS)
    assert G.assemble(StressOptions(amg_min_nodes=1 << 30))
    res = G.solve(fx.gravity_live(nodes), rtol=1e-10, maxit=20000)[1]
    assert res.converged
    return G


def existing_judge(G, fragility):
    import torch
    nb = len(G.bonds)
    phi = torch.zeros(nb, dtype=torch.float64, device="cuda")
    mode = torch.zeros(nb, dtype=torch.uint8, device="cuda")
    over = torch.zeros(max(nb, 1), dtype=torch.int32, device="cuda")
    n = c_i32(0)
    assert load_library().svxg_utilization_device(G._h, float(fragility), phi.data_ptr(), mode.data_ptr(),
                                                  over.data_ptr(), ctypes.byref(n)) == 0
    torch.cuda.synchronize()
    return phi.cpu().numpy(), mode.cpu().numpy(), over[:n.value].cpu().numpy()


class CallerBuffers:
    """Everything the entry point reads and writes, allocated by the caller (here: torch)."""

    def __init__(self, nodes, bonds, u):
        import torch
        dev = lambda a: torch.from_numpy(np.ascontiguousarray(a).view(np.uint8).copy()).cuda()
        self.nodes, self.bonds, self.mats = dev(nodes), dev(bonds), dev(MATS)
        self.u = torch.from_numpy(np.ascontiguousarray(u, dtype=np.float64)).cuda()
        self.n, self.nb = len(nodes), len(bonds)
        self.phi = torch.full((self.nb,), -1.0, dtype=torch.float64, device="cuda")
        self.mode = torch.full((self.nb,), 255, dtype=torch.uint8, device="cuda")
        self.over = torch.full((max(self.nb, 1),), -1, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()

    def call(self, fragility):
        import torch
        n_over = c_i32(-1)
        e = noalloc_fn()(self.nodes.data_ptr(), self.n, self.bonds.data_ptr(), self.nb, self.mats.data_ptr(),
                         self.u.data_ptr(), float(fragility), self.phi.data_ptr(), self.mode.data_ptr(),
                         self.over.data_ptr(), ctypes.byref(n_over), torch.cuda.current_stream().cuda_stream)
        assert e == 0, load_library().svxg_last_error()
        return self.phi.cpu().numpy(), self.mode.cpu().numpy(), self.over[:n_over.value].cpu().numpy()


def test_noalloc_matches_existing_judge_on_two_calls_in_a_row():
    import torch
    cases = [(fx.lattice(12), 400.0),                   # 4896 bonds in 20 blocks, 1440 failing
             (fx.cantilever(12, 0.5, 300.0), 1.0)]     # 12 bonds in one block, 7 failing
    prepared = []
    for (nodes, bonds), frag in cases:
        G = solved(nodes, bonds)
        prepared.append((CallerBuffers(nodes, bonds, G.current()), existing_judge(G, frag), frag))
    # (a first call on this device, whose one-time set-up and kernel loading may take memory, unless
    # an earlier test made it already)
    prepared[1][0].call(prepared[1][2])
    for buf, (phi0, mode0, over0), frag in prepared:
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        phi, mode, over = buf.call(frag)
        torch.cuda.synchronize()
        assert torch.cuda.mem_get_info()[0] == free0
        assert 0 < len(over0) < len(phi0)
        assert np.array_equal(phi, phi0) and np.array_equal(mode, mode0)
        assert np.array_equal(over, over0)
        assert np.array_equal(over, np.nonzero(phi0 >= 1.0)[0])


def test_noalloc_matches_existing_judge_above_a_thousand_blocks():
    """More than 262,144 bonds: the scan of the per-block counts then gives each of its threads
    several blocks. Any displacement will do for the judge's arithmetic: a seeded random one, at a
    fragility that puts about half the bonds over strength."""
    import torch
    nodes, bonds = fx.lattice(45)
    assert len(bonds) > 262_144
    G = StressProblem(nodes, bonds, MATS)
    assert G.assemble(StressOptions(amg_min_nodes=1 << 30))
    rng = np.random.default_rng(17)
    u = 1e-4 * rng.standard_normal(6 * len(nodes))
    u[np.repeat(nodes["fixed"] != 0, 6)] = 0.0
    G.begin(fx.gravity_live(nodes), u)
    G.iterate(0, 1e-30)
    phi1, _, _ = existing_judge(G, 1.0)
    frag = 1.0 / float(np.median(phi1[phi1 > 0]))
    phi0, mode0, over0 = existing_judge(G, frag)
    assert 0.3 * len(bonds) < len(over0) < 0.7 * len(bonds)
    buf = CallerBuffers(nodes, bonds, G.current())
    for _ in range(2):
        phi, mode, over = buf.call(frag)
        torch.cuda.synchronize()
        assert np.array_equal(phi, phi0) and np.array_equal(mode, mode0)
        assert np.array_equal(over, over0)


def test_noalloc_rejects_sizes_beyond_its_maximum():
    f = noalloc_fn()
    n_over = c_i32(-1)
    assert f(None, 1, None, MAX_BONDS + 1, None, None, 1.0, None, None, None, ctypes.byref(n_over), None) == -1
    assert b"maximum" in load_library().svxg_last_error()
    assert n_over.value == -1


def test_noalloc_reports_out_of_range_bonds():
    nodes, bonds = fx.lattice(4)
    bad = bonds.copy()
    bad["b"][3] = len(nodes)          # a node index past the end
    bad["ma"][5] = 200                # a material id past the table
    bad["a"][7] = -1                  # a node index below the start
    buf = CallerBuffers(nodes, bad, np.zeros(6 * len(nodes)))
    n_over = c_i32(-1)
    import torch
    e = noalloc_fn()(buf.nodes.data_ptr(), buf.n, buf.bonds.data_ptr(), buf.nb, buf.mats.data_ptr(), buf.u.data_ptr(),
                     1.0, buf.phi.data_ptr(), buf.mode.data_ptr(), buf.over.data_ptr(), ctypes.byref(n_over),
                     torch.cuda.current_stream().cuda_stream)
    assert e == -1 and b"out of range" in load_library().svxg_last_error()
    # the valid bonds are still judged (u = 0: phi = 0)
    phi = buf.phi.cpu().numpy()
    assert phi[3] == -1.0 and phi[5] == -1.0 and phi[7] == -1.0 and np.all(phi[[0, 1, 2, 4, 6]] == 0.0)
