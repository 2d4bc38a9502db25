"""Per-phase device timing of the setup (svxg_phase_timing / svxg_phase_times): every phase
boundary of an assemble recorded as a CUDA event on the problem's stream - K, each level's
aggregation, lambda_max, prolongation, Galerkin products, the coarsest factor - the phases
non-negative, labelled, and summing to no more than the assemble's wall time; off, nothing is
recorded; the results the same with it on."""
import ctypes
import time

import numpy as np
import pytest

from opus_destruct_2_gb300 import StressProblem, load_library, synth
from opus_destruct_2_gb300.graph import PhaseTime, StressOptions

pytestmark = pytest.mark.gpu


def phases(L, h):
    cnt = ctypes.c_int32()
    out = (PhaseTime * 256)()
    assert L.svxg_phase_times(h, out, 256, ctypes.byref(cnt)) == 0
    return [(out[i].label.decode(), out[i].ms) for i in range(min(cnt.value, 256))]


def test_setup_phases_recorded():
    nodes, bonds, f, mats = synth.tower_graph(storeys=10, seed=1)
    L = load_library()
    L.svxg_phase_timing.argtypes = [ctypes.c_void_p, ctypes.c_int32]
    L.svxg_phase_times.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.POINTER(ctypes.c_int32)]
    G = StressProblem(nodes, bonds, mats)
    assert G.assemble(StressOptions())
    u0, _ = G.solve(f, rtol=1e-8, maxit=500)
    h = G._h
    assert L.svxg_phase_timing(h, 1) == 0
    t0 = time.perf_counter()
    assert G.assemble(StressOptions())
    wall_ms = 1e3 * (time.perf_counter() - t0)
    ph = phases(L, h)
    labels = [p[0] for p in ph]
    assert "K assembled" in labels and "coarsest factored" in labels and "coarsen: coarse values" in labels
    assert labels.count("level coarsened") == G.info().levels - 1
    assert all(ms >= 0.0 for _, ms in ph)
    assert 0.0 < sum(ms for _, ms in ph) <= wall_ms * 1.05 + 0.5
    u1, _ = G.solve(f, rtol=1e-8, maxit=500)
    assert np.array_equal(u0, u1)
    assert L.svxg_phase_timing(h, 0) == 0
    assert G.assemble(StressOptions())
    assert phases(L, h) == []


def test_galerkin_kernel_timer():
    """svxg_timer_enable_kernel(SVXG_TIMER_GALERKIN_AP): one timed launch per coarsening with its
    block products counted (the build-work count of A P / 6); the solve's SpMV is not timed
    meanwhile and the results are unchanged."""
    nodes, bonds, f, mats = synth.tower_graph(storeys=10, seed=1)
    L = load_library()
    L.svxg_timer_enable_kernel.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32]
    L.svxg_timer_read_work.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double),
                                       ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64)]
    G = StressProblem(nodes, bonds, mats)
    assert G.assemble(StressOptions())
    u0, _ = G.solve(f, rtol=1e-8, maxit=500)
    assert L.svxg_timer_enable_kernel(G._h, 1, 1) == 0
    assert G.assemble(StressOptions())
    u1, _ = G.solve(f, rtol=1e-8, maxit=500)
    ms, n, work = ctypes.c_double(), ctypes.c_int64(), ctypes.c_int64()
    assert L.svxg_timer_read_work(G._h, ctypes.byref(ms), ctypes.byref(n), ctypes.byref(work)) == 0
    assert n.value == G.info().levels - 1 and work.value > 0 and ms.value > 0.0
    assert np.array_equal(u0, u1)
    assert L.svxg_timer_enable_kernel(G._h, 7, 1) == -1
    assert L.svxg_timer_enable_kernel(G._h, 1, 0) == 0
