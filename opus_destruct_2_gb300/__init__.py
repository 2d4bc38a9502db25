"""GB300-native stress solve of fragment graphs (the svx_core StressProblem path on sm_103a).

``StressProblem`` mirrors the reference's ``svx::StressProblem`` (core/include/svx/stress/stress.hpp:
74-160) over the C ABI of ``include/svxg.h``: the same members (nodes, bonds, mats), the same
calls (assemble, solve, begin/iterate/current, bond_load, remove_bond, retire_nodes, release ...)
and the same results and error behaviour (assemble -> False on a singular diagonal; a solve of
non-finite loads -> breakdown with rel_res = inf; zero load -> converged, u = 0). Every number is
computed by the CUDA library; there is no CPU path: if the library cannot be loaded, or no GPU
is present, the calls raise.
"""
from __future__ import annotations

import ctypes
import os
import sys

import numpy as np

from . import build as _build
from .graph import (BOND_DTYPE, LOAD_DTYPE, MATERIAL_DTYPE, NODE_DTYPE, CascadeOptions, CascadeResult, PcgResult,
                    PieceOptions, PieceResult, StressOptions, default_materials, ptr)

__all__ = ["Batch", "StressProblem", "StressOptions", "PcgResult", "Info", "load_library", "default_materials",
           "NODE_DTYPE", "BOND_DTYPE", "SvxgError", "CascadeOptions", "CascadeResult", "build_bonds",
           "PieceOptions", "PieceResult"]

c_i32, c_i64, c_f64, c_vp = ctypes.c_int32, ctypes.c_int64, ctypes.c_double, ctypes.c_void_p

ERRORS = {-1: "bad argument", -2: "CUDA error", -3: "out of device memory", -4: "wrong state", -5: "timeout",
          -6: "no CUDA device"}


class SvxgError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"svxg error {code} ({ERRORS.get(code, '?')}): {msg}")
        self.code = code


class Info(ctypes.Structure):
    _fields_ = [("nfree", c_i32), ("levels", c_i32), ("block_jacobi", c_i32), ("chol_n", c_i32),
                ("level_sizes", c_i32 * 16), ("level_blocks", c_i64 * 32), ("matrix_blocks", c_i64),
                ("work_per_iteration", c_i64), ("assembly_work", c_i64), ("work_per_apply", c_i64),
                ("build_work", c_i64), ("device_bytes", c_i64), ("precision", c_i32), ("mixed_fallbacks", c_i32),
                ("graph_bytes", c_i64), ("error_estimate", c_f64)]

    def sizes(self) -> list[int]:
        return [self.level_sizes[i] for i in range(self.levels)]

    def blocks(self) -> list[int]:
        return [self.level_blocks[i] for i in range(2 * self.levels)]


_lib: ctypes.CDLL | None = None


def library_path() -> str:
    return os.path.join(_build.LIBDIR, _build.CUDA_LIB)


def load_library() -> ctypes.CDLL:
    """The CUDA library (built in-tree by __graft_entry__.build()); raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not os.path.exists(path):
        raise RuntimeError(f"the CUDA library is not built ({path}); run __graft_entry__.build()")
    L = ctypes.CDLL(path)
    sig = {
        "svxg_last_error": (ctypes.c_char_p, []),
        "svxg_device_count": (c_i32, []),
        "svxg_problem_create": (c_i32, [ctypes.POINTER(c_vp), c_i32]),
        "svxg_problem_destroy": (None, [c_vp]),
        "svxg_problem_stream": (c_vp, [c_vp]),
        "svxg_set_graph": (c_i32, [c_vp, c_vp, c_i32, c_vp, c_i32, c_vp]),
        "svxg_set_graph_device": (c_i32, [c_vp, c_vp, c_i32, c_vp, c_i32, c_vp]),
        "svxg_set_graphs": (c_i32, [c_vp, c_i32, c_vp, c_vp, c_vp, c_vp, c_vp]),
        "svxg_set_graphs_device": (c_i32, [c_vp, c_i32, c_vp, c_vp, c_vp, c_vp, c_vp]),
        "svxg_graph_results": (c_i32, [c_vp, c_i32, c_vp, c_vp, c_vp, c_vp]),
        "svxg_time_spmv": (c_i32, [c_vp, c_i32, c_i32, ctypes.POINTER(c_f64)]),
        "svxg_structure_loads": (c_i32, [c_i32, c_vp, c_vp, c_vp]),
        "svxg_body_loads": (c_i32, [c_vp, c_vp, c_i32, c_vp, c_vp, c_vp, c_vp, c_i32, c_i32, c_vp]),
        "svxg_bond_strength": (c_i32, [c_vp, c_f64, c_vp, c_vp]),
        "svxg_bond_utilization": (c_f64, [c_vp, c_vp, c_f64, c_vp, c_vp]),
        "svxg_measure_fp64_rate": (c_i32, [c_i32, ctypes.POINTER(c_f64)]),
        "svxg_assemble": (c_i32, [c_vp, c_vp, ctypes.POINTER(c_i32)]),
        "svxg_assembled": (c_i32, [c_vp]),
        "svxg_reassemble": (c_i32, [c_vp, c_vp, c_i32, c_vp, c_i32, c_vp, ctypes.POINTER(c_i32)]),
        "svxg_appended": (c_i32, [c_vp]),
        "svxg_extend_warm_start": (c_i32, [c_vp, c_vp, c_i32]),
        "svxg_invalidate": (c_i32, [c_vp]),
        "svxg_preconditioner_current": (c_i32, [c_vp]),
        "svxg_block_jacobi": (c_i32, [c_vp]),
        "svxg_release": (c_i32, [c_vp]),
        "svxg_remove_bond": (c_i32, [c_vp, c_i32]),
        "svxg_retire_nodes": (c_i32, [c_vp, c_vp, c_i32]),
        "svxg_remove_bonds": (c_i32, [c_vp, c_vp, c_i32]),
        "svxg_bond_flags": (c_i32, [c_vp, c_vp, c_vp]),
        "svxg_solve": (c_i32, [c_vp, c_vp, c_vp, c_f64, c_i32, c_i32, c_vp]),
        "svxg_solve_device": (c_i32, [c_vp, c_vp, c_vp, c_f64, c_i32, c_i32, c_vp]),
        "svxg_begin": (c_i32, [c_vp, c_vp, c_vp]),
        "svxg_iterate": (c_i32, [c_vp, c_i32, c_f64, c_vp]),
        "svxg_running": (c_i32, [c_vp]),
        "svxg_stop": (c_i32, [c_vp]),
        "svxg_current": (c_i32, [c_vp, c_vp]),
        "svxg_bond_loads": (c_i32, [c_vp, c_vp, c_vp]),
        "svxg_utilization": (c_i32, [c_vp, c_f64, c_vp, c_vp, c_vp, c_i32, ctypes.POINTER(c_i32)]),
        "svxg_get_info": (c_i32, [c_vp, c_vp]),
        "svxg_debug_matrix": (c_i32, [c_vp, ctypes.POINTER(c_i32), ctypes.POINTER(c_i64), c_vp, c_vp, c_vp, c_vp,
                                      ctypes.POINTER(c_f64)]),
        "svxg_debug_level_dims": (c_i32, [c_vp, c_i32, ctypes.POINTER(c_i32), ctypes.POINTER(c_i64),
                                          ctypes.POINTER(c_i64)]),
        "svxg_debug_level": (c_i32, [c_vp, c_i32] + [c_vp] * 9 + [ctypes.POINTER(c_f64)]),
        "svxg_debug_precondition": (c_i32, [c_vp, c_vp, c_vp]),
        "svxg_debug_apply": (c_i32, [c_vp, c_vp, c_vp]),
        "svxg_debug_seq_norm": (c_i32, [c_vp, c_i64, ctypes.POINTER(c_f64)]),
        "svxg_launch_count": (c_i64, []),
        "svxg_graph_launch_count": (c_i64, []),
        "svxg_utilization_device": (c_i32, [c_vp, c_f64, c_vp, c_vp, c_vp, ctypes.POINTER(c_i32)]),
        "svxg_timer_enable": (c_i32, [c_vp, c_i32]),
        "svxg_timer_read": (c_i32, [c_vp, ctypes.POINTER(c_f64), ctypes.POINTER(c_i64)]),
        "svxg_cascade": (c_i32, [c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_i32, c_vp, c_i32, c_vp]),
        "svxg_build_bonds": (c_i32, [c_vp, c_i32, c_vp, c_i32, c_vp, c_i64, c_vp, c_i64, c_vp, c_i32, c_i32, c_vp,
                                     c_vp]),
        "svxg_piece_rounds": (c_i32, [c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_i32, c_vp, c_i32, c_vp]),
        "svxg_build_bonds_device": (c_i32, [c_vp, c_i32, c_vp, c_i32, c_vp, c_i64, c_vp, c_i64, c_vp, c_i32, c_i32,
                                            c_vp, c_vp, c_vp, c_vp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def _check(code: int) -> int:
    if code < 0:
        msg = load_library().svxg_last_error()
        raise SvxgError(code, msg.decode() if msg else "")
    return code


def build_bonds(nodes, secs, faces, mats=None, junctions=None, lattices=None, samples: int = 2) -> np.ndarray:
    """The bonds of voxel-face interfaces on the GPU (SecAcc::finish + section_strengths(_general),
    core/src/world/world_internal.hpp:130-441): bond k from secs[k] (SECTION_DTYPE), its faces
    (FACE_DTYPE) and junction samples (JUNCTION_DTYPE), with the lattices (LATTICE_DTYPE) of the
    faces and samples. Returns BOND_DTYPE records."""
    from .graph import FACE_DTYPE, JUNCTION_DTYPE, LATTICE_DTYPE, SECTION_DTYPE
    L = load_library()
    nodes = np.ascontiguousarray(nodes, dtype=NODE_DTYPE)
    secs = np.ascontiguousarray(secs, dtype=SECTION_DTYPE)
    faces = np.ascontiguousarray(faces, dtype=FACE_DTYPE)
    mats = np.ascontiguousarray(default_materials() if mats is None else mats, dtype=MATERIAL_DTYPE)
    js = None if junctions is None else np.ascontiguousarray(junctions, dtype=JUNCTION_DTYPE)
    ls = None if lattices is None else np.ascontiguousarray(lattices, dtype=LATTICE_DTYPE)
    out = np.zeros(len(secs), BOND_DTYPE)
    _check(L.svxg_build_bonds(ptr(nodes), len(nodes), ptr(secs), len(secs), ptr(faces), len(faces), ptr(js),
                              0 if js is None else len(js), ptr(ls), 0 if ls is None else len(ls), int(samples),
                              ptr(mats), ptr(out)))
    return out


class StressProblem:
    """svx::StressProblem on the GPU. ``nodes``/``bonds`` are numpy records (graph.NODE_DTYPE /
    BOND_DTYPE), ``mats`` a material table; assign them, then call assemble() (the graph is sent
    to the device at assemble time, or whenever it changed)."""

    def __init__(self, nodes=None, bonds=None, mats=None, device: int = 0):
        L = load_library()
        if L.svxg_device_count() <= device:
            raise SvxgError(-6, "no CUDA device")
        h = c_vp()
        _check(L.svxg_problem_create(ctypes.byref(h), device))
        self._h = h
        self._L = L
        self.nodes = np.zeros(0, NODE_DTYPE) if nodes is None else np.array(nodes, dtype=NODE_DTYPE)
        self.bonds = np.zeros(0, BOND_DTYPE) if bonds is None else np.array(bonds, dtype=BOND_DTYPE)
        self.mats = default_materials() if mats is None else np.array(mats, dtype=MATERIAL_DTYPE)
        if len(self.mats) != 127:
            raise ValueError("mats: 127 resolved material records")
        self._sent = None

    def __del__(self):
        h = getattr(self, "_h", None)
        if sys.is_finalizing():  # (the CUDA runtime may be gone already; the process frees all)
            return
        if h is not None and h.value:
            self._L.svxg_problem_destroy(h)
            self._h = None

    # -- the graph -------------------------------------------------------------------------
    def _sync_graph(self):
        key = (self.nodes.__array_interface__["data"][0], self.nodes.tobytes(), self.bonds.tobytes(),
               self.mats.tobytes())
        if self._sent == key:
            return
        self.nodes = np.ascontiguousarray(self.nodes, dtype=NODE_DTYPE)
        self.bonds = np.ascontiguousarray(self.bonds, dtype=BOND_DTYPE)
        _check(self._L.svxg_set_graph(self._h, ptr(self.nodes), len(self.nodes), ptr(self.bonds), len(self.bonds),
                                      ptr(self.mats)))
        self._sent = key

    def _pull_flags(self):
        br = np.zeros(len(self.bonds), np.uint8)
        ik = np.zeros(len(self.bonds), np.uint8)
        _check(self._L.svxg_bond_flags(self._h, ptr(br), ptr(ik)))
        self.bonds["broken"] = br
        self.bonds["in_k"] = ik
        self._sent = (self.nodes.__array_interface__["data"][0], self.nodes.tobytes(), self.bonds.tobytes(),
                      self.mats.tobytes())

    # -- StressProblem's calls -------------------------------------------------------------------
    def assemble(self, opt: StressOptions | None = None) -> bool:
        self._sync_graph()
        ok = c_i32(0)
        _check(self._L.svxg_assemble(self._h, ctypes.byref(opt) if opt is not None else None, ctypes.byref(ok)))
        self._pull_flags()
        return bool(ok.value)

    def reassemble(self) -> bool:
        """StressProblem::reassemble (stress.cpp:178-211): K again from the current nodes and bonds;
        nodes appended since the last assemble() get their own preconditioner (their multigrid,
        or their diagonal blocks), the old one keeps the rest."""
        self.nodes = np.ascontiguousarray(self.nodes, dtype=NODE_DTYPE)
        self.bonds = np.ascontiguousarray(self.bonds, dtype=BOND_DTYPE)
        ok = c_i32(0)
        _check(self._L.svxg_reassemble(self._h, ptr(self.nodes), len(self.nodes), ptr(self.bonds), len(self.bonds),
                                       ptr(self.mats), ctypes.byref(ok)))
        self._pull_flags()
        return bool(ok.value)

    def appended(self) -> int:
        """Free nodes the last assemble()'s multigrid does not cover (StressProblem::appended)."""
        return int(self._L.svxg_appended(self._h))

    def extend_warm_start(self, u, first_new: int):
        """StressProblem::extend_warm_start (stress.cpp:213-244): u (6 per node) with the nodes from
        first_new on set from their bonded, older neighbours' motion; returns the new array."""
        self._sync_graph()
        out = np.array(u, dtype=np.float64)
        if out.size != 6 * len(self.nodes):
            raise ValueError("u: 6 per node")
        _check(self._L.svxg_extend_warm_start(self._h, ptr(out), int(first_new)))
        return out

    def assembled(self) -> bool:
        return bool(self._L.svxg_assembled(self._h))

    def invalidate(self):
        _check(self._L.svxg_invalidate(self._h))

    def preconditioner_current(self) -> bool:
        return bool(self._L.svxg_preconditioner_current(self._h))

    def block_jacobi(self) -> bool:
        return bool(self._L.svxg_block_jacobi(self._h))

    def release(self):
        _check(self._L.svxg_release(self._h))
        self.bonds["in_k"] = 0

    def remove_bond(self, b: int):
        _check(self._L.svxg_remove_bond(self._h, int(b)))
        self._pull_flags()

    def remove_bonds(self, lst):
        """remove_bond of each listed bond in order, in one device pass."""
        a = np.ascontiguousarray(lst, dtype=np.int32)
        _check(self._L.svxg_remove_bonds(self._h, ptr(a), len(a)))
        self._pull_flags()

    def retire_nodes(self, lst):
        a = np.ascontiguousarray(lst, dtype=np.int32)
        _check(self._L.svxg_retire_nodes(self._h, ptr(a), len(a)))
        self.nodes["gone"][a] = 1
        self._pull_flags()

    def solve(self, f, u=None, rtol: float = 2e-3, maxit: int = -1, warm: bool = False):
        """Returns (u, PcgResult); u: 6 per node."""
        self._sync_graph()
        f = np.ascontiguousarray(f, dtype=np.float64)
        if f.size != 6 * len(self.nodes):
            raise ValueError("f: 6 per node")
        u = np.zeros(6 * len(self.nodes)) if u is None else np.array(u, dtype=np.float64)
        res = PcgResult()
        _check(self._L.svxg_solve(self._h, ptr(f), ptr(u), float(rtol), int(maxit), int(bool(warm)),
                                  ctypes.byref(res)))
        self._pull_flags()
        return u, res

    def begin(self, f, u0=None):
        self._sync_graph()
        f = np.ascontiguousarray(f, dtype=np.float64)
        u0 = None if u0 is None else np.ascontiguousarray(u0, dtype=np.float64)
        _check(self._L.svxg_begin(self._h, ptr(f), ptr(u0)))

    def iterate(self, maxit: int, rtol: float) -> PcgResult:
        res = PcgResult()
        _check(self._L.svxg_iterate(self._h, int(maxit), float(rtol), ctypes.byref(res)))
        return res

    def running(self) -> bool:
        return bool(self._L.svxg_running(self._h))

    def stop(self):
        _check(self._L.svxg_stop(self._h))

    def current(self):
        u = np.zeros(6 * len(self.nodes))
        _check(self._L.svxg_current(self._h, ptr(u)))
        return u

    def bond_loads(self, u=None) -> np.ndarray:
        out = np.zeros(len(self.bonds), LOAD_DTYPE)
        u = None if u is None else np.ascontiguousarray(u, dtype=np.float64)
        _check(self._L.svxg_bond_loads(self._h, ptr(u), ptr(out)))
        return out

    def bond_load(self, b: int, u) -> np.ndarray:
        return self.bond_loads(u)[b]

    def cascade(self, f, u=None, options: CascadeOptions | None = None, opt: StressOptions | None = None,
                judged=None, has=None):
        """The judge's break rounds of this structure (World::Impl::judge,
        core/src/world/world.cpp:1162-1277, with the tick's solve restarts and
        detach_unsupported): solve, judge, break the round's worst bonds, retire what no support
        holds, again until nothing is over strength. Returns (u, CascadeResult, extras) with
        extras = dict(broken=[bonds in the order broken], retired=[nodes in the order retired],
        phi=last utilizations, judged=LOAD_DTYPE records, has=uint8 flags). The problem's bonds and
        nodes are left broken and retired (self.bonds / self.nodes follow)."""
        self._sync_graph()
        n, nb = len(self.nodes), len(self.bonds)
        f = np.ascontiguousarray(f, dtype=np.float64)
        if f.size != 6 * n:
            raise ValueError("f: 6 per node")
        u = np.zeros(6 * n) if u is None else np.array(u, dtype=np.float64)
        judged = np.zeros(nb, LOAD_DTYPE) if judged is None else np.array(judged, dtype=LOAD_DTYPE)
        has = np.zeros(nb, np.uint8) if has is None else np.array(has, dtype=np.uint8)
        phi = np.zeros(max(nb, 1))
        broken = np.zeros(max(nb, 1), np.int32)
        retired = np.zeros(max(n, 1), np.int32)
        res = CascadeResult()
        o = CascadeOptions() if options is None else options
        _check(self._L.svxg_cascade(self._h, ctypes.byref(opt) if opt is not None else None, ctypes.byref(o),
                                    ptr(f), ptr(u), ptr(judged), ptr(has), ptr(phi), ptr(broken), len(broken),
                                    ptr(retired), len(retired), ctypes.byref(res)))
        rl = retired[:min(res.nodes_retired, len(retired))].copy()
        self.nodes["gone"][rl] = 1
        self._pull_flags()
        extras = dict(broken=broken[:min(res.bonds_broken, len(broken))].tolist(), retired=rl.tolist(),
                      phi=phi[:nb].copy(), judged=judged, has=has)
        return u, res, extras

    def piece_rounds(self, f, u=None, options: PieceOptions | None = None, gf=None, opt: StressOptions | None = None):
        """A loose piece's break rounds within one substep (World::Impl::body_stress_run,
        core/src/world/world_pieces.cpp:614-808). f: the piece's load (inertial relief and point
        forces). Returns (u, f with the chips' loads moved, PieceResult, extras) with extras =
        dict(broken=[bonds in the order broken], modes=[their failure modes], chips=[chip nodes
        retired]); the problem's bonds and nodes are left broken and retired."""
        from .graph import default_fracture_energies
        self._sync_graph()
        n, nb = len(self.nodes), len(self.bonds)
        f = np.array(f, dtype=np.float64)
        if f.size != 6 * n:
            raise ValueError("f: 6 per node")
        u = np.zeros(6 * n) if u is None else np.array(u, dtype=np.float64)
        gf = np.ascontiguousarray(default_fracture_energies() if gf is None else gf, dtype=np.float64)
        broken = np.zeros(max(nb, 1), np.int32)
        modes = np.zeros(max(nb, 1), np.uint8)
        chips = np.zeros(max(n, 1), np.int32)
        res = PieceResult()
        o = PieceOptions() if options is None else options
        _check(self._L.svxg_piece_rounds(self._h, ctypes.byref(opt) if opt is not None else None, ctypes.byref(o),
                                         ptr(gf), ptr(f), ptr(u), ptr(broken), ptr(modes), len(broken), ptr(chips),
                                         len(chips), ctypes.byref(res)))
        cl = chips[:min(res.chips, len(chips))].copy()
        self.nodes["gone"][cl] = 1
        self._pull_flags()
        k = min(res.bonds_broken, len(broken))
        return u, f, res, dict(broken=broken[:k].tolist(), modes=modes[:k].tolist(), chips=cl.tolist())

    def utilization(self, fragility: float = 1.0):
        """(phi, mode, failing bond indices) at the current solution."""
        nb = len(self.bonds)
        phi = np.zeros(nb)
        mode = np.zeros(nb, np.uint8)
        over = np.zeros(max(nb, 1), np.int32)
        n_over = c_i32(0)
        _check(self._L.svxg_utilization(self._h, float(fragility), ptr(phi), ptr(mode), ptr(over), len(over),
                                        ctypes.byref(n_over)))
        return phi, mode, over[:n_over.value].copy()

    def info(self) -> Info:
        i = Info()
        _check(self._L.svxg_get_info(self._h, ctypes.byref(i)))
        return i

    def matrix_blocks(self) -> int:
        return int(self.info().matrix_blocks)

    def free_nodes(self) -> int:
        return int(self.info().nfree)

    def work_per_iteration(self) -> int:
        return int(self.info().work_per_iteration)

    def assembly_work(self) -> int:
        return int(self.info().assembly_work)

    def memory_bytes(self) -> int:
        return int(self.info().device_bytes)

    def stream(self) -> int:
        return int(self._L.svxg_problem_stream(self._h) or 0)

    def solve_device(self, f_ptr: int, u_ptr: int, rtol: float, maxit: int = -1, warm: bool = False) -> PcgResult:
        res = PcgResult()
        _check(self._L.svxg_solve_device(self._h, c_vp(f_ptr), c_vp(u_ptr), float(rtol), int(maxit),
                                         int(bool(warm)), ctypes.byref(res)))
        return res

    # -- parity access -----------------------------------------------------------------------------
    def debug_matrix(self) -> dict:
        nf, nz, ids = c_i32(), c_i64(), c_f64()
        _check(self._L.svxg_debug_matrix(self._h, ctypes.byref(nf), ctypes.byref(nz), None, None, None, None,
                                         ctypes.byref(ids)))
        dof = np.zeros(len(self.nodes), np.int32)
        rowptr = np.zeros(nf.value + 1, np.int32)
        col = np.zeros(nz.value, np.int32)
        val = np.zeros((nz.value, 6, 6))
        _check(self._L.svxg_debug_matrix(self._h, ctypes.byref(nf), ctypes.byref(nz), ptr(dof), ptr(rowptr),
                                         ptr(col), ptr(val), ctypes.byref(ids)))
        return dict(nfree=nf.value, dof=dof, rowptr=rowptr, col=col, val=val, id_scale=ids.value)

    def debug_levels(self) -> list[dict]:
        out = []
        for l in range(self.info().levels):
            n, nz, pn = c_i32(), c_i64(), c_i64()
            _check(self._L.svxg_debug_level_dims(self._h, l, ctypes.byref(n), ctypes.byref(nz), ctypes.byref(pn)))
            d = dict(rowptr=np.zeros(n.value + 1, np.int32), col=np.zeros(nz.value, np.int32),
                     val=np.zeros((nz.value, 6, 6)), dinv=np.zeros((n.value, 6, 6)),
                     parent=np.full(n.value, -1, np.int32), prow=np.zeros(n.value + 1, np.int32),
                     pcol=np.zeros(pn.value, np.int32), pval=np.zeros((pn.value, 6, 6)), pos=np.zeros((n.value, 3)))
            lm = c_f64()
            _check(self._L.svxg_debug_level(self._h, l, ptr(d["rowptr"]), ptr(d["col"]), ptr(d["val"]),
                                            ptr(d["dinv"]), ptr(d["parent"]), ptr(d["prow"]), ptr(d["pcol"]),
                                            ptr(d["pval"]), ptr(d["pos"]), ctypes.byref(lm)))
            d["lmax"] = lm.value
            out.append(d)
        return out

    def debug_precondition(self, r):
        r = np.ascontiguousarray(r, dtype=np.float64)
        z = np.zeros_like(r)
        _check(self._L.svxg_debug_precondition(self._h, ptr(r), ptr(z)))
        return z

    def debug_apply(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros_like(x)
        _check(self._L.svxg_debug_apply(self._h, ptr(x), ptr(y)))
        return y


class Batch:
    """Several independent graphs solved as one problem (svxg_set_graphs): every launch of the
    assembly, the multigrid build and the solve covers the whole batch, and the solve stops when
    every graph meets its own target ||r_g|| <= rtol ||f_g||. ``graphs``: (nodes, bonds) pairs
    with one material table."""

    def __init__(self, graphs, mats=None, device: int = 0):
        L = load_library()
        if L.svxg_device_count() <= device:
            raise SvxgError(-6, "no CUDA device")
        h = c_vp()
        _check(L.svxg_problem_create(ctypes.byref(h), device))
        self._h, self._L = h, L
        self.graphs = [(np.ascontiguousarray(n, dtype=NODE_DTYPE), np.ascontiguousarray(b, dtype=BOND_DTYPE))
                       for n, b in graphs]
        self.mats = default_materials() if mats is None else np.ascontiguousarray(mats, dtype=MATERIAL_DTYPE)
        k = len(self.graphs)
        P = c_vp * k
        self._n = np.array([len(g[0]) for g in self.graphs], np.int32)
        self._nb = np.array([len(g[1]) for g in self.graphs], np.int32)
        _check(L.svxg_set_graphs(h, k, P(*[ptr(g[0]) for g in self.graphs]), ptr(self._n),
                                 P(*[ptr(g[1]) for g in self.graphs]), ptr(self._nb), ptr(self.mats)))
        self.node_off = np.concatenate([[0], np.cumsum(self._n)]).astype(np.int64)
        self.bond_off = np.concatenate([[0], np.cumsum(self._nb)]).astype(np.int64)

    def __del__(self):
        h = getattr(self, "_h", None)
        if sys.is_finalizing():
            return
        if h is not None and h.value:
            self._L.svxg_problem_destroy(h)
            self._h = None

    def assemble(self, opt: StressOptions | None = None) -> bool:
        ok = c_i32(0)
        _check(self._L.svxg_assemble(self._h, ctypes.byref(opt) if opt is not None else None, ctypes.byref(ok)))
        return bool(ok.value)

    def solve(self, fs, rtol: float = 1e-6, maxit: int = -1):
        """fs: one load per graph (6 per node). Returns (list of u, PcgResult of the batch, per-graph
        rel. residuals, per-graph converged flags); per-graph iterations in self.iters and, under the
        mixed-precision policy, error estimates in self.error_estimate."""
        f = np.concatenate([np.ascontiguousarray(x, dtype=np.float64).ravel() for x in fs])
        if f.size != 6 * int(self.node_off[-1]):
            raise ValueError("fs: 6 per node of each graph")
        u = np.zeros_like(f)
        res = PcgResult()
        _check(self._L.svxg_solve(self._h, ptr(f), ptr(u), float(rtol), int(maxit), 0, ctypes.byref(res)))
        k = len(self.graphs)
        rel = np.zeros(k)
        conv = np.zeros(k, np.int32)
        its = np.zeros(k, np.int32)
        est = np.zeros(k)
        if k > 1:
            _check(self._L.svxg_graph_results(self._h, k, ptr(rel), ptr(conv), ptr(its), ptr(est)))
        else:
            rel[0], conv[0], its[0] = res.rel_res, res.converged, res.iters
            est[0] = self.info().error_estimate
        self.iters, self.error_estimate = its, est
        us = [u[6 * self.node_off[g]:6 * self.node_off[g + 1]] for g in range(k)]
        return us, res, rel, conv.astype(bool)

    def utilization(self, fragility: float = 1.0):
        """Per graph (phi, mode, failing bonds in the graph's own numbering) at the last solution."""
        nb = int(self.bond_off[-1])
        phi = np.zeros(max(nb, 1))
        mode = np.zeros(max(nb, 1), np.uint8)
        over = np.zeros(max(nb, 1), np.int32)
        cnt = c_i32(0)
        _check(self._L.svxg_utilization(self._h, float(fragility), ptr(phi), ptr(mode), ptr(over), len(over),
                                        ctypes.byref(cnt)))
        over = over[:cnt.value]
        out = []
        for g in range(len(self.graphs)):
            a, b = self.bond_off[g], self.bond_off[g + 1]
            sel = over[(over >= a) & (over < b)] - a
            out.append((phi[a:b].copy(), mode[a:b].copy(), sel.astype(np.int32)))
        return out

    def info(self) -> Info:
        i = Info()
        _check(self._L.svxg_get_info(self._h, ctypes.byref(i)))
        return i


# ---- loads and the judge's free functions (host) ----------------------------------------------------

def structure_loads(weight, ext=None) -> np.ndarray:
    """World::Impl::load_vector (world.cpp:966-974): each node's weight down z plus ext (6 per node)."""
    w = np.ascontiguousarray(weight, dtype=np.float64)
    e = None if ext is None else np.ascontiguousarray(ext, dtype=np.float64)
    f = np.zeros(6 * len(w))
    _check(load_library().svxg_structure_loads(len(w), ptr(w), ptr(e), ptr(f)))
    return f


def pin_reference(nodes, com) -> int:
    """pin_reference (world_pieces.cpp:313-326): `fixed` cleared, the node nearest com fixed (in
    place, nodes a NODE_DTYPE array); returns its index."""
    from .graph import V3
    fn = load_library().svxg_pin_reference
    fn.restype, fn.argtypes = c_i32, [c_vp, c_i32, V3]
    if nodes.dtype != NODE_DTYPE or not nodes.flags["C_CONTIGUOUS"]:
        raise ValueError("nodes: a contiguous NODE_DTYPE array (changed in place)")
    return int(fn(ptr(nodes), len(nodes), V3(*[float(v) for v in com])))


def body_loads(state, nodes, forces, node_com=None, node_mass=None, node_inertia=None, inertia: bool = True):
    """A loose piece's load (world_pieces.cpp:566-603): state a graph.BodyState, forces a
    POINT_FORCE_DTYPE array, node_com (n x 3), node_mass (n), node_inertia (n x 9) for the inertial
    relief. Returns f (6 per node)."""
    from .graph import POINT_FORCE_DTYPE
    nodes = np.ascontiguousarray(nodes, dtype=NODE_DTYPE)
    forces = np.ascontiguousarray(forces, dtype=POINT_FORCE_DTYPE)
    arrs = [None if a is None else np.ascontiguousarray(a, dtype=np.float64) for a in (node_com, node_mass,
                                                                                        node_inertia)]
    f = np.zeros(6 * len(nodes))
    _check(load_library().svxg_body_loads(ctypes.byref(state), ptr(nodes), len(nodes), ptr(arrs[0]), ptr(arrs[1]),
                                          ptr(arrs[2]), ptr(forces), len(forces), int(bool(inertia)), ptr(f)))
    return f


def bond_utilization(bond, load, fragility: float, mats):
    """bond_utilization (stress.cpp:23-57) of one bond record under one load record: (phi, mode)."""
    b = np.ascontiguousarray(np.array([bond], dtype=BOND_DTYPE))
    ld = np.ascontiguousarray(np.array([load], dtype=LOAD_DTYPE))
    mode = np.zeros(1, np.uint8)
    phi = load_library().svxg_bond_utilization(ptr(b), ptr(ld), float(fragility), ptr(mats), ptr(mode))
    return float(phi), int(mode[0])
