"""ctypes bindings of the oracle (TEST INFRASTRUCTURE: the checker, never the product).

``Port``      - the C restatement ``oracle/_build/libsvxo.so`` (every machine).
``Reference`` - the reference compiled from source, ``oracle/_ref/libsvxref.so`` (only where
                the reference tree exists; ``reference_lib()`` returns None elsewhere).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import this module.
"""
from __future__ import annotations

import ctypes
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, HERE)
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import build_oracle  # noqa: E402
from opus_destruct_2_gb300.graph import (BOND_DTYPE, LOAD_DTYPE, MATERIAL_DTYPE, NODE_DTYPE,  # noqa: E402
                                         POINT_FORCE_DTYPE, V3, PcgResult, StressOptions, ptr)

c_i32, c_i64, c_f64, c_vp = ctypes.c_int32, ctypes.c_int64, ctypes.c_double, ctypes.c_void_p


class Info(ctypes.Structure):
    _fields_ = [("nfree", c_i32), ("levels", c_i32), ("block_jacobi", c_i32), ("chol_n", c_i32),
                ("level_sizes", c_i32 * 16), ("level_blocks", c_i64 * 32), ("matrix_blocks", c_i64),
                ("work_per_iteration", c_i64), ("assembly_work", c_i64), ("work_per_apply", c_i64),
                ("build_work", c_i64)]

    def sizes(self) -> list[int]:
        return [self.level_sizes[i] for i in range(self.levels)]

    def blocks(self) -> list[int]:
        return [self.level_blocks[i] for i in range(2 * self.levels)]


_port = None
_ref = None


def port_lib() -> ctypes.CDLL:
    global _port
    if _port is None:
        lib = ctypes.CDLL(build_oracle.build_port())
        lib.svxo_create.restype = c_vp
        lib.svxo_create.argtypes = [c_vp, c_i32, c_vp, c_i32, c_vp]
        lib.svxo_destroy.argtypes = [c_vp]
        lib.svxo_assemble.argtypes = [c_vp, c_vp]
        lib.svxo_solve.argtypes = [c_vp, c_vp, c_vp, c_f64, c_i32, c_i32, c_vp]
        lib.svxo_begin.argtypes = [c_vp, c_vp, c_vp]
        lib.svxo_iterate.argtypes = [c_vp, c_i32, c_f64, c_vp]
        lib.svxo_current.argtypes = [c_vp, c_vp]
        lib.svxo_remove_bond.argtypes = [c_vp, c_i32]
        lib.svxo_retire_nodes.argtypes = [c_vp, c_vp, c_i32]
        lib.svxo_get_info.argtypes = [c_vp, c_vp]
        lib.svxo_bond_flags.argtypes = [c_vp, c_vp, c_vp]
        lib.svxo_judge.argtypes = [c_vp, c_vp, c_f64, c_vp, c_vp, c_vp]
        lib.svxo_utilization.restype = c_f64
        lib.svxo_utilization.argtypes = [c_vp, c_vp, c_f64, c_vp, c_vp]
        lib.svxo_matrix_dims.argtypes = [c_vp, c_vp, c_vp]
        lib.svxo_matrix.argtypes = [c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]
        lib.svxo_keep_levels.argtypes = [c_vp, ctypes.c_int]
        lib.svxo_levels.argtypes = [c_vp]
        lib.svxo_level_dims.argtypes = [c_vp, c_i32, c_vp, c_vp, c_vp]
        lib.svxo_level_get.argtypes = [c_vp, c_i32] + [c_vp] * 10
        lib.svxo_chol_n.argtypes = [c_vp]
        lib.svxo_chol.argtypes = [c_vp, c_vp]
        lib.svxo_precondition.argtypes = [c_vp, c_vp, c_vp]
        lib.svxo_apply_k.argtypes = [c_vp, c_vp, c_vp]
        lib.svxo_set_threads.argtypes = [ctypes.c_int]
        lib.svxo_set_group_isolated.argtypes = [ctypes.c_int]
        lib.svxo_seq_sum.restype = c_f64
        lib.svxo_utilization_many.argtypes = [c_vp, c_vp, c_f64, c_vp, c_vp]
        lib.svxo_build_bonds.argtypes = [c_vp, c_vp, c_i32, c_vp, c_vp, c_vp, c_i32, c_vp, c_vp]
        lib.svxo_set_broken.argtypes = [c_vp, c_i32, ctypes.c_int]
        lib.svxo_invalidate.argtypes = [c_vp]
        lib.svxo_assembled.argtypes = [c_vp]
        lib.svxo_preconditioner_current.argtypes = [c_vp]
        lib.svxo_seq_sum.argtypes = [c_vp, c_i64]
        lib.svxo_structure_loads.argtypes = [c_i32, c_vp, c_vp, c_vp]
        lib.svxo_pin_reference.restype = c_i32
        lib.svxo_pin_reference.argtypes = [c_vp, c_i32, V3]
        lib.svxo_body_loads.argtypes = [c_vp, c_vp, c_i32, c_vp, c_vp, c_vp, c_vp, c_i32, c_i32, c_vp]
        _port = lib
    return _port


def reference_lib() -> ctypes.CDLL | None:
    global _ref
    if _ref is None:
        path = build_oracle.REF_LIB
        if not os.path.exists(path):
            path = build_oracle.build_reference()
        if not path or not os.path.exists(path):
            return None
        try:
            lib = ctypes.CDLL(path)
        except OSError:  # (built for another machine)
            return None
        lib.svxr_solve.restype = c_i32
        lib.svxr_solve.argtypes = [c_vp, c_i32, c_vp, c_i32, c_vp, c_vp, c_vp, c_vp, c_f64, c_i32, c_i32, c_vp, c_vp,
                                   c_vp, c_vp]
        lib.svxr_judge.argtypes = [c_vp, c_i32, c_vp, c_i32, c_vp, c_vp, c_f64, c_vp, c_vp, c_vp, c_vp]
        lib.svxr_extend_warm_start.argtypes = [c_vp, c_i32, c_vp, c_i32, c_vp, c_vp, c_i32]
        lib.svxr_utilization.restype = c_f64
        lib.svxr_utilization.argtypes = [c_vp, c_vp, c_f64, c_vp, c_vp]
        lib.svxr_matrix.restype = c_i32
        lib.svxr_matrix.argtypes = [c_vp, c_i32, c_vp, c_i32, c_vp] + [c_vp] * 7
        lib.svxr_hier_build.restype = c_vp
        lib.svxr_hier_build.argtypes = [c_vp, c_i32, c_vp, c_i32, c_vp, c_vp, c_vp]
        lib.svxr_hier_levels.argtypes = [c_vp]
        lib.svxr_hier_chol_n.argtypes = [c_vp]
        lib.svxr_hier_chol.argtypes = [c_vp, c_vp]
        lib.svxr_hier_dims.argtypes = [c_vp, c_i32, c_vp, c_vp, c_vp]
        lib.svxr_hier_get.argtypes = [c_vp, c_i32] + [c_vp] * 10
        lib.svxr_hier_free.argtypes = [c_vp]
        lib.svxr_set_threads.argtypes = [ctypes.c_int]
        lib.svxr_build_bonds.argtypes = [c_vp, c_vp, c_i32, c_vp, c_vp, c_vp, c_i32, c_i32, c_vp, c_vp]
        lib.svxr_p_create.restype = c_vp
        lib.svxr_p_create.argtypes = [c_vp, c_i32, c_vp, c_i32, c_vp]
        for name in ("destroy", "assembled", "invalidate", "preconditioner_current", "block_jacobi"):
            getattr(lib, "svxr_p_" + name).argtypes = [c_vp]
        lib.svxr_p_assemble.argtypes = [c_vp, c_vp]
        lib.svxr_p_solve.argtypes = [c_vp, c_vp, c_vp, c_f64, c_i32, c_i32, c_vp]
        lib.svxr_p_remove_bond.argtypes = [c_vp, c_i32]
        lib.svxr_p_set_broken.argtypes = [c_vp, c_i32, ctypes.c_int]
        lib.svxr_p_retire_nodes.argtypes = [c_vp, c_vp, c_i32]
        lib.svxr_p_bond_flags.argtypes = [c_vp, c_vp, c_vp]
        lib.svxr_p_judge.argtypes = [c_vp, c_vp, c_f64, c_vp, c_vp, c_vp]
        lib.svxr_p_utilization_many.argtypes = [c_vp, c_vp, c_f64, c_vp, c_vp]
        lib.svxr_p_matrix.argtypes = [c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]
        lib.svxr_body_loads.argtypes = [c_vp, c_vp, c_i32, c_vp, c_vp, c_vp, c_vp, c_i32, c_i32, c_vp]
        _ref = lib
    return _ref


def set_group_isolated(on: bool) -> None:
    """Pass 3 of the aggregation groups uncoupled leftover rows eight at a time (on: the
    reference) or keeps each single (off: the library's batches of graphs, which must not couple
    their graphs)."""
    port_lib().svxo_set_group_isolated(int(bool(on)))


def structure_loads(weight, ext=None) -> np.ndarray:
    """World::Impl::load_vector (core/src/world/world.cpp:966-974), restated in C."""
    w = np.ascontiguousarray(weight, dtype=np.float64)
    e = None if ext is None else np.ascontiguousarray(ext, dtype=np.float64)
    f = np.zeros(6 * len(w))
    port_lib().svxo_structure_loads(len(w), ptr(w), ptr(e), ptr(f))
    return f


def pin_reference(nodes, com) -> int:
    """pin_reference (core/src/world/world_pieces.cpp:313-326), restated in C; nodes in place."""
    assert nodes.dtype == NODE_DTYPE and nodes.flags["C_CONTIGUOUS"]
    return int(port_lib().svxo_pin_reference(ptr(nodes), len(nodes), V3(*[float(v) for v in com])))


def _body_args(state, nodes, forces, node_com, node_mass, node_inertia):
    nodes = np.ascontiguousarray(nodes, dtype=NODE_DTYPE)
    forces = np.ascontiguousarray(forces, dtype=POINT_FORCE_DTYPE)
    arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (node_com, node_mass, node_inertia)]
    return nodes, forces, arrs


def body_loads(state, nodes, forces, node_com, node_mass, node_inertia, inertia=True, reference=False):
    """A loose piece's loads (core/src/world/world_pieces.cpp:566-603): the C restatement, or with
    reference=True the reference's own vector operators and StressProblem::add_force (None where
    the reference tree is absent)."""
    nodes, forces, arrs = _body_args(state, nodes, forces, node_com, node_mass, node_inertia)
    f = np.zeros(6 * len(nodes))
    args = (ctypes.byref(state), ptr(nodes), len(nodes), ptr(arrs[0]), ptr(arrs[1]), ptr(arrs[2]), ptr(forces),
            len(forces), int(bool(inertia)), ptr(f))
    if reference:
        lib = reference_lib()
        if lib is None:
            return None
        lib.svxr_body_loads(*args)
    else:
        port_lib().svxo_body_loads(*args)
    return f


def set_threads(n: int) -> None:
    port_lib().svxo_set_threads(int(n))
    r = reference_lib()
    if r is not None:
        r.svxr_set_threads(int(n))


def records(nodes, bonds, mats):
    """The C record layouts (converted field by field when a caller's arrays are packed)."""
    n = np.array(nodes, dtype=NODE_DTYPE)
    b = np.array(bonds, dtype=BOND_DTYPE)
    m = np.array(mats, dtype=MATERIAL_DTYPE)
    assert n.dtype.itemsize == 40 and b.dtype.itemsize == 216 and m.dtype.itemsize == 64 and len(m) == 127
    return n, b, m


class Level:
    """One multigrid level in double precision (A, D^-1, aggregates, prolongation)."""

    def __init__(self, n, nnzb, pnnz):
        self.n, self.nnzb, self.pnnz = n, nnzb, pnnz
        self.rowptr = np.zeros(n + 1, np.int32)
        self.col = np.zeros(nnzb, np.int32)
        self.val = np.zeros((nnzb, 6, 6))
        self.dinv = np.zeros((n, 6, 6))
        self.parent = np.full(n, -1, np.int32)
        self.prow = np.zeros(n + 1, np.int32)
        self.pcol = np.zeros(pnnz, np.int32)
        self.pval = np.zeros((pnnz, 6, 6))
        self.pos = np.zeros((n, 3))
        self.lmax = ctypes.c_double(0.0)

    def args(self):
        return [ptr(self.rowptr), ptr(self.col), ptr(self.val), ptr(self.dinv), ptr(self.parent), ptr(self.prow),
                ptr(self.pcol), ptr(self.pval), ptr(self.pos), ctypes.byref(self.lmax)]


class Port:
    """The C restatement of StressProblem (stress.hpp:74-160)."""

    def __init__(self, nodes: np.ndarray, bonds: np.ndarray, mats: np.ndarray):
        self.lib = port_lib()
        self.nodes, self.bonds, self.mats = records(nodes, bonds, mats)
        self.h = self.lib.svxo_create(ptr(self.nodes), len(nodes), ptr(self.bonds), len(bonds), ptr(self.mats))

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.svxo_destroy(self.h)
            self.h = None

    def keep_levels(self, keep=True):
        self.lib.svxo_keep_levels(self.h, int(keep))

    def assemble(self, opt: StressOptions | None = None) -> bool:
        return bool(self.lib.svxo_assemble(self.h, ctypes.byref(opt) if opt is not None else None))

    def solve(self, f, u=None, rtol=1e-8, maxit=500, warm=False):
        n = len(self.nodes)
        f = np.ascontiguousarray(f, dtype=np.float64)
        u = np.zeros(6 * n) if u is None else np.array(u, dtype=np.float64)
        res = PcgResult()
        self.lib.svxo_solve(self.h, ptr(f), ptr(u), rtol, maxit, int(warm), ctypes.byref(res))
        return u, res

    def begin(self, f, u0=None):
        f = np.ascontiguousarray(f, dtype=np.float64)
        u0 = None if u0 is None else np.ascontiguousarray(u0, dtype=np.float64)
        self.lib.svxo_begin(self.h, ptr(f), ptr(u0))

    def iterate(self, maxit, rtol):
        res = PcgResult()
        self.lib.svxo_iterate(self.h, maxit, rtol, ctypes.byref(res))
        return res

    def current(self):
        u = np.zeros(6 * len(self.nodes))
        self.lib.svxo_current(self.h, ptr(u))
        return u

    def remove_bond(self, b):
        self.lib.svxo_remove_bond(self.h, int(b))

    def retire_nodes(self, lst):
        a = np.ascontiguousarray(lst, dtype=np.int32)
        self.lib.svxo_retire_nodes(self.h, ptr(a), len(a))

    def set_broken(self, b, v):
        self.lib.svxo_set_broken(self.h, int(b), int(bool(v)))

    def info(self) -> Info:
        i = Info()
        self.lib.svxo_get_info(self.h, ctypes.byref(i))
        return i

    def assembled(self) -> bool:
        return bool(self.lib.svxo_assembled(self.h))

    def invalidate(self):
        self.lib.svxo_invalidate(self.h)

    def preconditioner_current(self) -> bool:
        return bool(self.lib.svxo_preconditioner_current(self.h))

    def block_jacobi(self) -> bool:
        return bool(self.info().block_jacobi)

    def utilization_many(self, loads, fragility=1.0):
        """bond_utilization of every bond under `loads` (one record per bond)."""
        loads = np.ascontiguousarray(loads, dtype=LOAD_DTYPE)
        phi = np.zeros(len(self.bonds))
        mode = np.zeros(len(self.bonds), np.uint8)
        self.lib.svxo_utilization_many(self.h, ptr(loads), fragility, ptr(phi), ptr(mode))
        return phi, mode

    def bond_flags(self):
        br = np.zeros(len(self.bonds), np.uint8)
        ik = np.zeros(len(self.bonds), np.uint8)
        self.lib.svxo_bond_flags(self.h, ptr(br), ptr(ik))
        return br, ik

    def judge(self, u, fragility=1.0):
        nb = len(self.bonds)
        loads = np.zeros(nb, LOAD_DTYPE)
        phi = np.zeros(nb)
        mode = np.zeros(nb, np.uint8)
        u = np.ascontiguousarray(u, dtype=np.float64)
        self.lib.svxo_judge(self.h, ptr(u), fragility, ptr(loads), ptr(phi), ptr(mode))
        return loads, phi, mode

    def matrix(self):
        nf, nz = c_i32(), c_i64()
        self.lib.svxo_matrix_dims(self.h, ctypes.byref(nf), ctypes.byref(nz))
        dof = np.zeros(len(self.nodes), np.int32)
        rowptr = np.zeros(nf.value + 1, np.int32)
        col = np.zeros(nz.value, np.int32)
        val = np.zeros((nz.value, 6, 6))
        ids = c_f64()
        self.lib.svxo_matrix(self.h, ptr(dof), ptr(rowptr), ptr(col), ptr(val), ctypes.byref(ids))
        return dict(nfree=nf.value, dof=dof, rowptr=rowptr, col=col, val=val, id_scale=ids.value)

    def levels(self) -> list[Level]:
        out = []
        for l in range(self.lib.svxo_levels(self.h)):
            n, nz, pn = c_i32(), c_i64(), c_i64()
            self.lib.svxo_level_dims(self.h, l, ctypes.byref(n), ctypes.byref(nz), ctypes.byref(pn))
            L = Level(n.value, nz.value, pn.value)
            self.lib.svxo_level_get(self.h, l, *L.args())
            out.append(L)
        return out

    def chol(self):
        m = self.lib.svxo_chol_n(self.h)
        c = np.zeros((m, m))
        if m:
            self.lib.svxo_chol(self.h, ptr(c))
        return c

    def precondition(self, r):
        r = np.ascontiguousarray(r, dtype=np.float64)
        z = np.zeros_like(r)
        self.lib.svxo_precondition(self.h, ptr(r), ptr(z))
        return z

    def apply_k(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros_like(x)
        self.lib.svxo_apply_k(self.h, ptr(x), ptr(y))
        return y


def extend_warm_start(nodes, bonds, u, first_new: int):
    """StressProblem::extend_warm_start (core/src/stress/stress.cpp:213-244), restated: nodes from
    first_new on take the mean rigid transfer (u_a + th_a x (x_c - x_a)) of their intact bonds'
    known neighbours, for up to four passes, bonds in index order. Returns the new u."""
    n = len(nodes)
    u = np.array(u, dtype=np.float64)
    if first_new >= n or u.size != 6 * n:
        return u
    c = [(float(x), float(y), float(z)) for x, y, z in zip(nodes["c"]["x"], nodes["c"]["y"], nodes["c"]["z"])]
    known = [i < first_new and not nodes["gone"][i] for i in range(n)]
    for _ in range(4):
        acc = [[0.0] * 6 for _ in range(n)]
        w = [0.0] * n
        for a, b, broken in zip(bonds["a"], bonds["b"], bonds["broken"]):
            a, b = int(a), int(b)
            if broken or b < 0:
                continue
            for src, dst in ((a, b), (b, a)):
                if known[src] and not known[dst] and dst >= first_new:
                    r = (c[dst][0] - c[src][0], c[dst][1] - c[src][1], c[dst][2] - c[src][2])
                    th = (u[6 * src + 3], u[6 * src + 4], u[6 * src + 5])
                    t = (th[1] * r[2] - th[2] * r[1], th[2] * r[0] - th[0] * r[2], th[0] * r[1] - th[1] * r[0])
                    for q in range(3):
                        acc[dst][q] += u[6 * src + q] + t[q]
                    for q in range(3, 6):
                        acc[dst][q] += u[6 * src + q]
                    w[dst] += 1.0
                    break
        changed = False
        for i in range(first_new, n):
            if known[i] or w[i] == 0.0:
                continue
            for q in range(6):
                u[6 * i + q] = acc[i][q] / w[i]
            known[i] = True
            changed = True
        if not changed:
            break
    return u


class Reference:
    """The reference's own StressProblem, compiled from its sources (see ref_shim.cpp)."""

    def __init__(self, nodes, bonds, mats):
        self.lib = reference_lib()
        if self.lib is None:
            raise RuntimeError("the reference is not built on this machine")
        self.nodes, self.bonds, self.mats = records(nodes, bonds, mats)

    def solve(self, f, opt: StressOptions | None = None, u=None, rtol=1e-8, maxit=500, warm=False):
        n = len(self.nodes)
        f = np.ascontiguousarray(f, dtype=np.float64)
        u = np.zeros(6 * n) if u is None else np.array(u, dtype=np.float64)
        res, info = PcgResult(), Info()
        ta, ts = c_f64(), c_f64()
        ok = self.lib.svxr_solve(ptr(self.nodes), n, ptr(self.bonds), len(self.bonds), ptr(self.mats),
                                 ctypes.byref(opt) if opt is not None else None, ptr(f), ptr(u), rtol, maxit,
                                 int(warm), ctypes.byref(res), ctypes.byref(info), ctypes.byref(ta),
                                 ctypes.byref(ts))
        return dict(ok=bool(ok), u=u, res=res, info=info, t_assemble=ta.value, t_solve=ts.value)

    def extend_warm_start(self, u, first_new: int):
        out = np.array(u, dtype=np.float64)
        self.lib.svxr_extend_warm_start(ptr(self.nodes), len(self.nodes), ptr(self.bonds), len(self.bonds),
                                        ptr(self.mats), ptr(out), int(first_new))
        return out

    def judge(self, u, fragility=1.0):
        nb = len(self.bonds)
        loads = np.zeros(nb, LOAD_DTYPE)
        phi = np.zeros(nb)
        mode = np.zeros(nb, np.uint8)
        t = c_f64()
        u = np.ascontiguousarray(u, dtype=np.float64)
        self.lib.svxr_judge(ptr(self.nodes), len(self.nodes), ptr(self.bonds), nb, ptr(self.mats), ptr(u),
                            fragility, ptr(loads), ptr(phi), ptr(mode), ctypes.byref(t))
        return loads, phi, mode

    def matrix(self):
        nf, nz = c_i32(), c_i64()
        args = [ptr(self.nodes), len(self.nodes), ptr(self.bonds), len(self.bonds), ptr(self.mats)]
        self.lib.svxr_matrix(*args, ctypes.byref(nf), ctypes.byref(nz), None, None, None, None, None)
        dof = np.zeros(len(self.nodes), np.int32)
        rowptr = np.zeros(nf.value + 1, np.int32)
        col = np.zeros(nz.value, np.int32)
        val = np.zeros((nz.value, 6, 6))
        ids = c_f64()
        self.lib.svxr_matrix(*args, ctypes.byref(nf), ctypes.byref(nz), ptr(dof), ptr(rowptr), ptr(col), ptr(val),
                             ctypes.byref(ids))
        return dict(nfree=nf.value, dof=dof, rowptr=rowptr, col=col, val=val, id_scale=ids.value)

    def levels(self, opt: StressOptions | None = None):
        ok = c_i32()
        h = self.lib.svxr_hier_build(ptr(self.nodes), len(self.nodes), ptr(self.bonds), len(self.bonds),
                                     ptr(self.mats), ctypes.byref(opt) if opt is not None else None,
                                     ctypes.byref(ok))
        if not h:
            return None, None
        out = []
        for l in range(self.lib.svxr_hier_levels(h)):
            n, nz, pn = c_i32(), c_i64(), c_i64()
            self.lib.svxr_hier_dims(h, l, ctypes.byref(n), ctypes.byref(nz), ctypes.byref(pn))
            L = Level(n.value, nz.value, pn.value)
            self.lib.svxr_hier_get(h, l, *L.args())
            out.append(L)
        m = self.lib.svxr_hier_chol_n(h)
        chol = np.zeros((m, m))
        if m:
            self.lib.svxr_hier_chol(h, ptr(chol))
        self.lib.svxr_hier_free(h)
        return out, chol

    def utilization(self, bond, load, fragility=1.0):
        mode = ctypes.c_uint8()
        b = np.ascontiguousarray(bond)
        L = np.ascontiguousarray(load)
        phi = self.lib.svxr_utilization(ptr(b), ptr(L), fragility, ptr(self.mats), ctypes.byref(mode))
        return phi, mode.value


def build_bonds(nodes, secs, faces, mats, reference: bool = False, junctions=None, lattices=None,
                samples: int = 2):
    """The bonds of the interfaces `secs` (SECTION_DTYPE) over `faces` (FACE_DTYPE) and, where
    given, `junctions` (JUNCTION_DTYPE) and `lattices` (LATTICE_DTYPE): SecAcc::finish +
    section_strengths(_general) (core/src/world/world_internal.hpp:130-441). reference=False: the
    C restatement; True: the reference's own header code (ref_shim.cpp)."""
    from opus_destruct_2_gb300.graph import FACE_DTYPE, JUNCTION_DTYPE, LATTICE_DTYPE, SECTION_DTYPE
    nodes = np.ascontiguousarray(nodes, dtype=NODE_DTYPE)
    secs = np.ascontiguousarray(secs, dtype=SECTION_DTYPE)
    faces = np.ascontiguousarray(faces, dtype=FACE_DTYPE)
    mats = np.ascontiguousarray(mats, dtype=MATERIAL_DTYPE)
    js = None if junctions is None else np.ascontiguousarray(junctions, dtype=JUNCTION_DTYPE)
    ls = None if lattices is None else np.ascontiguousarray(lattices, dtype=LATTICE_DTYPE)
    out = np.zeros(len(secs), BOND_DTYPE)
    if reference:
        lib = reference_lib()
        if lib is None:
            raise RuntimeError("the reference is not built on this machine")
        lib.svxr_build_bonds(ptr(nodes), ptr(secs), len(secs), ptr(faces), ptr(js), ptr(ls),
                             0 if ls is None else len(ls), int(samples), ptr(mats), ptr(out))
    else:
        port_lib().svxo_build_bonds(ptr(nodes), ptr(secs), len(secs), ptr(faces), ptr(js), ptr(ls), int(samples),
                                    ptr(mats), ptr(out))
    return out


class RefProblem:
    """One of the reference's own StressProblem kept between calls (ref_shim.cpp), with Port's
    methods, so that the break rounds below run on the reference itself."""

    def __init__(self, nodes, bonds, mats):
        self.lib = reference_lib()
        if self.lib is None:
            raise RuntimeError("the reference is not built on this machine")
        self.nodes, self.bonds, self.mats = records(nodes, bonds, mats)
        self.h = self.lib.svxr_p_create(ptr(self.nodes), len(self.nodes), ptr(self.bonds), len(self.bonds),
                                        ptr(self.mats))

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.svxr_p_destroy(self.h)
            self.h = None

    def assemble(self, opt: StressOptions | None = None) -> bool:
        return bool(self.lib.svxr_p_assemble(self.h, ctypes.byref(opt) if opt is not None else None))

    def assembled(self) -> bool:
        return bool(self.lib.svxr_p_assembled(self.h))

    def invalidate(self):
        self.lib.svxr_p_invalidate(self.h)

    def preconditioner_current(self) -> bool:
        return bool(self.lib.svxr_p_preconditioner_current(self.h))

    def block_jacobi(self) -> bool:
        return bool(self.lib.svxr_p_block_jacobi(self.h))

    def solve(self, f, u=None, rtol=1e-8, maxit=500, warm=False):
        f = np.ascontiguousarray(f, dtype=np.float64)
        u = np.zeros(6 * len(self.nodes)) if u is None else np.array(u, dtype=np.float64)
        res = PcgResult()
        self.lib.svxr_p_solve(self.h, ptr(f), ptr(u), rtol, maxit, int(warm), ctypes.byref(res))
        return u, res

    def remove_bond(self, b):
        self.lib.svxr_p_remove_bond(self.h, int(b))

    def retire_nodes(self, lst):
        a = np.ascontiguousarray(lst, dtype=np.int32)
        self.lib.svxr_p_retire_nodes(self.h, ptr(a), len(a))

    def set_broken(self, b, v):
        self.lib.svxr_p_set_broken(self.h, int(b), int(bool(v)))

    def bond_flags(self):
        br = np.zeros(len(self.bonds), np.uint8)
        ik = np.zeros(len(self.bonds), np.uint8)
        self.lib.svxr_p_bond_flags(self.h, ptr(br), ptr(ik))
        return br, ik

    def judge(self, u, fragility=1.0):
        nb = len(self.bonds)
        loads = np.zeros(nb, LOAD_DTYPE)
        phi = np.zeros(nb)
        mode = np.zeros(nb, np.uint8)
        u = np.ascontiguousarray(u, dtype=np.float64)
        self.lib.svxr_p_judge(self.h, ptr(u), fragility, ptr(loads), ptr(phi), ptr(mode))
        return loads, phi, mode

    def utilization_many(self, loads, fragility=1.0):
        loads = np.ascontiguousarray(loads, dtype=LOAD_DTYPE)
        phi = np.zeros(len(self.bonds))
        mode = np.zeros(len(self.bonds), np.uint8)
        self.lib.svxr_p_utilization_many(self.h, ptr(loads), fragility, ptr(phi), ptr(mode))
        return phi, mode

    def matrix(self):
        nf, nz = c_i32(), c_i64()
        self.lib.svxr_p_matrix(self.h, ctypes.byref(nf), ctypes.byref(nz), None, None, None)
        rowptr = np.zeros(nf.value + 1, np.int32)
        col = np.zeros(nz.value, np.int32)
        val = np.zeros((nz.value, 6, 6))
        self.lib.svxr_p_matrix(self.h, ctypes.byref(nf), ctypes.byref(nz), ptr(rowptr), ptr(col), ptr(val))
        return dict(nfree=nf.value, rowptr=rowptr, col=col, val=val)


# ---- the judge's break rounds (restated) ---------------------------------------------------------

LOAD_FIELDS = ("N", "V1", "V2", "T", "M1", "M2")


def supported_nodes(n: int, bonds, broken, gone=None) -> np.ndarray:
    """graph_components (core/src/world/world_internal.hpp:660-705) as detach_unsupported seeds it
    (core/src/world/world.cpp:1371-1377): component 0 is every node reachable over intact
    node-to-node bonds from a node with an intact support bond. Returns a bool per node (True:
    in component 0). `gone` is not read: a node retired before has no intact bond left."""
    from scipy.sparse import coo_matrix
    from scipy.sparse.csgraph import connected_components
    a = np.asarray(bonds["a"], dtype=np.int64)
    b = np.asarray(bonds["b"], dtype=np.int64)
    live = np.asarray(broken) == 0
    seed = np.zeros(n, bool)
    seed[a[live & (b < 0)]] = True
    e = live & (b >= 0)
    if n == 0:
        return seed
    g = coo_matrix((np.ones(int(e.sum()), np.int8), (a[e], b[e])), shape=(n, n))
    _, lab = connected_components(g, directed=False)
    held = np.zeros(lab.max() + 1, bool)
    held[lab[seed]] = True
    return held[lab]


def select_breaks(over_b, over_phi, band: float, max_breaks: int) -> list[int]:
    """The bonds one round breaks (core/src/world/world.cpp:1219-1271): `over` sorted by phi
    descending then index ascending; thr = max(1, band x max phi); the loop takes bonds while
    phi >= thr or fewer than the quota max(1, (m + 3) / 4) are taken, at most max_breaks."""
    m = len(over_b)
    order = np.lexsort((over_b, -over_phi))
    ob, op = over_b[order], over_phi[order]
    top = float(op[0])
    x = band * top
    thr = x if 1.0 < x else 1.0
    quota = max(1, (m + 3) // 4)
    out = []
    for k in range(m):
        if (op[k] < thr and k >= quota) or len(out) >= max_breaks:
            break
        out.append(int(ob[k]))
    return out


def cascade(P, f, u, o, opt: StressOptions | None = None, judged=None, has=None):
    """The judge's break rounds of one structure, on a problem with Port's methods (Port: the C
    restatement; RefProblem: the reference itself). Each round:

      1. assemble if needed (after a restart on a stale preconditioner: amg_min_nodes = 0, the
         structure's multigrid flag, world.cpp:1030), then solve warm from u with at most o.maxit
         iterations (world.cpp:1041-1050). Breakdown: stop (status BREAKDOWN, u as it started).
         Not converged: restart as world.cpp:1070-1093 (keep the iterate unless it diverged,
         rel_res >= 10; rebuild the preconditioner if it is stale or block-Jacobi, else a diverged
         one starts from rest); o.solve_restarts in a row: stop (ABANDONED).
      2. converged after more than o.rebuild_after iterations on a stale preconditioner (or a
         block-Jacobi one): rebuild before the next solve (world.cpp:1109).
      3. judge (world.cpp:1162-1201): every intact bond's load L; its utilization under
         lerp(judged, L, dif) if a shock is on, dif != 1 and the bond was judged before, else
         under L; judged := L. No bond at or over 1, or o.max_rounds rounds done: stop.
      4. break the bonds select_breaks() picks, in that order, with remove_bond (world.cpp:1258-1270);
         a shock is on from now on.
      5. o.detach: retire every node not held by a support (world.cpp:1371-1458), zero their
         loads and motion (world.cpp:1460-1478).

    Returns a dict: u, f, judged, has, broken (in order), retired (in order), per_round (bonds
    broken per round), phi (last judgement), and the svxg_cascade_result fields."""
    n = len(P.nodes)
    nb = len(P.bonds)
    f = np.array(f, dtype=np.float64)
    u = np.array(u, dtype=np.float64)
    judged = np.zeros(nb, LOAD_DTYPE) if judged is None else np.array(judged, dtype=LOAD_DTYPE)
    has = np.zeros(nb, np.uint8) if has is None else np.array(has, dtype=np.uint8)
    gone = np.array(P.nodes["gone"], dtype=np.uint8)
    opt = StressOptions() if opt is None else opt
    opt_mg = StressOptions()
    ctypes.memmove(ctypes.byref(opt_mg), ctypes.byref(opt), ctypes.sizeof(StressOptions))
    opt_mg.amg_min_nodes = 0
    shock = bool(o.shock)
    multigrid = False
    restarts = 0
    out = dict(status=0, rounds=0, bonds_broken=0, nodes_retired=0, solves=0, restarts=0, pcg_iters=0,
               max_utilization=0.0, rel_res=0.0, broken=[], retired=[], per_round=[], phi=np.zeros(nb))
    while True:
        if not P.assembled() and not P.assemble(opt_mg if multigrid else opt):
            out["status"] = 4
            break
        u0 = u.copy()
        u, r = P.solve(f, u, o.rtol, o.maxit, True)
        out["solves"] += 1
        out["pcg_iters"] += r.iters
        out["rel_res"] = r.rel_res
        if r.breakdown:
            u = u0
            out["status"] = 3
            break
        if not r.converged:
            rebuild = (not P.preconditioner_current()) or P.block_jacobi()
            diverging = not (r.rel_res < 10.0)
            if diverging:
                u = u0
            if rebuild:
                P.invalidate()
                multigrid = True
            elif diverging:
                u = np.zeros_like(u)
            restarts += 1
            out["restarts"] += 1
            if restarts >= o.solve_restarts:
                out["status"] = 2
                break
            continue
        restarts = 0
        if r.iters > o.rebuild_after and ((not P.preconditioner_current()) or P.block_jacobi()):
            P.invalidate()
        broken, _ = P.bond_flags()
        live = broken == 0
        loads, _, _ = P.judge(u, o.fragility)
        le = loads.copy()
        if shock and o.dif != 1.0:
            w = live & (has != 0)
            for k in LOAD_FIELDS:
                le[k][w] = judged[k][w] + o.dif * (loads[k][w] - judged[k][w])
        phi, _ = P.utilization_many(le, o.fragility)
        judged[live] = loads[live]
        has[live] = 1
        phi = np.where(live, phi, 0.0)
        out["phi"] = phi
        mx = 0.0
        for v in phi[live]:
            mx = v if mx < v else mx
        out["max_utilization"] = float(mx)
        over = np.nonzero(live & (phi >= 1.0))[0]
        if len(over) == 0:
            out["status"] = 0
            break
        if out["rounds"] >= o.max_rounds:
            out["status"] = 1
            break
        sel = select_breaks(over, phi[over], o.break_band, o.max_breaks_per_round)
        for b in sel:
            P.remove_bond(b)
        out["broken"].extend(sel)
        out["per_round"].append(len(sel))
        out["bonds_broken"] += len(sel)
        out["rounds"] += 1
        shock = True
        if o.detach:
            broken, _ = P.bond_flags()
            held = supported_nodes(n, P.bonds, broken)
            ret = np.nonzero(~held & (gone == 0))[0].astype(np.int32)
            if len(ret):
                P.retire_nodes(ret)
                gone[ret] = 1
                for q in range(6):
                    f[6 * ret + q] = 0.0
                    u[6 * ret + q] = 0.0
                out["retired"].extend(int(i) for i in ret)
                out["nodes_retired"] += len(ret)
    out.update(u=u, f=f, judged=judged, has=has)
    return out


# ---- a loose piece's break rounds (restated) -----------------------------------------------------

CRUSH = 2  # FailMode::Crush (svxg_types.h SVXG_FAIL_CRUSH)


def _cross(a, b):
    return (a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0])


def pin_components(n: int, bonds, broken, pin: int):
    """graph_components (core/src/world/world_internal.hpp:660-705) seeded by the pinned node:
    component 0 holds every node reachable from it over intact node-to-node bonds, the others are
    numbered from 1 in node order. Returns (labels, count)."""
    from scipy.sparse import coo_matrix
    from scipy.sparse.csgraph import connected_components
    a = np.asarray(bonds["a"], dtype=np.int64)
    b = np.asarray(bonds["b"], dtype=np.int64)
    e = (np.asarray(broken) == 0) & (b >= 0)
    g = coo_matrix((np.ones(int(e.sum()), np.int8), (a[e], b[e])), shape=(n, n))
    _, lab = connected_components(g, directed=False)
    comp = np.full(n, -1, np.int64)
    comp[lab == lab[pin]] = 0
    nc = 1
    for i in range(n):
        if comp[i] < 0:
            comp[lab == lab[i]] = nc
            nc += 1
    return comp, nc


def piece_rounds(P, f, u, o, gf, opt: StressOptions | None = None):
    """A loose piece's break rounds within one substep (World::Impl::body_stress_run,
    core/src/world/world_pieces.cpp:614-808) on a problem with Port's methods, load f given (its
    inertial relief and point forces), warm start u. Each round: solve (at most o.maxit
    iterations; a failed solve after the first round rebuilds the preconditioner once, then
    gives up); judge every intact bond whose node a is not retired; break the worst (phi >=
    max(1, band x max phi), at least ceil(round_fraction x m), at most max_breaks), each crack paid
    from o.energy when it is >= 0 (crushing costs crush_energy x more); stop when the energy runs
    out, nothing broke or it was the last round; else split from the pinned node: a part heavier
    than chip_fraction x the piece ends the rounds (the piece came apart), lighter parts (chips)
    pass their load to the nodes they broke from and retire. gf: Gf per material id.
    Returns a dict with u, f, broken (in order), modes (of those), chips (in order) and the
    svxg_piece_result fields."""
    n, nb = len(P.nodes), len(P.bonds)
    f = np.array(f, dtype=np.float64)
    u = np.array(u, dtype=np.float64)
    gone = np.array(P.nodes["gone"], dtype=np.uint8)
    fixed = np.array(P.nodes["fixed"], dtype=np.uint8)
    mass = np.array(P.nodes["mass"], dtype=np.float64)
    c = [(float(x), float(y), float(z)) for x, y, z in zip(P.nodes["c"]["x"], P.nodes["c"]["y"], P.nodes["c"]["z"])]
    body_mass = 0.0
    for i in range(n):
        if not gone[i]:
            body_mass += float(mass[i])
    base = StressOptions() if opt is None else opt
    so = StressOptions()
    ctypes.memmove(ctypes.byref(so), ctypes.byref(base), ctypes.sizeof(StressOptions))
    so.rtol = o.rtol
    so.amg_min_nodes = 0
    out = dict(status=0, checks=0, bonds_broken=0, chips=0, pcg_iters=0, rebuilt=0, spent=0.0,
               first_max_utilization=0.0, max_utilization=0.0, broken=[], modes=[], chip_nodes=[])
    if not P.assembled() and not P.assemble(so):
        out["status"] = 6
        out.update(u=u, f=f)
        return out
    impact = o.energy >= 0.0
    rounds = max(1, o.rounds)
    spent = 0.0
    rebuilt = False
    a_of = np.asarray(P.bonds["a"], np.int64)
    b_of = np.asarray(P.bonds["b"], np.int64)
    area = np.asarray(P.bonds["area"], np.float64)
    strength = np.asarray(P.bonds["strength"], np.float64)
    ma, mb = np.asarray(P.bonds["ma"]), np.asarray(P.bonds["mb"])
    for rnd in range(rounds):
        u, r = P.solve(f, u, o.rtol, o.maxit, True)
        if not r.converged and (r.breakdown or r.rel_res > 5.0 * o.rtol) and rnd > 0 and not rebuilt:
            rebuilt = True
            out["rebuilt"] = 1
            P.invalidate()
            if P.assemble(so):
                u, r = P.solve(f, u, o.rtol, o.maxit, True)
        if not r.converged and (r.breakdown or r.rel_res > 5.0 * o.rtol):
            P.invalidate()
            u = np.zeros_like(u)
            out["status"] = 4
            break
        out["checks"] += 1
        out["pcg_iters"] += r.iters
        broken, _ = P.bond_flags()
        _, phi, mode = P.judge(u, o.fragility)
        live = (broken == 0) & (gone[a_of] == 0)
        mx = 0.0
        for v in phi[live]:
            mx = v if mx < v else mx
        if rnd == 0:
            out["first_max_utilization"] = float(mx)
        out["max_utilization"] = float(mx)
        over = np.nonzero(live & (phi >= 1.0))[0]
        if len(over) == 0:
            out["status"] = 0
            break
        order = np.lexsort((over, -phi[over]))
        ob, op = over[order], phi[over][order]
        x = o.break_band * float(op[0])
        thr = x if 1.0 < x else 1.0
        quota = int(math.ceil(o.round_fraction * float(len(over))))
        sel = []
        poor = False
        for q in range(len(ob)):
            k = int(ob[q])
            if (op[q] < thr and q >= quota) or len(sel) >= o.max_breaks_per_round:
                break
            if impact:
                crush = o.crush_energy if mode[k] == CRUSH else 1.0
                g1, g2 = float(gf[ma[k]]), float(gf[mb[k]])
                cost = o.fracture_energy * crush * float(area[k]) * (g2 if g2 < g1 else g1) * float(strength[k])
                if spent + cost > o.energy:
                    poor = True
                    break
                spent += cost
            sel.append(k)
        for k in sel:
            P.remove_bond(k)
        out["broken"].extend(sel)
        out["modes"].extend(int(mode[k]) for k in sel)
        out["bonds_broken"] += len(sel)
        out["spent"] = spent
        if poor or not sel or rnd + 1 == rounds:
            out["status"] = 1 if poor else (0 if not sel else 3)
            break
        pin = -1
        for i in range(n):
            if fixed[i]:
                pin = i
        if pin < 0:
            out["status"] = 5
            break
        broken, _ = P.bond_flags()
        comp, nc = pin_components(n, P.bonds, broken, pin)
        if nc <= 1:
            continue
        cmass = [0.0] * nc
        for i in range(n):
            if not gone[i]:
                cmass[comp[i]] += float(mass[i])
        if any(cmass[k] > o.chip_fraction * body_mass for k in range(1, nc)):
            out["status"] = 2
            break
        # chips (world_pieces.cpp:752-808)
        attach = [[] for _ in range(nc)]
        for k in range(nb):
            if not broken[k] or b_of[k] < 0:
                continue
            ca, cb = comp[a_of[k]], comp[b_of[k]]
            if ca > 0 and cb == 0 and not gone[b_of[k]]:
                attach[ca].append(int(b_of[k]))
            if cb > 0 and ca == 0 and not gone[a_of[k]]:
                attach[cb].append(int(a_of[k]))
        cF = [[0.0, 0.0, 0.0] for _ in range(nc)]
        cM = [[0.0, 0.0, 0.0] for _ in range(nc)]
        chip_nodes = []
        for i in range(n):
            ci = comp[i]
            if ci == 0 or gone[i]:
                continue
            chip_nodes.append(i)
            A = attach[ci]
            if not A:
                best, bj = 1e300, -1
                for j in range(n):
                    if comp[j] != 0 or gone[j]:
                        continue
                    d = (c[j][0] - c[i][0], c[j][1] - c[i][1], c[j][2] - c[i][2])
                    d2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2]
                    if d2 < best:
                        best, bj = d2, j
                if bj < 0:
                    continue
                A.append(bj)
            Fi = (float(f[6 * i]), float(f[6 * i + 1]), float(f[6 * i + 2]))
            for q in range(3):
                cF[ci][q] += Fi[q]
            t = _cross(c[i], Fi)
            Mi = (float(f[6 * i + 3]) + t[0], float(f[6 * i + 4]) + t[1], float(f[6 * i + 5]) + t[2])
            for q in range(3):
                cM[ci][q] += Mi[q]
            f[6 * i:6 * i + 6] = 0.0
        for ci in range(1, nc):
            A = sorted(set(attach[ci]))
            if not A:
                continue
            w = 1.0 / float(len(A))
            Fj = (cF[ci][0] * w, cF[ci][1] * w, cF[ci][2] * w)
            Mr = list(cM[ci])
            for j in A:
                t = _cross(c[j], Fj)
                Mr = [Mr[0] - t[0], Mr[1] - t[1], Mr[2] - t[2]]
            Mj = (Mr[0] * w, Mr[1] * w, Mr[2] * w)
            for j in A:
                for q in range(3):
                    f[6 * j + q] += Fj[q]
                    f[6 * j + 3 + q] += Mj[q]
        inner = [k for k in range(nb) if not broken[k] and b_of[k] >= 0 and comp[a_of[k]] > 0
                 and comp[a_of[k]] == comp[b_of[k]]]
        P.retire_nodes(chip_nodes)
        for k in inner:
            P.set_broken(k, False)
        for i in chip_nodes:
            gone[i] = 1
            u[6 * i:6 * i + 6] = 0.0
        out["chip_nodes"].extend(chip_nodes)
        out["chips"] += len(chip_nodes)
    out.update(u=u, f=f)
    return out
