"""ctypes bindings of the oracle (TEST INFRASTRUCTURE: the checker, never the product).

``Port``      - the C restatement ``oracle/_build/libsvxo.so`` (every machine).
``Reference`` - the reference compiled from source, ``oracle/_ref/libsvxref.so`` (only where
                the reference tree exists; ``reference_lib()`` returns None elsewhere).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import this module.
"""
from __future__ import annotations

import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, HERE)
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import build_oracle  # noqa: E402
from opus_destruct_2_gb300.graph import (BOND_DTYPE, LOAD_DTYPE, MATERIAL_DTYPE, NODE_DTYPE, PcgResult,  # noqa: E402
                                         StressOptions, ptr)

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
        lib.svxo_seq_sum.restype = c_f64
        lib.svxo_seq_sum.argtypes = [c_vp, c_i64]
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
        _ref = lib
    return _ref


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

    def info(self) -> Info:
        i = Info()
        self.lib.svxo_get_info(self.h, ctypes.byref(i))
        return i

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
