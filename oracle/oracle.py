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
        lib.svxo_utilization_many.argtypes = [c_vp, c_vp, c_f64, c_vp, c_vp]
        lib.svxo_build_bonds.argtypes = [c_vp, c_vp, c_i32, c_vp, c_vp, c_vp]
        lib.svxo_invalidate.argtypes = [c_vp]
        lib.svxo_assembled.argtypes = [c_vp]
        lib.svxo_preconditioner_current.argtypes = [c_vp]
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
        lib.svxr_build_bonds.argtypes = [c_vp, c_vp, c_i32, c_vp, c_vp, c_vp]
        lib.svxr_p_create.restype = c_vp
        lib.svxr_p_create.argtypes = [c_vp, c_i32, c_vp, c_i32, c_vp]
        for name in ("destroy", "assembled", "invalidate", "preconditioner_current", "block_jacobi"):
            getattr(lib, "svxr_p_" + name).argtypes = [c_vp]
        lib.svxr_p_assemble.argtypes = [c_vp, c_vp]
        lib.svxr_p_solve.argtypes = [c_vp, c_vp, c_vp, c_f64, c_i32, c_i32, c_vp]
        lib.svxr_p_remove_bond.argtypes = [c_vp, c_i32]
        lib.svxr_p_retire_nodes.argtypes = [c_vp, c_vp, c_i32]
        lib.svxr_p_bond_flags.argtypes = [c_vp, c_vp, c_vp]
        lib.svxr_p_judge.argtypes = [c_vp, c_vp, c_f64, c_vp, c_vp, c_vp]
        lib.svxr_p_utilization_many.argtypes = [c_vp, c_vp, c_f64, c_vp, c_vp]
        lib.svxr_p_matrix.argtypes = [c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]
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


def build_bonds(nodes, secs, faces, mats, reference: bool = False):
    """The bonds of the interfaces `secs` (SECTION_DTYPE) over `faces` (FACE_DTYPE):
    SecAcc::finish_lattice + section_strengths (core/src/world/world_internal.hpp:133-232,
    :370-399). reference=False: the C restatement; True: the reference's own header code
    (ref_shim.cpp)."""
    from opus_destruct_2_gb300.graph import FACE_DTYPE, SECTION_DTYPE
    nodes = np.ascontiguousarray(nodes, dtype=NODE_DTYPE)
    secs = np.ascontiguousarray(secs, dtype=SECTION_DTYPE)
    faces = np.ascontiguousarray(faces, dtype=FACE_DTYPE)
    mats = np.ascontiguousarray(mats, dtype=MATERIAL_DTYPE)
    out = np.zeros(len(secs), BOND_DTYPE)
    if reference:
        lib = reference_lib()
        if lib is None:
            raise RuntimeError("the reference is not built on this machine")
        lib.svxr_build_bonds(ptr(nodes), ptr(secs), len(secs), ptr(faces), ptr(mats), ptr(out))
    else:
        port_lib().svxo_build_bonds(ptr(nodes), ptr(secs), len(secs), ptr(faces), ptr(mats), ptr(out))
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
