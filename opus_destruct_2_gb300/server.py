"""Many stress solves in flight on one GPU: the serving loop and the batched solve
(``include/svxg_server.h``).

The reference runs independent graphs concurrently on host threads, one StressProblem per graph
(core/src/world/world_pieces.cpp:1460-1463). ``Server`` does that on the device: its slots (host
threads of the CUDA library) each drive a problem on its own CUDA stream, new structures are
admitted against an HBM budget, structures can be kept resident for warm-started repeat solves
after in-place bond removal, and every request's latency is recorded. ``batch_solve`` is the
same engine given a list of graphs at once.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import SvxgError, _check, load_library
from .graph import (BOND_DTYPE, MATERIAL_DTYPE, NODE_DTYPE, PieceOptions, PieceResult, StressOptions,
                    default_fracture_energies, ptr)

c_i32, c_i64, c_f64, c_vp = ctypes.c_int32, ctypes.c_int64, ctypes.c_double, ctypes.c_void_p


class RequestResult(ctypes.Structure):
    _fields_ = [("ticket", c_i64), ("status", c_i32), ("iters", c_i32), ("converged", c_i32),
                ("breakdown", c_i32), ("failing", c_i32), ("warm", c_i32), ("rel_res", c_f64),
                ("queue_ms", c_f64), ("latency_ms", c_f64), ("err_est", c_f64)]


class ServingStats(ctypes.Structure):
    _fields_ = [("completed", c_i64), ("failed", c_i64), ("evictions", c_i64), ("admission_waits", c_i64),
                ("resident", c_i64), ("resident_bytes", c_i64), ("peak_bytes", c_i64), ("pad", c_i64),
                ("p50_ms", c_f64), ("p99_ms", c_f64), ("max_ms", c_f64), ("wall_s", c_f64),
                ("batches", c_i64), ("batched_requests", c_i64)]


_bound = False


def _bind():
    global _bound
    L = load_library()
    if _bound:
        return L
    sig = {
        "svxg_server_create": (c_i32, [ctypes.POINTER(c_vp), c_i32, c_i64, c_i32]),
        "svxg_server_destroy": (None, [c_vp]),
        "svxg_server_submit": (c_i64, [c_vp, c_i64, c_vp, c_i32, c_vp, c_i32, c_vp, c_vp, c_vp, c_f64, c_i32,
                                       c_f64, c_vp, c_vp]),
        "svxg_server_submit_repeat": (c_i64, [c_vp, c_i64, c_vp, c_i32, c_vp, c_i32, c_f64, c_i32, c_f64, c_vp,
                                              c_vp]),
        "svxg_server_submit_device": (c_i64, [c_vp, c_i64, c_vp, c_i32, c_vp, c_i32, c_vp, c_vp, c_vp, c_f64,
                                              c_i32, c_f64, c_vp, c_vp]),
        "svxg_server_submit_repeat_device": (c_i64, [c_vp, c_i64, c_vp, c_i32, c_vp, c_i32, c_f64, c_i32, c_f64,
                                                     c_vp, c_vp]),
        "svxg_server_set_batching": (c_i32, [c_vp, c_i32, c_i32, c_i64]),
        "svxg_server_hold": (c_i32, [c_vp, c_i32]),
        "svxg_server_wait": (c_i32, [c_vp, c_i64, c_vp]),
        "svxg_server_drain": (c_i32, [c_vp]),
        "svxg_server_stats": (c_i32, [c_vp, c_vp]),
        "svxg_server_reset_stats": (c_i32, [c_vp]),
        "svxg_server_forget": (c_i32, [c_vp, c_i64]),
        "svxg_server_estimate_bytes": (c_i64, [c_i32, c_i32]),
        "svxg_batch_solve": (c_i32, [c_vp, c_i32, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_f64, c_i32, c_f64,
                                     c_vp, c_vp, c_vp]),
        "svxg_batch_piece_rounds": (c_i32, [c_vp, c_i32, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp,
                                            c_vp, c_vp, c_vp, c_vp, c_vp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _bound = True
    return L


def _graph(nodes, bonds, f):
    nodes = np.ascontiguousarray(nodes, dtype=NODE_DTYPE)
    bonds = np.ascontiguousarray(bonds, dtype=BOND_DTYPE)
    f = np.ascontiguousarray(f, dtype=np.float64)
    if f.size != 6 * len(nodes):
        raise ValueError("f: 6 per node")
    return nodes, bonds, f


def estimate_bytes(n: int, nb: int) -> int:
    """The bytes a server reserves for a new structure of n nodes and nb bonds while it runs."""
    return int(_bind().svxg_server_estimate_bytes(int(n), int(nb)))


class Server:
    """A request loop on one GPU: ``workers`` slots, ``budget`` bytes of problem memory."""

    def __init__(self, device: int = 0, budget: int = 40 << 30, workers: int = 8):
        self._L = _bind()
        h = c_vp()
        _check(self._L.svxg_server_create(ctypes.byref(h), int(device), int(budget), int(workers)))
        self._h = h
        self._keep = {}  # ticket -> buffers the library writes into (alive until waited for)

    def close(self):
        if self._h:
            self._L.svxg_server_destroy(self._h)
            self._h = None
            self._keep.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def submit(self, nodes, bonds, mats, f, structure: int = -1, opt: StressOptions | None = None,
               rtol: float = 1e-6, maxit: int = -1, fragility: float = 1.0, want_u: bool = True,
               want_over: bool = False) -> int:
        """A new graph: assemble, solve from zero, judge. Returns the ticket."""
        nodes, bonds, f = _graph(nodes, bonds, f)
        mats = np.ascontiguousarray(mats, dtype=MATERIAL_DTYPE)
        u = np.zeros(6 * len(nodes)) if want_u else None
        over = np.zeros(max(len(bonds), 1), np.int32) if want_over else None
        t = self._L.svxg_server_submit(self._h, int(structure), ptr(nodes), len(nodes), ptr(bonds), len(bonds),
                                       ptr(mats), ptr(f), ctypes.byref(opt) if opt is not None else None,
                                       float(rtol), int(maxit), float(fragility), ptr(u), ptr(over))
        _check(int(t) if t < 0 else 0)
        self._keep[int(t)] = (u, over)
        return int(t)

    def submit_repeat(self, structure: int, remove, f, rtol: float = 1e-6, maxit: int = -1,
                      fragility: float = 1.0, want_u: bool = True, want_over: bool = False,
                      nb: int | None = None) -> int:
        """A repeat of resident `structure`: remove bonds in place, warm solve, judge."""
        remove = np.ascontiguousarray(remove, dtype=np.int32)
        f = np.ascontiguousarray(f, dtype=np.float64)
        n = f.size // 6
        u = np.zeros(6 * n) if want_u else None
        over = np.zeros(max(int(nb or 0), 1), np.int32) if want_over else None
        t = self._L.svxg_server_submit_repeat(self._h, int(structure), ptr(remove), len(remove), ptr(f), n,
                                              float(rtol), int(maxit), float(fragility), ptr(u), ptr(over))
        _check(int(t) if t < 0 else 0)
        self._keep[int(t)] = (u, over)
        return int(t)

    def submit_device(self, nodes_dev: int, n: int, bonds_dev: int, nb: int, mats_dev: int, f_dev: int,
                      structure: int = -1, opt: StressOptions | None = None, rtol: float = 1e-6, maxit: int = -1,
                      fragility: float = 1.0, u_dev: int | None = None) -> int:
        """A new graph whose records, material table and load are in device memory (addresses that
        stay valid until waited for); u_dev: where the solution goes (device address) or None."""
        t = self._L.svxg_server_submit_device(self._h, int(structure), c_vp(nodes_dev), int(n), c_vp(bonds_dev),
                                              int(nb), c_vp(mats_dev), c_vp(f_dev),
                                              ctypes.byref(opt) if opt is not None else None, float(rtol),
                                              int(maxit), float(fragility), c_vp(u_dev) if u_dev else None, None)
        _check(int(t) if t < 0 else 0)
        self._keep[int(t)] = (None, None)
        return int(t)

    def submit_repeat_device(self, structure: int, remove, f_dev: int, n: int, rtol: float = 1e-6,
                             maxit: int = -1, fragility: float = 1.0, u_dev: int | None = None) -> int:
        """A repeat of resident `structure` with its load in device memory."""
        remove = np.ascontiguousarray(remove, dtype=np.int32)
        t = self._L.svxg_server_submit_repeat_device(self._h, int(structure), ptr(remove), len(remove), c_vp(f_dev),
                                                     int(n), float(rtol), int(maxit), float(fragility),
                                                     c_vp(u_dev) if u_dev else None, None)
        _check(int(t) if t < 0 else 0)
        self._keep[int(t)] = (None, None)
        return int(t)

    def set_batching(self, max_graphs: int = 16, max_graph_nodes: int = 20000, max_nodes: int = 65536):
        """New requests queued together run as one problem: at most max_graphs graphs (1: none) of at
        most max_graph_nodes nodes, max_nodes in all."""
        _check(self._L.svxg_server_set_batching(self._h, int(max_graphs), int(max_graph_nodes), int(max_nodes)))

    def hold(self, on: bool = True):
        """Slots take no new request while held (submissions queue); release to run them - together,
        batched."""
        _check(self._L.svxg_server_hold(self._h, int(bool(on))))

    def wait(self, ticket: int):
        """(RequestResult, u or None, failing bonds or None)."""
        r = RequestResult()
        _check(self._L.svxg_server_wait(self._h, int(ticket), ctypes.byref(r)))
        u, over = self._keep.pop(int(ticket), (None, None))
        if over is not None:
            over = over[:r.failing].copy()
        return r, u, over

    def drain(self):
        _check(self._L.svxg_server_drain(self._h))

    def stats(self) -> ServingStats:
        s = ServingStats()
        _check(self._L.svxg_server_stats(self._h, ctypes.byref(s)))
        return s

    def reset_stats(self):
        _check(self._L.svxg_server_reset_stats(self._h))

    def forget(self, structure: int):
        _check(self._L.svxg_server_forget(self._h, int(structure)))

    def batch_solve(self, graphs, mats, opt: StressOptions | None = None, rtol: float = 1e-6, maxit: int = -1,
                    fragility: float = 1.0, want_u: bool = True):
        """graphs: list of (nodes, bonds, f). Returns (results, list of u or None)."""
        gs = [_graph(*g) for g in graphs]
        k = len(gs)
        mats = np.ascontiguousarray(mats, dtype=MATERIAL_DTYPE)
        P = c_vp * max(k, 1)
        nodes = P(*[ptr(g[0]) for g in gs])
        bonds = P(*[ptr(g[1]) for g in gs])
        fs = P(*[ptr(g[2]) for g in gs])
        n = np.array([len(g[0]) for g in gs] or [0], np.int32)
        nb = np.array([len(g[1]) for g in gs] or [0], np.int32)
        us = [np.zeros(6 * len(g[0])) for g in gs] if want_u else None
        up = P(*[ptr(u) for u in us]) if want_u else None
        res = (RequestResult * max(k, 1))()
        _check(self._L.svxg_batch_solve(self._h, k, nodes, ptr(n), bonds, ptr(nb), ptr(mats), fs,
                                        ctypes.byref(opt) if opt is not None else None, float(rtol), int(maxit),
                                        float(fragility), up, None, res))
        return list(res)[:k], us


    def batch_piece_rounds(self, pieces, mats, options: PieceOptions | None = None, gf=None,
                           opt: StressOptions | None = None, want_lists: bool = False):
        """A substep's loose pieces: each (nodes, bonds, f) through its break rounds
        (svxg_piece_rounds), all in flight at once. Returns (PieceResults, RequestResults, u
        per piece, f per piece with the chips' loads moved, lists) with lists = [dict(broken,
        modes, chips)] when want_lists."""
        gs = [_graph(*g) for g in pieces]
        k = len(gs)
        mats = np.ascontiguousarray(mats, dtype=MATERIAL_DTYPE)
        gf = np.ascontiguousarray(default_fracture_energies() if gf is None else gf, dtype=np.float64)
        P = c_vp * max(k, 1)
        nodes = P(*[ptr(g[0]) for g in gs])
        bonds = P(*[ptr(g[1]) for g in gs])
        fs = [np.array(g[2], dtype=np.float64) for g in gs]
        us = [np.zeros(6 * len(g[0])) for g in gs]
        n = np.array([len(g[0]) for g in gs] or [0], np.int32)
        nb = np.array([len(g[1]) for g in gs] or [0], np.int32)
        br = [np.zeros(max(len(g[1]), 1), np.int32) for g in gs] if want_lists else None
        md = [np.zeros(max(len(g[1]), 1), np.uint8) for g in gs] if want_lists else None
        ch = [np.zeros(max(len(g[0]), 1), np.int32) for g in gs] if want_lists else None
        pres = (PieceResult * max(k, 1))()
        res = (RequestResult * max(k, 1))()
        o = PieceOptions() if options is None else options
        _check(self._L.svxg_batch_piece_rounds(
            self._h, k, nodes, ptr(n), bonds, ptr(nb), ptr(mats), ptr(gf), P(*[ptr(x) for x in fs]),
            P(*[ptr(x) for x in us]), ctypes.byref(opt) if opt is not None else None, ctypes.byref(o),
            P(*[ptr(x) for x in br]) if want_lists else None, P(*[ptr(x) for x in md]) if want_lists else None,
            P(*[ptr(x) for x in ch]) if want_lists else None, pres, res))
        lists = None
        if want_lists:
            lists = [dict(broken=br[i][:pres[i].bonds_broken].tolist(), modes=md[i][:pres[i].bonds_broken].tolist(),
                          chips=ch[i][:pres[i].chips].tolist()) for i in range(k)]
        return list(pres)[:k], list(res)[:k], us, fs, lists


__all__ = ["Server", "estimate_bytes", "RequestResult", "ServingStats", "SvxgError"]
