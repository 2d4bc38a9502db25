"""Seeded synthetic workloads of the stress solve (wrapper of csrc/synth.cpp).

Graph generators:
  tower_graph  - one storey-frame tower (the 10-storey 8 x 8 m tower of 0.5 m voxels: ~2k fragments)
  city_graph   - a city block of towers of 5-40 storeys in four jittered materials (~200k fragments)
  piece_graph  - a loose piece: a random connected voxel cluster, free (inertial relief, pinned
                 reference node) or ground-supported, with one impact force
  batch_graphs - many pieces of log-normal size (the batched workload)
Each returns (nodes, bonds, f, mats): numpy records (graph.NODE_DTYPE / BOND_DTYPE), the load
vector (6 per node) and the material table.
"""
from __future__ import annotations

import ctypes
import math
import os

import numpy as np

from . import build as _build
from .graph import (BOND_DTYPE, CONCRETE, FACE_DTYPE, MASONRY, NODE_DTYPE, RC, SECTION_DTYPE, STEEL, WOOD,
                    default_materials, ptr, register_material)


class _Mat(ctypes.Structure):
    _fields_ = [("rho", ctypes.c_double), ("ft", ctypes.c_double), ("fb", ctypes.c_double), ("fc", ctypes.c_double),
                ("coh", ctypes.c_double), ("mu", ctypes.c_double), ("id", ctypes.c_int32), ("pad", ctypes.c_int32)]


_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        L = ctypes.CDLL(_build.synth_library())
        vp = ctypes.c_void_p
        L.svxs_tower.restype = vp
        L.svxs_tower.argtypes = [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_double, ctypes.c_double,
                                 vp, ctypes.c_uint64]
        L.svxs_city.restype = vp
        L.svxs_city.argtypes = [ctypes.c_int32] * 6 + [vp, ctypes.c_int32, ctypes.c_uint64]
        L.svxs_piece.restype = vp
        L.svxs_piece.argtypes = [ctypes.c_int64, ctypes.c_int32, ctypes.c_double, vp, ctypes.c_uint64]
        L.svxs_num_nodes.argtypes = [vp]
        L.svxs_num_bonds.argtypes = [vp]
        L.svxs_get.argtypes = [vp, vp, vp, vp]
        L.svxs_free.argtypes = [vp]
        L.svxs_num_sections.argtypes = [vp]
        L.svxs_num_faces.restype = ctypes.c_int64
        L.svxs_num_faces.argtypes = [vp]
        L.svxs_get_sections.argtypes = [vp, vp, vp]
        _lib = L
    return _lib


def _mat(table: np.ndarray, mid: int) -> _Mat:
    m = table[mid]
    return _Mat(float(m["rho"]), float(m["ft"]), float(m["fb"]), float(m["fc"]), float(m["cohesion"]),
                float(m["friction"]), mid, 0)


_last_sections = None


def _take(h):
    L = lib()
    n, nb = L.svxs_num_nodes(h), L.svxs_num_bonds(h)
    nodes = np.zeros(n, NODE_DTYPE)
    bonds = np.zeros(nb, BOND_DTYPE)
    f = np.zeros(6 * n)
    L.svxs_get(h, ptr(nodes), ptr(bonds), ptr(f))
    global _last_sections
    secs = np.zeros(L.svxs_num_sections(h), SECTION_DTYPE)
    faces = np.zeros(L.svxs_num_faces(h), FACE_DTYPE)
    L.svxs_get_sections(h, ptr(secs), ptr(faces))
    _last_sections = (secs, faces)
    L.svxs_free(h)
    return nodes, bonds, f


def last_sections():
    """The interfaces (SECTION_DTYPE, FACE_DTYPE) of the graph the last generator call made: its
    bonds' voxel faces, one section per bond in the same order."""
    return _last_sections


def tower_graph(storeys: int = 10, wx: int = 16, wy: int = 16, seed: int = 1, material: int = RC):
    """A storey-frame tower (default: 10 storeys, 8 x 8 m plan, concrete E = 30 GPa, nu = 0.2)."""
    mats = default_materials()
    m = _mat(mats, material)
    h = lib().svxs_tower(wx, wy, storeys, 0.0, 0.0, ctypes.byref(m), seed)
    nodes, bonds, f = _take(h)
    return nodes, bonds, f, mats


def jittered_materials(seed: int = 7, per_base: int = 28):
    """Concrete 30 GPa, steel 200 GPa, masonry 10 GPa, wood 11 GPa, each in `per_base` variants
    with stiffness (and strength) jittered by a uniform +-20%, registered as materials 12..."""
    rng = np.random.default_rng(seed)
    mats = default_materials()
    used: set[int] = set()
    ids = []
    bases = [(RC, 30e9), (STEEL, 200e9), (MASONRY, 10e9), (WOOD, 11e9)]
    for base, E in bases:
        b = mats[base]
        for _ in range(per_base):
            j = rng.uniform(0.8, 1.2)
            Ej = E * j
            G = Ej / (2.0 * 1.2) if base in (RC, MASONRY) else float(b["G"]) * j
            props = (Ej, G, float(b["rho"]), float(b["ft"]) * j, float(b["fb"]) * j, float(b["fc"]) * j,
                     float(b["cohesion"]) * j, float(b["friction"]))
            ids.append(register_material(mats, props, used))
    return mats, ids


def city_graph(lots_x: int = 7, lots_y: int = 7, smin: int = 5, smax: int = 40, wmin: int = 12, wmax: int = 20,
               seed: int = 2):
    """A city block of seeded random towers in four jittered materials."""
    mats, ids = jittered_materials(seed + 100)
    arr = (_Mat * len(ids))(*[_mat(mats, i) for i in ids])
    h = lib().svxs_city(lots_x, lots_y, smin, smax, wmin, wmax, arr, len(ids), seed)
    nodes, bonds, f = _take(h)
    return nodes, bonds, f, mats


def piece_graph(target_nodes: int, free: bool = True, seed: int = 1, impact: float | None = None,
                material: int = CONCRETE):
    """A loose piece of about `target_nodes` fragments (about 11 voxels each) with one impact
    force (default: log-uniform 1e4-1e6 N)."""
    rng = np.random.default_rng(seed)
    if impact is None:
        impact = float(10 ** rng.uniform(4.0, 6.0))
    mats = default_materials()
    m = _mat(mats, material)
    voxels = max(8, int(target_nodes * 11))
    h = lib().svxs_piece(voxels, int(free), impact, ctypes.byref(m), seed)
    nodes, bonds, f = _take(h)
    return nodes, bonds, f, mats


def lognormal_sizes(count: int, median: float, lo: int, hi: int, sigma: float = 1.0, seed: int = 0):
    rng = np.random.default_rng(seed)
    s = np.exp(rng.normal(math.log(median), sigma, size=count))
    return np.clip(np.round(s), lo, hi).astype(np.int64)


def batch_graphs(count: int = 512, median: int = 300, lo: int = 10, hi: int = 20000, seed: int = 3):
    """The batched workload: pieces of log-normal size, half free and half ground-supported."""
    sizes = lognormal_sizes(count, median, lo, hi, seed=seed)
    rng = np.random.default_rng(seed + 1)
    out = []
    for k, s in enumerate(sizes):
        out.append(piece_graph(int(s), free=bool(rng.integers(0, 2)), seed=seed * 100003 + k))
    return out
