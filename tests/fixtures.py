"""Graph fixtures of the reference's own stress tests (tests/core/test_stress.cpp), as numpy records.

bond()       <- test_stress.cpp:14-32   a square section of side a between two nodes or a support
cantilever() <- test_stress.cpp:35-46   n cubes of side L along x from a support at x = 0
gravity()    <- test_stress.cpp:48-52
lattice()    <- test_stress.cpp:93-114, :204-227, :311-333   n^3 cubes on supports (optionally
                retiring the nodes at z >= keep_z, or leaving them out)
gravity_live() <- test_stress.cpp:229-234
"""
from __future__ import annotations

import math

import numpy as np

from opus_destruct_2_gb300.graph import CONCRETE, empty_bonds, empty_nodes, set_v3


def _cross(a, b):
    return (a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0])


def _dot(a, b):
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]


def bond_record(nodes, A, B, n, p, a):
    """One bond as the reference's fixture builds it."""
    s = empty_bonds(1)[0]
    s["a"], s["b"] = A, B
    s["ma"] = s["mb"] = CONCRETE
    t1 = (0.0, 1.0, 0.0) if abs(n[0]) > 0.5 else (1.0, 0.0, 0.0)
    t2 = _cross(n, t1)
    for name, v in (("n", n), ("t1", t1), ("t2", t2), ("p", p)):
        s[name]["x"], s[name]["y"], s[name]["z"] = v
    s["area"] = a * a
    s["s1"] = s["s2"] = a * a * a * a / 12.0
    s["c1"] = s["c2"] = 0.5 * a
    s["rmax"] = math.sqrt(0.5) * a
    ca = nodes[A]["c"]
    ca = (float(ca["x"]), float(ca["y"]), float(ca["z"]))
    s["la"] = abs(_dot((p[0] - ca[0], p[1] - ca[1], p[2] - ca[2]), n))
    if B >= 0:
        cb = nodes[B]["c"]
        cb = (float(cb["x"]), float(cb["y"]), float(cb["z"]))
        s["lb"] = abs(_dot((cb[0] - p[0], cb[1] - p[1], cb[2] - p[2]), n))
    else:
        s["lb"] = s["la"]
    s["faces"] = 16
    return s


def _bonds(lst):
    b = empty_bonds(len(lst))
    for i, s in enumerate(lst):
        b[i] = s
    return b


def cantilever(n: int, L: float, mass: float):
    nodes = empty_nodes(n)
    set_v3(nodes["c"], [((i + 0.5) * L, 0.0, 0.0) for i in range(n)])
    nodes["mass"] = mass
    lst = [bond_record(nodes, 0, -1, (-1.0, 0.0, 0.0), (0.0, 0.0, 0.0), L)]
    for i in range(n - 1):
        lst.append(bond_record(nodes, i, i + 1, (1.0, 0.0, 0.0), ((i + 1) * L, 0.0, 0.0), L))
    return nodes, _bonds(lst)


def add_bond(nodes, bonds, A, B, n, p, a):
    out = empty_bonds(len(bonds) + 1)  # (np.concatenate would pack the padded record layout)
    out[:-1] = bonds
    out[-1] = bond_record(nodes, A, B, n, p, a)
    return out


def gravity(nodes):
    f = np.zeros(6 * len(nodes))
    f[2::6] = -9.81 * nodes["mass"]
    return f


def gravity_live(nodes):
    f = gravity(nodes)
    f[2::6][nodes["gone"] != 0] = 0.0
    return f


def lattice(n: int, L: float = 0.4, keep_z: int | None = None, retire_top: bool = False, mass: float = 400.0):
    keep_z = n if keep_z is None else keep_z
    nz = n if retire_top else keep_z
    idx = lambda x, y, z: (x * n + y) * nz + z  # noqa: E731
    nodes = empty_nodes(n * n * nz)
    c = np.zeros((n * n * nz, 3))
    for x in range(n):
        for y in range(n):
            for z in range(nz):
                c[idx(x, y, z)] = ((x + 0.5) * L, (y + 0.5) * L, (z + 0.5) * L)
    set_v3(nodes["c"], c)
    nodes["mass"] = mass
    for x in range(n):
        for y in range(n):
            for z in range(nz):
                nodes[idx(x, y, z)]["gone"] = 1 if z >= keep_z else 0
    lst = []
    for x in range(n):
        for y in range(n):
            for z in range(nz):
                cc = c[idx(x, y, z)]
                if z == 0:
                    lst.append(bond_record(nodes, idx(x, y, z), -1, (0.0, 0.0, -1.0),
                                           (cc[0], cc[1], cc[2] - 0.5 * L), L))
                if x + 1 < n:
                    lst.append(bond_record(nodes, idx(x, y, z), idx(x + 1, y, z), (1.0, 0.0, 0.0),
                                           (cc[0] + 0.5 * L, cc[1], cc[2]), L))
                if y + 1 < n:
                    lst.append(bond_record(nodes, idx(x, y, z), idx(x, y + 1, z), (0.0, 1.0, 0.0),
                                           (cc[0], cc[1] + 0.5 * L, cc[2]), L))
                if z + 1 < nz:
                    lst.append(bond_record(nodes, idx(x, y, z), idx(x, y, z + 1), (0.0, 0.0, 1.0),
                                           (cc[0], cc[1], cc[2] + 0.5 * L), L))
    return nodes, _bonds(lst)


def same_records(a, b) -> bool:
    """Field by field, bit for bit (the padding between fields is not compared: numpy does not
    keep it through save/load)."""
    if a.dtype.names != b.dtype.names or len(a) != len(b):
        return False
    return all(np.ascontiguousarray(a[k]).tobytes() == np.ascontiguousarray(b[k]).tobytes() for k in a.dtype.names)
