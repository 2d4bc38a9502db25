"""Interfaces (SECTION_DTYPE / FACE_DTYPE) of the section-geometry tests: the generator's towers,
city block and free piece, and hand-made interfaces that reach every branch of
SecAcc::finish_lattice / section_strengths (core/src/world/world_internal.hpp:133-232, :370-399):
L- and T-shaped faces (the principal-axis rotation), faces whose normals cancel (the centre line
as the normal), coincident centres (the +z fallback), supports along every axis and side, air on
either side of a face, full damage, unequal strength multipliers. Shared by test_oracle_pin.py,
test_oracle_golden.py (via golden/make_golden.py) and test_gpu_sections.py."""
from __future__ import annotations

import numpy as np

from opus_destruct_2_gb300 import synth
from opus_destruct_2_gb300.graph import FACE_DTYPE, SECTION_DTYPE, default_materials, empty_nodes, set_v3


def generated(kind: str):
    if kind == "tower":
        nodes, _, _, mats = synth.tower_graph(4, seed=5)
    elif kind == "city":
        nodes, _, _, mats = synth.city_graph(lots_x=2, lots_y=2, seed=4)
    else:
        nodes, _, _, mats = synth.piece_graph(400, free=True, seed=13)
    secs, faces = synth.last_sections()
    return nodes, secs, faces, mats


def voxel(x: int, y: int, z: int):
    """A voxel of the hand-made lattice (one value and damage per position, as a grid holds):
    air, a material (some anchored), damage (some full)."""
    h = (int(x) * 73856093) ^ (int(y) * 19349663) ^ (int(z) * 83492791)
    h = (h ^ (h >> 13)) & 0xFFFFFFFF
    if h % 7 == 0:
        return 0, 0
    v = (h % 126) + 1
    if (h >> 8) % 5 == 0:
        v |= 0x80
    r = (h >> 12) % 20
    dmg = 255 if r == 0 else (int((h >> 16) % 256) if r < 6 else 0)
    return v, dmg


def handmade(seed: int = 0, count: int = 400):
    """Random interfaces between random nodes, with the corner cases above planted."""
    rng = np.random.default_rng(seed)
    n = 64
    nodes = empty_nodes(n)
    c = rng.uniform(-2.0, 2.0, size=(n, 3))
    c[1] = c[0]  # (coincident centres)
    set_v3(nodes["c"], c)
    nodes["mass"] = 100.0
    secs = np.zeros(count, SECTION_DTYPE)
    faces = []
    for k in range(count):
        a = int(rng.integers(0, n))
        b = int(rng.integers(-1, n)) if k > 4 else [1, -1, 1, -1, 2][k]
        if k == 0:
            a = 0
        if b == a:
            b = -1
        nf = int(rng.integers(1, 40))
        base = rng.integers(-20, 20, size=3)
        fs = np.zeros(nf, FACE_DTYPE)
        shape = int(rng.integers(0, 4))
        for f in range(nf):
            ax = int(rng.integers(0, 3)) if shape == 0 else (f % 2 if shape == 1 else 2)
            if k in (0, 2):
                ax = 0
            off = rng.integers(-3, 4, size=3) if shape != 3 else np.array([f // 5, f % 5, 0])
            fs[f]["x"], fs[f]["y"], fs[f]["z"] = (base + off).tolist()
            fs[f]["axis"] = ax
            fs[f]["sign"] = 1 if (k in (0, 2) and f % 2) or rng.uniform() < 0.7 else -1
            if k in (0, 2):  # (normals that cancel: the centre line, or +z when the centres coincide)
                fs[f]["sign"] = 1 if f % 2 else -1
            lo_v = (fs[f]["x"], fs[f]["y"], fs[f]["z"])
            hi_v = list(lo_v)
            hi_v[ax] += 1
            fs[f]["vox_lo"], fs[f]["damage_lo"] = voxel(*lo_v)
            fs[f]["vox_hi"], fs[f]["damage_hi"] = voxel(*hi_v)
        if k in (0, 2) and nf % 2:
            fs = fs[:-1] if nf > 1 else fs
        s = secs[k]
        s["a"], s["b"] = a, b
        s["first_face"] = sum(len(x) for x in faces)
        s["faces"] = len(fs)
        s["axis"] = int(rng.integers(0, 3))
        s["sign"] = 1 if rng.uniform() < 0.5 else -1
        s["ma"], s["mb"] = int(rng.integers(0, 127)), int(rng.integers(0, 127))
        s["sectioned"] = 0 if k % 7 == 3 else 1
        s["h"] = float(rng.choice([0.5, 0.25, 1.0, 0.3]))
        s["strength_a"] = float(rng.uniform(0.5, 2.0))
        s["strength_b"] = 1e9 if b < 0 else float(rng.uniform(0.5, 2.0))
        faces.append(fs)
    return nodes, secs, np.concatenate(faces) if faces else np.zeros(0, FACE_DTYPE), default_materials()


def cases():
    out = {k: generated(k) for k in ("tower", "city", "piece")}
    out["handmade"] = handmade()
    return out


def lattices(seed: int = 0):
    """Four lattices: the identity (h 0.5), two placed by seeded rotations and offsets (h 0.25,
    0.5) and an identity of h 0.125."""
    from opus_destruct_2_gb300.graph import LATTICE_DTYPE
    rng = np.random.default_rng(seed)
    L = np.zeros(4, LATTICE_DTYPE)
    for g, (h, ident) in enumerate(((0.5, 1), (0.25, 0), (0.5, 0), (0.125, 1))):
        L[g]["h"] = h
        L[g]["identity"] = ident
        if ident:
            L[g]["R"] = np.eye(3).ravel()
            continue
        q = rng.normal(size=4)
        q /= np.linalg.norm(q)
        w, x, y, z = q
        R = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                      [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                      [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])
        L[g]["R"] = R.ravel()
        L[g]["off"] = rng.uniform(-3.0, 3.0, size=3)
    return L


def lattice_voxel(g: int, x: int, y: int, z: int):
    v, d = voxel(x + 1000 * g, y, z)
    return v, d


def general(seed: int = 1, count: int = 300, samples: int = 2):
    """Interfaces of placed lattices and junction samples between lattices: the general path
    (SecAcc::finish_general, section_strengths_general) and, for the sections without samples on
    identity lattices, the lattice path. Returns (nodes, secs, faces, junctions, lattices, mats)."""
    from opus_destruct_2_gb300.graph import JUNCTION_DTYPE
    rng = np.random.default_rng(seed)
    L = lattices(seed)
    n = 48
    nodes = empty_nodes(n)
    set_v3(nodes["c"], rng.uniform(-3.0, 3.0, size=(n, 3)))
    nodes["mass"] = 50.0
    secs = np.zeros(count, SECTION_DTYPE)
    faces, juncs = [], []
    nf_tot = nj_tot = 0
    for k in range(count):
        a = int(rng.integers(0, n))
        b = int(rng.integers(-1, n))
        if b == a:
            b = -1
        grid = int(rng.integers(0, 4))
        kind = k % 4  # 0: faces only, 1: faces + samples, 2: samples only, 3: faces only, placed or not
        nf = 0 if kind == 2 else int(rng.integers(1, 12))
        nj = 0 if kind in (0, 3) else int(rng.integers(1, 10))
        fs = np.zeros(nf, FACE_DTYPE)
        base = rng.integers(-10, 10, size=3)
        for f in range(nf):
            ax = int(rng.integers(0, 3))
            off = rng.integers(-2, 3, size=3)
            p = base + off
            fs[f]["x"], fs[f]["y"], fs[f]["z"] = p.tolist()
            fs[f]["axis"] = ax
            fs[f]["sign"] = 1 if rng.uniform() < 0.7 else -1
            hi = list(p)
            hi[ax] += 1
            fs[f]["vox_lo"], fs[f]["damage_lo"] = lattice_voxel(grid, *p)
            fs[f]["vox_hi"], fs[f]["damage_hi"] = lattice_voxel(grid, *hi)
        js = np.zeros(nj, JUNCTION_DTYPE)
        for q in range(nj):
            vg, og = int(rng.integers(0, 4)), int(rng.integers(0, 4))
            v = rng.integers(-8, 8, size=3)
            o = rng.integers(-8, 8, size=3)
            js[q]["v"], js[q]["o"] = v, o
            js[q]["vg"], js[q]["og"] = vg, og
            js[q]["face"] = int(rng.integers(0, 6))
            js[q]["sub"] = int(rng.integers(0, samples * samples))
            js[q]["kind"] = 1 if rng.uniform() < 0.2 else 0
            js[q]["sign"] = 1 if rng.uniform() < 0.6 else -1
            js[q]["weight"] = 0.5 if rng.uniform() < 0.5 else 1.0
            js[q]["vox_v"], js[q]["damage_v"] = lattice_voxel(vg, *v)
            js[q]["vox_o"], js[q]["damage_o"] = lattice_voxel(og, *o)
        s = secs[k]
        s["a"], s["b"] = a, b
        s["first_face"], s["faces"] = nf_tot, nf
        s["first_junction"], s["junctions"] = nj_tot, nj
        s["grid"] = grid
        s["axis"] = int(rng.integers(0, 3))
        s["sign"] = 1 if rng.uniform() < 0.5 else -1
        s["ma"], s["mb"] = int(rng.integers(0, 127)), int(rng.integers(0, 127))
        s["sectioned"] = 0 if k % 9 == 4 else 1
        s["h"] = float(L[grid]["h"])
        s["strength_a"] = float(rng.uniform(0.5, 2.0))
        s["strength_b"] = 1e9 if b < 0 else float(rng.uniform(0.5, 2.0))
        faces.append(fs)
        juncs.append(js)
        nf_tot += nf
        nj_tot += nj
    return nodes, secs, np.concatenate(faces), np.concatenate(juncs), L, default_materials()
