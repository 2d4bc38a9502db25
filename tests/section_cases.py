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
