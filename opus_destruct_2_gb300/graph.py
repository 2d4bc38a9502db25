"""Host-side records of the stress solve: numpy layouts of the C-ABI structs in ``include/svxg_types.h``.

A fragment graph is two numpy structured arrays (``NODE_DTYPE``, ``BOND_DTYPE``) and a material
table (``MATERIAL_DTYPE``, ``SVXG_MAX_MATERIALS`` entries). They are the images of the
reference's ``svx::SNode`` / ``svx::SBond`` (core/include/svx/stress/stress.hpp:21-51) and the
solve's fields of ``svx::Material`` (core/include/svx/material/material.hpp:47-57), laid out
byte for byte like the C structs so a pointer to the array is the C-ABI argument.
"""
from __future__ import annotations

import ctypes

import numpy as np

SVXG_MAX_MATERIALS = 127

V3 = [("x", "<f8"), ("y", "<f8"), ("z", "<f8")]

NODE_DTYPE = np.dtype(
    {
        "names": ["c", "mass", "fixed", "gone"],
        "formats": [np.dtype(V3), "<f8", "u1", "u1"],
        "offsets": [0, 24, 32, 33],
        "itemsize": 40,
    }
)

BOND_DTYPE = np.dtype(
    {
        "names": ["a", "b", "broken", "in_k", "ma", "mb", "sectioned", "n", "t1", "t2", "area", "p", "s1", "s2",
                  "c1", "c2", "rmax", "la", "lb", "strength", "ft", "fb", "fc", "coh", "mu", "faces", "tag"],
        "formats": ["<i4", "<i4", "u1", "u1", "u1", "u1", "u1", np.dtype(V3), np.dtype(V3), np.dtype(V3), "<f8",
                    np.dtype(V3), "<f8", "<f8", "<f8", "<f8", "<f8", "<f8", "<f8", "<f8", "<f4", "<f4", "<f4",
                    "<f4", "<f4", "<i4", "<i4"],
        "offsets": [0, 4, 8, 9, 10, 11, 12, 16, 40, 64, 88, 96, 120, 128, 136, 144, 152, 160, 168, 176, 184, 188,
                    192, 196, 200, 204, 208],
        "itemsize": 216,
    }
)

MATERIAL_DTYPE = np.dtype(
    [("E", "<f8"), ("G", "<f8"), ("rho", "<f8"), ("ft", "<f8"), ("fb", "<f8"), ("fc", "<f8"),
     ("cohesion", "<f8"), ("friction", "<f8")]
)

# svxg_section / svxg_face / svxg_lattice / svxg_junction (svxg_types.h): a bond's interface of
# voxel faces and junction samples, before it is a bond
SECTION_DTYPE = np.dtype(
    [("a", "<i4"), ("b", "<i4"), ("first_face", "<i8"), ("faces", "<i4"), ("axis", "u1"), ("sign", "i1"),
     ("ma", "u1"), ("mb", "u1"), ("sectioned", "u1"), ("pad", "u1"), ("grid", "<u2"), ("junctions", "<i4"),
     ("first_junction", "<i8"), ("h", "<f8"), ("strength_a", "<f8"), ("strength_b", "<f8")])
FACE_DTYPE = np.dtype(
    [("x", "<i4"), ("y", "<i4"), ("z", "<i4"), ("axis", "u1"), ("sign", "i1"), ("vox_lo", "u1"), ("vox_hi", "u1"),
     ("damage_lo", "u1"), ("damage_hi", "u1"), ("pad", "u1", (2,))])
LATTICE_DTYPE = np.dtype([("off", "<f8", (3,)), ("R", "<f8", (9,)), ("h", "<f8"), ("identity", "u1"),
                          ("pad", "u1", (7,))])
JUNCTION_DTYPE = np.dtype(
    [("v", "<i4", (3,)), ("o", "<i4", (3,)), ("vg", "<u2"), ("og", "<u2"), ("face", "u1"), ("sub", "u1"),
     ("kind", "u1"), ("sign", "i1"), ("weight", "<f4"), ("vox_v", "u1"), ("vox_o", "u1"), ("damage_v", "u1"),
     ("damage_o", "u1")])
assert (SECTION_DTYPE.itemsize, FACE_DTYPE.itemsize, LATTICE_DTYPE.itemsize, JUNCTION_DTYPE.itemsize) == \
    (64, 20, 112, 40)

LOAD_DTYPE = np.dtype([("N", "<f8"), ("V1", "<f8"), ("V2", "<f8"), ("T", "<f8"), ("M1", "<f8"), ("M2", "<f8")])

# Material ids of the standard presets (svx::MaterialId, material.hpp:26-43).
RC, CONCRETE, STEEL, MASONRY, SOIL, ROCK, BEDROCK, WOOD, STONE, GLASS, REBAR, STEEL_SECTION = range(12)

# The standard presets' solve fields, in id order (the reference's preset table,
# core/src/material/material.cpp:72-98): E, G, rho, ft, fb, fc, cohesion, friction.
_PRESETS = [
    (30e9, 12.5e9, 2400, 1.2e6, 3.5e6, 30e6, 1.6e6, 0.7),     # rc
    (28e9, 11.5e9, 2300, 0.8e6, 1.2e6, 25e6, 1.2e6, 0.7),     # concrete
    (200e9, 80e9, 7850, 180e6, 180e6, 200e6, 100e6, 0.35),    # steel
    (10e9, 4e9, 1900, 0.15e6, 0.3e6, 8e6, 0.35e6, 0.75),      # masonry
    (0.1e9, 0.04e9, 1700, 0.01e6, 0.01e6, 0.4e6, 0.03e6, 0.55),  # soil
    (40e9, 16e9, 2600, 2.5e6, 3.0e6, 80e6, 4e6, 0.8),         # rock
    (60e9, 25e9, 2800, 10e6, 10e6, 200e6, 15e6, 0.8),         # bedrock
    (11e9, 0.7e9, 550, 1.2e6, 8e6, 20e6, 2e6, 0.5),           # wood
    (30e9, 12e9, 2600, 0.25e6, 0.4e6, 40e6, 0.5e6, 0.7),      # stone
    (70e9, 29e9, 2500, 3e6, 4e6, 100e6, 3e6, 0.4),            # glass
    (34e9, 13e9, 2550, 9e6, 10e6, 35e6, 4e6, 0.7),            # rebar
    (26e9, 10e9, 980, 44e6, 44e6, 40e6, 25e6, 0.35),          # steel_section
]


def default_materials() -> np.ndarray:
    """The standard presets; ids never registered resolve to id 0's properties."""
    t = np.zeros(SVXG_MAX_MATERIALS, dtype=MATERIAL_DTYPE)
    for i in range(SVXG_MAX_MATERIALS):
        t[i] = _PRESETS[i] if i < len(_PRESETS) else _PRESETS[0]
    return t


def register_material(table: np.ndarray, props: tuple, used: set[int]) -> int:
    """Take the next free id after the presets (svx::MaterialTable::add, material.cpp:106-115)."""
    for i in range(len(_PRESETS), SVXG_MAX_MATERIALS):
        if i not in used:
            table[i] = props
            used.add(i)
            return i
    raise ValueError("material table full")


def empty_nodes(n: int) -> np.ndarray:
    return np.zeros(n, dtype=NODE_DTYPE)


def empty_bonds(n: int) -> np.ndarray:
    b = np.zeros(n, dtype=BOND_DTYPE)
    b["a"] = -1
    b["b"] = -1
    b["ma"] = CONCRETE
    b["mb"] = CONCRETE
    b["n"]["z"] = 1.0
    b["t1"]["x"] = 1.0
    b["t2"]["y"] = 1.0
    b["strength"] = 1.0
    b["tag"] = -1
    return b


def v3(a) -> np.ndarray:
    """(k, 3) float64 view of a V3 field."""
    return np.stack([a["x"], a["y"], a["z"]], axis=-1)


def set_v3(field, arr) -> None:
    arr = np.asarray(arr, dtype=np.float64)
    field["x"] = arr[..., 0]
    field["y"] = arr[..., 1]
    field["z"] = arr[..., 2]


class AmgOptions(ctypes.Structure):
    _fields_ = [("coarse_max", ctypes.c_int32), ("smoothed", ctypes.c_int32), ("strength", ctypes.c_double),
                ("coarse_scale", ctypes.c_double), ("max_levels", ctypes.c_int32), ("gamma", ctypes.c_int32),
                ("sgs", ctypes.c_int32), ("sweeps", ctypes.c_int32), ("cheb_degree", ctypes.c_int32),
                ("dense_work_per_unknown", ctypes.c_int32), ("coarsen_dense", ctypes.c_int32),
                ("reaggregate", ctypes.c_int32)]


# StressOptions.precision (svxg_types.h): FP64 (bit-exact setup); the mixed-precision policy (fast
# multigrid build, FP32 V-cycle, FP64 Krylov vectors); that with FP32 inner sequences
PRECISION_FP64, PRECISION_MIXED, PRECISION_MIXED_ALL = 0, 1, 2


class StressOptions(ctypes.Structure):
    """svx::StressOptions (stress.hpp:68-72) plus the arithmetic of the solve."""
    _fields_ = [("rtol", ctypes.c_double), ("amg", AmgOptions), ("amg_min_nodes", ctypes.c_int32),
                ("precision", ctypes.c_int32)]

    def __init__(self, **kw):
        super().__init__()
        self.rtol = 2e-3
        a = self.amg
        a.coarse_max, a.smoothed, a.strength, a.coarse_scale = 48, 1, 0.1, 0.6
        a.max_levels, a.gamma, a.sgs, a.sweeps, a.cheb_degree = 16, 1, 1, 1, 3
        a.dense_work_per_unknown, a.coarsen_dense, a.reaggregate = 0, 1, 1
        self.amg_min_nodes = 160
        self.precision = 0
        for k, v in kw.items():
            if hasattr(a, k) and k not in ("rtol",):
                setattr(a, k, v)
            else:
                setattr(self, k, v)


class PcgResult(ctypes.Structure):
    """svx::PcgResult (amg.hpp:120-125)."""
    _fields_ = [("iters", ctypes.c_int32), ("converged", ctypes.c_int32), ("breakdown", ctypes.c_int32),
                ("pad", ctypes.c_int32), ("rel_res", ctypes.c_double)]

    def __repr__(self) -> str:
        return (f"PcgResult(iters={self.iters}, rel_res={self.rel_res:.3e}, converged={bool(self.converged)}, "
                f"breakdown={bool(self.breakdown)})")


class CascadeOptions(ctypes.Structure):
    """svxg_cascade_options: the judge's break rounds of one structure (World::Impl::judge,
    core/src/world/world.cpp:1162-1277); defaults from WorldConfig/WorldParams (world.hpp)."""
    _fields_ = [("rtol", ctypes.c_double), ("fragility", ctypes.c_double), ("dif", ctypes.c_double),
                ("break_band", ctypes.c_double), ("max_breaks_per_round", ctypes.c_int32),
                ("max_rounds", ctypes.c_int32), ("maxit", ctypes.c_int32), ("solve_restarts", ctypes.c_int32),
                ("rebuild_after", ctypes.c_int32), ("shock", ctypes.c_int32), ("detach", ctypes.c_int32),
                ("pad", ctypes.c_int32)]

    def __init__(self, **kw):
        super().__init__()
        self.rtol, self.fragility, self.dif, self.break_band = 3e-3, 1.0, 1.5, 0.85
        self.max_breaks_per_round, self.max_rounds, self.maxit = 256, 400, 120
        self.solve_restarts, self.rebuild_after, self.shock, self.detach = 60, 60, 0, 1
        for k, v in kw.items():
            setattr(self, k, v)


# svxg_cascade_result.status
CASCADE_SETTLED, CASCADE_MAX_ROUNDS, CASCADE_ABANDONED, CASCADE_BREAKDOWN, CASCADE_SINGULAR = 0, 1, 2, 3, 4


class CascadeResult(ctypes.Structure):
    """svxg_cascade_result."""
    _fields_ = [("status", ctypes.c_int32), ("rounds", ctypes.c_int32), ("bonds_broken", ctypes.c_int32),
                ("nodes_retired", ctypes.c_int32), ("solves", ctypes.c_int32), ("restarts", ctypes.c_int32),
                ("pcg_iters", ctypes.c_int64), ("max_utilization", ctypes.c_double), ("rel_res", ctypes.c_double)]

    def __repr__(self) -> str:
        return (f"CascadeResult(status={self.status}, rounds={self.rounds}, broken={self.bonds_broken}, "
                f"retired={self.nodes_retired}, solves={self.solves}, restarts={self.restarts}, "
                f"iters={self.pcg_iters}, max_phi={self.max_utilization:.4g}, rel_res={self.rel_res:.3e})")


class PieceOptions(ctypes.Structure):
    """svxg_piece_options: a loose piece's break rounds within a substep (World::Impl::body_stress_run,
    core/src/world/world_pieces.cpp:614-808); defaults from WorldConfig (world.hpp)."""
    _fields_ = [("rtol", ctypes.c_double), ("fragility", ctypes.c_double), ("break_band", ctypes.c_double),
                ("round_fraction", ctypes.c_double), ("energy", ctypes.c_double), ("fracture_energy", ctypes.c_double),
                ("crush_energy", ctypes.c_double), ("chip_fraction", ctypes.c_double), ("maxit", ctypes.c_int32),
                ("rounds", ctypes.c_int32), ("max_breaks_per_round", ctypes.c_int32), ("pad", ctypes.c_int32)]

    def __init__(self, **kw):
        super().__init__()
        self.rtol, self.fragility, self.break_band, self.round_fraction = 1e-2, 1.0, 0.85, 0.25
        self.energy, self.fracture_energy, self.crush_energy, self.chip_fraction = -1.0, 1.0, 20.0, 0.04
        self.maxit, self.rounds, self.max_breaks_per_round = 60, 8, 256
        for k, v in kw.items():
            setattr(self, k, v)


# svxg_piece_result.status
(PIECE_SETTLED, PIECE_ENERGY, PIECE_APART, PIECE_LAST_ROUND, PIECE_SOLVE_FAILED, PIECE_NO_PIN,
 PIECE_SINGULAR) = range(7)


class PieceResult(ctypes.Structure):
    """svxg_piece_result."""
    _fields_ = [("status", ctypes.c_int32), ("checks", ctypes.c_int32), ("bonds_broken", ctypes.c_int32),
                ("chips", ctypes.c_int32), ("pcg_iters", ctypes.c_int32), ("rebuilt", ctypes.c_int32),
                ("spent", ctypes.c_double), ("first_max_utilization", ctypes.c_double),
                ("max_utilization", ctypes.c_double)]

    def __repr__(self) -> str:
        return (f"PieceResult(status={self.status}, checks={self.checks}, broken={self.bonds_broken}, "
                f"chips={self.chips}, iters={self.pcg_iters}, spent={self.spent:.4g}, "
                f"max_phi={self.max_utilization:.4g})")


def default_fracture_energies() -> np.ndarray:
    """Gf (J/m^2) per material id, SVXG_MAX_MATERIALS entries, as the reference's preset table
    holds them (MaterialTable::reset, core/src/material/material.cpp:72-93); ids never registered
    resolve to id 0's, as the table's lookup does (material.hpp:97-100)."""
    gf = np.full(127, 2000.0)
    gf[:12] = [2000.0, 400.0, 1e6, 120.0, 20.0, 600.0, 2000.0, 6000.0, 120.0, 4.0, 50000.0, 2e5]
    return gf


def ptr(a: np.ndarray | None):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


class V3(ctypes.Structure):
    """svxg_v3 by value."""
    _fields_ = [("x", ctypes.c_double), ("y", ctypes.c_double), ("z", ctypes.c_double)]


class BodyState(ctypes.Structure):
    """svxg_body_state: a moving piece's rigid-body state (x, q = (x, y, z, w), com in the shape
    frame, angular velocity w, body-frame inertia and inverse, 1 / mass, gravity)."""
    _fields_ = [("x", ctypes.c_double * 3), ("q", ctypes.c_double * 4), ("com", ctypes.c_double * 3),
                ("w", ctypes.c_double * 3), ("inertia", ctypes.c_double * 9), ("inv_inertia", ctypes.c_double * 9),
                ("inv_mass", ctypes.c_double), ("gravity", ctypes.c_double)]


POINT_FORCE_DTYPE = np.dtype([("F", np.float64, 3), ("p", np.float64, 3), ("node", np.int32), ("pad", np.int32)],
                             align=True)


class PhaseTime(ctypes.Structure):
    """svxg_phase_time: a setup or solve phase's label and its milliseconds since the previous one."""
    _fields_ = [("label", ctypes.c_char * 48), ("ms", ctypes.c_double)]
