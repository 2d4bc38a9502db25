"""The C ABI without a GPU: the library builds and loads, exports every function include/*.h
declares, the record layouts match the headers, and the host-side checks reject bad calls."""
import ctypes
import glob
import os
import re

import numpy as np
import pytest

from opus_destruct_2_gb300 import Info, build, load_library
from opus_destruct_2_gb300.graph import BOND_DTYPE, MATERIAL_DTYPE, NODE_DTYPE, PcgResult, StressOptions

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*(svxg_[a-z_0-9]+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return sorted(n for n in names if not n.startswith("svxg_default_"))  # (static inline)


def test_library_exports_every_declared_function():
    L = load_library()
    names = declared_functions()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_record_layouts():
    assert NODE_DTYPE.itemsize == 40 and BOND_DTYPE.itemsize == 216 and MATERIAL_DTYPE.itemsize == 64
    assert ctypes.sizeof(StressOptions) == 72 and ctypes.sizeof(PcgResult) == 24
    assert ctypes.sizeof(Info) == 16 + 64 + 256 + 40 + 8 + 8 + 8 + 8


def test_built_for_sm_103a():
    assert "arch=compute_103a,code=sm_103a" in " ".join(build.ARCH)
    assert os.path.exists(os.path.join(build.LIBDIR, build.CUDA_LIB))


def test_host_checks_without_a_device():
    L = load_library()
    if L.svxg_device_count() > 0:
        pytest.skip("a GPU is present: covered by the gpu tests")
    h = ctypes.c_void_p()
    assert L.svxg_problem_create(ctypes.byref(h), 0) == -6  # SVXG_ERR_NODEVICE
    assert L.svxg_assemble(None, None, None) == -1
    assert L.svxg_set_graph(None, None, 0, None, 0, None) == -1
    assert b"null problem" in L.svxg_last_error()


def test_argument_checks_run_before_any_device_work():
    """The new entry points reject bad arguments on the host (no GPU needed): null problems,
    sections whose faces, samples or lattices lie outside the arrays, bad sample counts."""
    import numpy as np

    from opus_destruct_2_gb300.graph import (FACE_DTYPE, JUNCTION_DTYPE, LATTICE_DTYPE, SECTION_DTYPE,
                                             default_materials, empty_nodes, ptr)
    L = load_library()
    assert L.svxg_cascade(None, None, None, None, None, None, None, None, None, 0, None, 0, None) == -1
    assert L.svxg_piece_rounds(None, None, None, None, None, None, None, None, 0, None, 0, None) == -1
    assert L.svxg_remove_bonds(None, None, 0) == -1
    nodes = empty_nodes(2)
    mats = default_materials()
    secs = np.zeros(1, SECTION_DTYPE)
    secs[0]["a"], secs[0]["b"], secs[0]["faces"], secs[0]["h"] = 0, 1, 2, 0.5
    faces = np.zeros(1, FACE_DTYPE)  # (the section names two faces: one too many)
    out = np.zeros(1, dtype=np.dtype([("x", "u1", (216,))]))

    def call(secs_, faces_, js=None, lats=None, samples=2):
        return L.svxg_build_bonds(ptr(nodes), 2, ptr(secs_), len(secs_), ptr(faces_), len(faces_), ptr(js),
                                  0 if js is None else len(js), ptr(lats), 0 if lats is None else len(lats),
                                  samples, ptr(mats), ptr(out))

    assert call(secs, faces) == -1
    secs[0]["faces"] = 1
    assert call(secs, faces, samples=0) == -1
    secs[0]["junctions"] = 1  # (samples without a lattice table)
    js = np.zeros(1, JUNCTION_DTYPE)
    assert call(secs, faces, js=js) == -1
    lats = np.zeros(1, LATTICE_DTYPE)
    js[0]["vg"] = 3  # (a lattice that is not there)
    assert call(secs, faces, js=js, lats=lats) == -1
    secs[0]["junctions"], secs[0]["b"] = 0, 5  # (a node that is not there)
    assert call(secs, faces) == -1
