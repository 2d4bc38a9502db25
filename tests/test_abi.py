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
    assert ctypes.sizeof(Info) == 16 + 64 + 256 + 40 + 8 + 8


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
