"""Build recipe of the oracle (TEST INFRASTRUCTURE: the checker, never the product).

Two libraries:

* ``oracle/_build/libsvxo.so`` - the C restatement of the reference's stress solve
  (``oracle/svx_oracle.c``). Built on every machine (plain gcc + OpenMP).
* ``oracle/_ref/libsvxref.so`` - the reference's own solve sources compiled where they lie
  (core/src/solve/amg.cpp, core/src/stress/stress.cpp, core/src/material/material.cpp,
  core/src/base/parallel.cpp under the reference tree) with its own flags (Release,
  ``-ffp-contract=off -fno-fast-math -fno-exceptions -fno-rtti``, CMakeLists.txt:17, :53), plus
  ``oracle/ref_shim.cpp``. Built only where the reference tree exists (``SVX_REFERENCE_TREE``, or a
  checkout named ``reference`` beside this repository); nothing is copied.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
# The reference tree: SVX_REFERENCE_TREE, else a checkout named `reference` beside this repository
# (absent on machines that only run the prebuilt checker: then only the C restatement is built).
REFERENCE = os.environ.get("SVX_REFERENCE_TREE") or os.path.join(os.path.dirname(ROOT), "reference")
REF_SOURCES = [
    "core/src/solve/amg.cpp",
    "core/src/stress/stress.cpp",
    "core/src/material/material.cpp",
    "core/src/base/parallel.cpp",
]
PORT_LIB = os.path.join(HERE, "_build", "libsvxo.so")
REF_LIB = os.path.join(HERE, "_ref", "libsvxref.so")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        raise RuntimeError(f"oracle build failed: {cmd[0]} exit {r.returncode}")


def _stale(out: str, deps: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build_port(force: bool = False) -> str:
    """The C restatement (runs on the GPU machine's host cores too)."""
    src = os.path.join(HERE, "svx_oracle.c")
    deps = [src, os.path.join(HERE, "svx_oracle.h"), os.path.join(ROOT, "include", "svxg_types.h")]
    if force or _stale(PORT_LIB, deps):
        os.makedirs(os.path.dirname(PORT_LIB), exist_ok=True)
        _run(["gcc", "-std=c11", "-O3", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC", "-shared",
              "-I", os.path.join(ROOT, "include"), src, "-o", PORT_LIB, "-lm"])
    return PORT_LIB


def reference_available() -> bool:
    return all(os.path.exists(os.path.join(REFERENCE, s)) for s in REF_SOURCES)


def build_reference(force: bool = False) -> str | None:
    """The reference's own solve sources + the shim (only where the reference tree exists)."""
    if not reference_available():
        return None
    srcs = [os.path.join(REFERENCE, s) for s in REF_SOURCES] + [os.path.join(HERE, "ref_shim.cpp")]
    objdir = os.path.join(HERE, "_ref", "obj")
    os.makedirs(objdir, exist_ok=True)
    flags = ["g++", "-std=c++20", "-O3", "-DNDEBUG", "-ffp-contract=off", "-fno-fast-math", "-fno-exceptions",
             "-fno-rtti", "-fPIC", "-pthread", "-I", os.path.join(REFERENCE, "core", "include"),
             "-I", os.path.join(REFERENCE, "core", "src", "world"),
             "-I", os.path.join(ROOT, "include")]
    objs = []
    jobs = []
    for s in srcs:
        o = os.path.join(objdir, os.path.basename(s) + ".o")
        objs.append(o)
        if force or _stale(o, [s, os.path.join(ROOT, "include", "svxg_types.h")]):
            jobs.append(flags + ["-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        list(ex.map(_run, jobs))
    if force or jobs or not os.path.exists(REF_LIB):
        _run(["g++", "-shared", "-pthread", "-o", REF_LIB] + objs)
    return REF_LIB


if __name__ == "__main__":
    print(build_port(force="--force" in sys.argv))
    print(build_reference(force="--force" in sys.argv))
