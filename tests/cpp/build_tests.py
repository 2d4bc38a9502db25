"""Builds the C++ host tests against the in-tree CUDA library (tests/cpp/_build/)."""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
LIBDIR = os.path.join(ROOT, "opus_destruct_2_gb300", "_lib")


def build() -> str:
    out = os.path.join(HERE, "_build", "test_adapter")
    src = os.path.join(HERE, "test_adapter.cpp")
    hdr = os.path.join(ROOT, "include", "svxg_stress_problem.hpp")
    lib = os.path.join(LIBDIR, "libsvxg.so")
    if os.path.exists(out) and os.path.getmtime(out) >= max(os.path.getmtime(p) for p in (src, hdr, lib)):
        return out
    os.makedirs(os.path.dirname(out), exist_ok=True)
    # (the reference's own host flags: no exceptions, no RTTI - the adapter must build under them)
    cmd = ["g++", "-std=c++20", "-O2", "-fno-exceptions", "-fno-rtti", "-I", os.path.join(ROOT, "include"), src, "-o", out, "-L", LIBDIR, "-lsvxg",
           f"-Wl,-rpath,{LIBDIR}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode:
        sys.stderr.write(r.stdout + r.stderr)
        raise RuntimeError("C++ host test build failed")
    return out


if __name__ == "__main__":
    print(build())
