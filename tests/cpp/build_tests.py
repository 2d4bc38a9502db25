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


def build_binding() -> str | None:
    """The reference-side binding (include/svxg_svx.hpp) against the reference's headers, linked
    with the reference's compiled stress sources (the oracle's libsvxref.so) and libsvxg.so. None
    where the reference tree is absent."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import build_oracle
    ref_lib = build_oracle.build_reference()
    if not ref_lib or not os.path.exists(ref_lib):
        return None
    out = os.path.join(HERE, "_build", "test_svx_binding")
    src = os.path.join(HERE, "test_svx_binding.cpp")
    deps = [src, ref_lib, os.path.join(LIBDIR, "libsvxg.so")] + \
        [os.path.join(ROOT, "include", h) for h in ("svxg_svx.hpp", "svxg_stress_problem.hpp", "svxg.h")]
    if os.path.exists(out) and os.path.getmtime(out) >= max(os.path.getmtime(p) for p in deps):
        return out
    os.makedirs(os.path.dirname(out), exist_ok=True)
    ref_dir = os.path.dirname(ref_lib)
    # (the reference's own flags: C++20, no exceptions, no RTTI, no contraction)
    cmd = ["g++", "-std=c++20", "-O2", "-ffp-contract=off", "-fno-exceptions", "-fno-rtti",
           "-I", os.path.join(build_oracle.REFERENCE, "core", "include"), "-I", os.path.join(ROOT, "include"), src,
           "-o", out, "-L", LIBDIR, "-lsvxg", "-L", ref_dir, "-lsvxref", f"-Wl,-rpath,{LIBDIR}:{ref_dir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode:
        sys.stderr.write(r.stdout + r.stderr)
        raise RuntimeError("binding test build failed")
    return out


if __name__ == "__main__":
    print(build())
