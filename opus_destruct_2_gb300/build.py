"""In-tree build of the native libraries (nvcc for sm_103a, g++ for host code).

libsvxg.so        - the CUDA stress solve and its C ABI (include/svxg.h)
libsvxg_synth.so  - the seeded workload generator (host only)

Both land in opus_destruct_2_gb300/_lib/. Translation units compile in parallel; nothing is
rebuilt when its sources are older than its output.
"""
from __future__ import annotations

import glob
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "_lib")
INCLUDE = os.path.join(ROOT, "include")
NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_LIB = "libsvxg.so"
SYNTH_LIB = "libsvxg_synth.so"


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        raise RuntimeError(f"build failed: {os.path.basename(cmd[-1])}")


def _newest(paths: list[str]) -> float:
    return max(os.path.getmtime(p) for p in paths)


def _headers() -> list[str]:
    return sum((glob.glob(os.path.join(CSRC, pat)) for pat in ("*.cuh", "*.hpp", "*.h")), []) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))


def synth_library(force: bool = False) -> str:
    out = os.path.join(LIBDIR, SYNTH_LIB)
    src = os.path.join(CSRC, "synth.cpp")
    if force or not os.path.exists(out) or _newest([src] + _headers()) > os.path.getmtime(out):
        os.makedirs(LIBDIR, exist_ok=True)
        _run(["g++", "-std=c++20", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-I", INCLUDE, src, "-o", out])
    return out


def cuda_sources() -> list[str]:
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def cuda_library(force: bool = False, verbose_ptxas: bool = False) -> str:
    out = os.path.join(LIBDIR, CUDA_LIB)
    srcs = cuda_sources() + sorted(glob.glob(os.path.join(CSRC, "host_*.cpp")))
    if not force and os.path.exists(out) and _newest(srcs + _headers()) <= os.path.getmtime(out):
        return out
    objdir = os.path.join(LIBDIR, "obj")
    os.makedirs(objdir, exist_ok=True)
    jobs, objs = [], []
    for s in srcs:
        o = os.path.join(objdir, os.path.basename(s) + ".o")
        objs.append(o)
        if s.endswith(".cu"):
            # (host code without contraction either: the same host arithmetic on x86 and Arm)
            cmd = [NVCC, *ARCH, "-std=c++20", "-O3", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off", "-I", INCLUDE,
                   "-I", CSRC,
                   "--expt-relaxed-constexpr", "-c", s, "-o", o]
            if os.path.basename(s).startswith("exact_"):
                cmd.insert(1, "-fmad=false")  # (bit-exact setup arithmetic: no contraction)
            if verbose_ptxas:
                cmd.insert(1, "-Xptxas=-v")
        else:
            cmd = ["g++", "-std=c++20", "-O2", "-ffp-contract=off", "-fPIC", "-I", INCLUDE, "-I", CSRC, "-c", s, "-o", o]
        jobs.append(cmd)
    with ThreadPoolExecutor(max_workers=max(1, min(8, len(jobs)))) as ex:
        list(ex.map(_run, jobs))
    _run([NVCC, *ARCH, "-shared", "-o", out] + objs + ["-lcudart"])
    return out


def build_all(force: bool = False) -> dict:
    return {"synth": synth_library(force), "cuda": cuda_library(force) if cuda_sources() else None}


if __name__ == "__main__":
    print(build_all(force="--force" in sys.argv))
