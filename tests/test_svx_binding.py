"""The reference-side binding (include/svxg_svx.hpp: svx::GpuStressProblem and the world's load
builders in the reference's own types) compiled against the reference's headers and linked with
the reference's compiled stress sources and the CUDA library (tests/cpp/test_svx_binding.cpp).

On a machine without a GPU the host part runs (record conversion, bond_utilization and add_force
bit for bit against the reference's compiled functions, pin_reference) and the device part
reports itself skipped; where a GPU and the reference tree are both present the same binary runs
World::Impl::probe_utilization (world.cpp:1907-1940) on svx::StressProblem and on the binding.
Skipped where the reference tree is absent."""
import os
import subprocess
import sys

import pytest

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "cpp"))
import build_tests  # noqa: E402


def test_binding_builds_against_the_reference_headers_and_runs():
    exe = build_tests.build_binding()
    if exe is None:
        pytest.skip("the reference tree is absent")
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), r.stdout + r.stderr
