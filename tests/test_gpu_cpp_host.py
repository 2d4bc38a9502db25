"""The C++20 host class over the C ABI (include/svxg_stress_problem.hpp), running the reference's
own stress cases as the reference writes them (tests/cpp/test_adapter.cpp)."""
import os
import subprocess
import sys

import pytest

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "cpp"))
import build_tests  # noqa: E402

pytestmark = pytest.mark.gpu


def test_cpp_host_class_runs_the_reference_cases():
    exe = build_tests.build()
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), r.stdout + r.stderr


def test_cpp_host_builds():
    assert os.path.exists(build_tests.build())
