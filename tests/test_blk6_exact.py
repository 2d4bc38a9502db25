"""The device assembly's reduced rigid-block products equal the full loops of the reference's
blk6::atbd_add (core/src/solve/amg.cpp:155-170) value for value: blk6.cuh compiled for the host
with the reference's -ffp-contract=off, 7.2 million entries compared."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reduced_products_equal_full_loops(tmp_path):
    exe = str(tmp_path / "blk6")
    subprocess.run(["g++", "-std=c++20", "-O2", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"), "-I",
                    os.path.join(ROOT, "opus_destruct_2_gb300", "csrc"), os.path.join(ROOT, "tests", "cpp",
                    "test_blk6_exact.cpp"), "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "value mismatches 0" in r.stdout, r.stdout
