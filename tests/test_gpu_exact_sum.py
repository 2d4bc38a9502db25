"""The device's parallel reproduction of a sequential double sum (the multigrid setup's norm,
core/src/solve/amg.cpp:267-268) against the sequential loop itself: bit for bit, on magnitudes
spread over 80 binades, exact ties, subnormals, zeros, and non-finite terms - in one block for
shorter vectors (one warp up to 4096 terms) and by chunks over many blocks for vectors past
131,072 terms."""
import ctypes
import math

import numpy as np
import pytest

from opus_destruct_2_gb300 import load_library
from opus_destruct_2_gb300.graph import ptr

pytestmark = pytest.mark.gpu


def seq_norm(v):
    s = 0.0
    for x in v:
        s = s + float(x) * float(x)
    return math.sqrt(s)


def dev_norm(v):
    v = np.ascontiguousarray(v, dtype=np.float64)
    out = ctypes.c_double()
    assert load_library().svxg_debug_seq_norm(ptr(v), len(v), ctypes.byref(out)) == 0
    return out.value


CASES = {
    "uniform": lambda r: r.random(200_000),
    "wide": lambda r: np.exp(r.uniform(-90, 90, 50_000)),
    "ties": lambda r: np.sqrt((r.integers(0, 8, 100_000) * 0.5) * 2.0 ** r.integers(-3, 3, 100_000)),
    "tiny": lambda r: r.random(30_000) * 1e-160,
    "zeros_first": lambda r: np.concatenate([np.zeros(20_000), r.normal(size=20_000)]),
    "power_iteration": lambda r: r.normal(size=1_131_000) * 1e-3,
    "wide_many_chunks": lambda r: np.exp(r.uniform(-90, 90, 400_000)),
    "ties_many_chunks": lambda r: np.sqrt((r.integers(0, 8, 300_000) * 0.5) * 2.0 ** r.integers(-3, 3, 300_000)),
    "growing_many_chunks": lambda r: np.arange(1, 500_001, dtype=np.float64) ** 0.5 * r.uniform(0.9, 1.1, 500_000),
    "zeros_then_chunks": lambda r: np.concatenate([np.zeros(150_000), r.normal(size=150_000)]),
    "wide_short": lambda r: np.exp(r.uniform(-90, 90, 3000)),
    "ties_short": lambda r: np.sqrt((r.integers(0, 8, 4096) * 0.5) * 2.0 ** r.integers(-3, 3, 4096)),
    "zeros_first_short": lambda r: np.concatenate([np.zeros(1000), r.normal(size=1000)]),
    "all_zero_short": lambda r: np.zeros(500),
    "subnormal_short": lambda r: r.random(2000) * 1e-160,
    "single": lambda r: np.array([3.0]),
    "empty": lambda r: np.zeros(0),
}


@pytest.mark.parametrize("name", list(CASES))
def test_sequential_norm_bits(name):
    v = CASES[name](np.random.default_rng(7))
    a, b = dev_norm(v), seq_norm(v)
    assert (a == b) or (math.isnan(a) and math.isnan(b)), (a, b)


@pytest.mark.parametrize("n", [2_000, 10_000, 300_000])
def test_non_finite_terms(n):
    v = np.ones(n)
    v[n // 2] = np.inf
    assert dev_norm(v) == math.inf
    v[n // 2 + n // 8] = np.nan
    assert math.isnan(dev_norm(v))
