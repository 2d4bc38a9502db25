"""The summation algorithms of the device code, restated on the CPU and checked against what they
stand for, on small vectors (the GPU tests check the kernels themselves):

* exact_runs.cuh: the sequential double sum of nonnegative terms by predicted binade runs - an
  approximate prefix predicts each partial sum's binade, runs between predicted crossings are
  applied as composed integer increment pairs, the other terms are single hardware additions,
  and a run made for the wrong binade falls back to term-by-term addition. Bit for bit equal to
  the sequential loop (amg.cpp:267-268's norm), here with small tiles so that vectors of a few
  thousand terms span many tiles.
* mixed.cu's inner dots: exact float products (TwoProduct), Dot2 partial sums per thread and the
  accurate double-word addition between partials (the double-float sums of the mixed-precision
  solve), within a few units of 2^-44 of the exact dot.
"""
import math
import struct
from fractions import Fraction

import numpy as np
import pytest

KCAP = 1 << 54
TOP = 1 << 53
MANT = (1 << 52) - 1
SKIP, SINGLE, RANGE = 100000, 100001, 100002


def bits(x):
    return struct.unpack("<Q", struct.pack("<d", x))[0]


def dbl(b):
    return struct.unpack("<d", struct.pack("<Q", b))[0]


def sat(a, b):
    return min(a + b, KCAP)


def compose(x, y):
    return (sat(x[0], y[1] if x[0] & 1 else y[0]), sat(x[1], y[0] if x[1] & 1 else y[1]))


def split(s):
    b = bits(s)
    e = (b >> 52) & 0x7FF
    if e == 0:
        return b & MANT, -1074
    return (b & MANT) | (1 << 52), e - 1075


def join(S, u):
    if S < (1 << 52):
        return dbl(S)
    return dbl(((u + 1075) << 52) | (S & MANT))


def term_pair(t, u):
    b = bits(t)
    e = (b >> 52) & 0x7FF
    if e == 0x7FF or (b >> 63):
        return (KCAP, KCAP)
    if e == 0:
        m, et = b & MANT, -1074
    else:
        m, et = (b & MANT) | (1 << 52), e - 1075
    if m == 0:
        return (0, 0)
    sh = et - u
    if sh >= 0:
        if sh > 1:
            return (KCAP, KCAP)
        a = m << sh
        return (KCAP, KCAP) if a >= TOP else (a, a)
    r = -sh
    if r > 60:
        return (0, 0)
    i, rem, half = m >> r, m & ((1 << r) - 1), 1 << (r - 1)
    if rem < half:
        return (i, i)
    if rem > half:
        return (i + 1, i + 1)
    return (i + (1 if i & 1 else 0), i + (0 if i & 1 else 1))


def seg_code(t, pe, pi):
    """exact_runs.cuh seg_code: integer tests on the bits of the approximate sums"""
    bt, be, bi = bits(t), bits(pe), bits(pi)
    if (bt | bi) == 0:
        return SKIP
    ee, ei = be >> 52, bi >> 52
    if ee == 0 or ee >= 0x7FE or ei != ee:
        return SINGLE
    if (be & MANT) < (1 << 26) or (bi & MANT) > MANT - (1 << 27):
        return SINGLE
    return ee - 1075


def segments(terms, a, b, before, cap):
    pre = before + np.concatenate([[0.0], np.cumsum(terms[a:b])])
    codes = [seg_code(float(terms[k]), float(pre[k - a]), float(pre[k - a + 1])) for k in range(a, b)]
    out, i = [], 0
    while i < b - a:
        c = codes[i]
        if c == SINGLE:
            out.append((SINGLE, a + i, 1, (0, 0), float(terms[a + i])))
            i += 1
            continue
        j, pr = i, (0, 0)
        while j < b - a and codes[j] == c:
            pr = compose(pr, term_pair(float(terms[a + j]), c) if c < SKIP else (0, 0))
            j += 1
        out.append((c, a + i, j - i, pr, 0.0))
        i = j
    return out if len(out) <= cap else [(RANGE, a, b - a, (0, 0), 0.0)]


def sequential(s, terms, a, b):
    for k in range(a, b):
        s = s + float(terms[k])
    return s


def run_sum(terms, tile, cap):
    """sum of terms by tiles of `tile` terms, at most `cap` segments a tile; (sum, fallbacks)"""
    m = len(terms)
    ntile = max(1, -(-m // tile))
    tsum = [float(np.sum(terms[c * tile:min(m, (c + 1) * tile)])) for c in range(ntile)]
    segs = []
    for c in range(ntile):
        segs += segments(terms, c * tile, min(m, (c + 1) * tile), float(sum(tsum[:c])), cap)
    s, fallbacks = 0.0, 0
    for code, first, count, pr, t in segs:
        if code == SKIP:
            continue
        if code == SINGLE:
            s = s + t
        else:
            if code != RANGE and s > 0.0:
                S, ue = split(s)
                if ue == code:
                    S2 = sat(S, pr[1] if S & 1 else pr[0])
                    if S2 < TOP:
                        s = join(S2, ue)
                        continue
            fallbacks += 1
            s = sequential(s, terms, first, first + count)
        if not (s < math.inf):
            rest = terms[first + count:]
            return (math.nan if s == s and np.isnan(rest).any() else s), fallbacks
    return s, fallbacks


CASES = {
    "uniform": lambda r: r.random(3000),
    "wide": lambda r: np.exp(r.uniform(-90, 90, 2000)),
    "ties": lambda r: np.sqrt((r.integers(0, 8, 3000) * 0.5) * 2.0 ** r.integers(-3, 3, 3000)),
    "growing": lambda r: np.arange(1, 3001, dtype=np.float64) ** 0.5 * r.uniform(0.9, 1.1, 3000),
    "zeros_first": lambda r: np.concatenate([np.zeros(700), r.normal(size=1500)]),
    "subnormal": lambda r: r.random(500) * 1e-160,
    "all_zero": lambda r: np.zeros(300),
    "single": lambda r: np.array([3.0]),
    "empty": lambda r: np.zeros(0),
}


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("tile", [64, 512])
def test_binade_runs_equal_the_sequential_sum(name, tile):
    v = CASES[name](np.random.default_rng(11))
    terms = v * v
    got, _ = run_sum(terms, tile, cap=tile // 8)
    want = sequential(0.0, terms, 0, len(terms))
    assert bits(got) == bits(want), (got, want)


def test_runs_rarely_fall_back():
    # the predictions choose the path only: well-behaved sums take the one-step runs
    v = np.random.default_rng(3).normal(size=4000)
    _, fallbacks = run_sum(v * v, 512, cap=64)
    assert fallbacks == 0


@pytest.mark.parametrize("pos", [0.3, 0.9])
def test_non_finite_terms(pos):
    v = np.ones(2000)
    v[int(pos * 2000)] = np.inf
    assert run_sum(v * v, 256, 32)[0] == math.inf
    v[-1] = np.nan
    assert math.isnan(run_sum(v * v, 256, 32)[0])


# ---- double-float dots (mixed.cu) -----------------------------------------------------------------
f32 = np.float32


def two_sum(a, b):
    s = f32(a + b)
    bb = f32(s - a)
    return s, f32(f32(a - f32(s - bb)) + f32(b - bb))


def fast_two_sum(a, b):
    s = f32(a + b)
    return s, f32(b - f32(s - a))


def two_prod(x, y):
    h = f32(x * y)
    # the FMA's exact remainder: x*y is exact in double (24 + 24 bits)
    return h, f32(float(x) * float(y) - float(h))


def dot2_add(acc, x, y):
    h, r = two_prod(x, y)
    s, e = two_sum(acc[0], h)
    return s, f32(acc[1] + f32(e + r))


def ff_add(a, b):
    s = two_sum(a[0], b[0])
    t = two_sum(a[1], b[1])
    s = fast_two_sum(s[0], f32(s[1] + t[0]))
    return fast_two_sum(s[0], f32(s[1] + t[1]))


def ff_dot(p, q, per_thread=6, width=256):
    """the device's order: Dot2 over each thread's terms, then pairwise double-word additions"""
    parts = []
    for t0 in range(0, len(p), per_thread):
        acc = (f32(0), f32(0))
        for k in range(t0, min(len(p), t0 + per_thread)):
            acc = dot2_add(acc, p[k], q[k])
        parts.append(two_sum(*acc))
    while len(parts) > 1:
        parts = [ff_add(parts[i], parts[i + 1]) if i + 1 < len(parts) else parts[i] for i in range(0, len(parts), 2)]
    return float(parts[0][0]) + float(parts[0][1]) if parts else 0.0


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_double_float_dot_is_fp64_class(seed):
    r = np.random.default_rng(seed)
    n = 6 * 700
    p = (r.normal(size=n) * np.exp(r.uniform(-4, 4, n))).astype(f32)
    q = (r.normal(size=n) * np.exp(r.uniform(-4, 4, n))).astype(f32)
    exact = sum(Fraction(float(a)) * Fraction(float(b)) for a, b in zip(p, q))
    scale = sum(abs(Fraction(float(a)) * Fraction(float(b))) for a, b in zip(p, q))
    err = abs(Fraction(ff_dot(p, q)) - exact) / scale
    assert err < 2.0 ** -40, float(err)
    # a plain FP32 sum of the same terms is far off
    naive = np.float32(0)
    for a, b in zip(p, q):
        naive = f32(naive + f32(a * b))
    assert abs(Fraction(float(naive)) - exact) / scale > err
