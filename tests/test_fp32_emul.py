"""The FP32 emulation the certification tests rely on, against exact
rational arithmetic."""
from fractions import Fraction

import numpy as np

from fp32_emul import F, f32_dir, f32_trunc, fma32


def _nearest_even(ex):
    f = np.float32(float(ex))
    cand = [np.nextafter(f, F(-np.inf)), f, np.nextafter(f, F(np.inf))]
    return min(cand, key=lambda y: (abs(Fraction(float(y)) - ex), int(np.float32(y).view(np.uint32)) & 1))


def test_fma32_is_correctly_rounded():
    rng = np.random.default_rng(3)
    n = 3000
    a = rng.normal(size=n).astype(np.float32)
    b = rng.normal(size=n).astype(np.float32)
    # sums that cancel most of the product, and unrelated sums
    c = (-(a.astype(np.float64) * b) * (1 + rng.normal(size=n) * 1e-7)).astype(np.float32)
    c[:500] = rng.normal(size=500).astype(np.float32)
    got = fma32(a, b, c)
    for i in range(n):
        ex = Fraction(float(a[i])) * Fraction(float(b[i])) + Fraction(float(c[i]))
        assert got[i] == _nearest_even(ex), i


def test_fma32_midpoint_after_fp64_rounding():
    """(2^-12 (1 + 2^-18)) (2^-12 (1 - 2^-18)) + (1 + 2^-23) is 2^-60 below
    the midpoint 1 + 3 2^-24; its FP64 sum is the midpoint itself, which a
    plain conversion would round to even (up).  The FMA rounds down."""
    a = np.array([2.0 ** -12 * (1 + 2.0 ** -18)], dtype=np.float32)
    b = np.array([2.0 ** -12 * (1 - 2.0 ** -18)], dtype=np.float32)
    c = np.array([1 + 2.0 ** -23], dtype=np.float32)
    assert (a.astype(np.float64) * b + c.astype(np.float64))[0] == 1 + 3 * 2.0 ** -24
    assert fma32(a, b, c)[0] == F(1 + 2.0 ** -23)
    # an exact midpoint keeps ties-to-even
    h = np.array([2.0 ** -12], dtype=np.float32)
    assert fma32(h, h, np.ones(1, dtype=np.float32))[0] == F(1)


def test_directed_roundings():
    x = np.array([1.0 + 2.0 ** -30, -1.0 - 2.0 ** -30, 3.0, 1e-300, -1e-300, 1e39, 2.0 ** -127])
    up, down = f32_dir(x[:5], True), f32_dir(x[:5], False)
    assert (up.astype(np.float64) >= x[:5]).all() and (down.astype(np.float64) <= x[:5]).all()
    t = f32_trunc(x)
    assert t[0] == F(1) and t[1] == F(-1) and t[2] == F(3)
    assert t[3] == 0 and np.signbit(t[4]) and t[4] == 0 and np.isinf(t[5]) and t[6] == 0
