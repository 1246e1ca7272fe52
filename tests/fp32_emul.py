"""IEEE FP32 operations of the kernels, emulated in numpy for the CPU
certification tests of the mixed path's FP32 filters: correctly rounded
fused multiply-add (to nearest, and up), rounding toward zero with flush of subnormals (the
engine's f32_trunc), and directed rounding of FP64 values to FP32."""
import numpy as np

F = np.float32
U = F(5.9604645e-08)  # 2^-24


def fma32(a, b, c):
    """Correctly rounded FP32 fused multiply-add (__fmaf_rn): the product of
    two floats is exact in FP64; the sum is split error-free (TwoSum), and a
    sum that lands exactly between two floats is resolved by the sign of the
    error."""
    a, b, c = (np.asarray(x, dtype=np.float32) for x in (a, b, c))
    p = a.astype(np.float64) * b.astype(np.float64)
    c64 = c.astype(np.float64)
    with np.errstate(over="ignore", invalid="ignore"):
        s = p + c64
        bb = s - p
        err = (p - (s - bb)) + (c64 - bb)
        f = s.astype(np.float32)
        fd = f.astype(np.float64)
        other = np.where(fd < s, np.nextafter(f, F(np.inf)), np.nextafter(f, F(-np.inf)))
        mid = np.isfinite(s) & (fd != s) & ((fd + other.astype(np.float64)) * 0.5 == s)
        toward = np.where(err > 0, np.maximum(f, other), np.minimum(f, other))
        return np.where(mid & (err != 0), toward, f).astype(np.float32)


def fma32_up(a, b, c):
    """FP32 fused multiply-add rounded up (__fmaf_ru): the smallest float at
    or above a b + c.  The FP64 sum s of the exact product and c is within
    half an FP64 ulp of the exact value; rounding s up is exact unless s is
    itself a float and the TwoSum error is positive."""
    a, b, c = (np.asarray(x, dtype=np.float32) for x in (a, b, c))
    p = a.astype(np.float64) * b.astype(np.float64)
    c64 = c.astype(np.float64)
    with np.errstate(over="ignore", invalid="ignore"):
        s = p + c64
        bb = s - p
        err = (p - (s - bb)) + (c64 - bb)
        f = np.atleast_1d(f32_dir(s, up=True))
        bump = (f.astype(np.float64) == s) & (err > 0)
        f[bump] = np.nextafter(f[bump], F(np.inf))
        return f


def f32_trunc(x):
    """FP64 -> FP32 toward zero; magnitudes below FLT_MIN flush to (signed)
    zero, at or above 2^128 to infinity."""
    x = np.asarray(x, dtype=np.float64)
    with np.errstate(over="ignore"):
        f = x.astype(np.float32)
    big = (np.abs(f.astype(np.float64)) > np.abs(x)) & np.isfinite(f)
    f[big] = np.nextafter(f[big], F(0))
    ovf = np.abs(x) >= 2.0 ** 128
    f[ovf] = np.copysign(F(np.inf), x[ovf]).astype(np.float32)
    tiny = np.abs(x) < 2.0 ** -126
    f[tiny] = np.copysign(F(0), x[tiny]).astype(np.float32)
    return f


def f32_dir(x, up):
    """FP64 -> FP32 rounded up (the smallest float >= x) or down."""
    x = np.asarray(x, dtype=np.float64)
    f = x.astype(np.float32)
    if up:
        m = f.astype(np.float64) < x
        f[m] = np.nextafter(f[m], F(np.inf))
    else:
        m = f.astype(np.float64) > x
        f[m] = np.nextafter(f[m], F(-np.inf))
    return f
