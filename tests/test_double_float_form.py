"""CPU check of the double-float arithmetic of the mixed step's residual
pass (dd_from_bits, dd_fma, dd_add of the operator kernel), restated in
numpy float32 with the FMA emulated exactly (a float32 product is exact in
float64, so round32(a*b - p) computed in float64 is the FMA's result).

Checked against exact rational arithmetic:
  * the bit split of an FP64 value into hi + lo floats is within 2^-47 of
    the value (relative) and hi is the value truncated to 24 bits;
  * a sum of n products of split values, accumulated like the kernel's
    table and gather loops, is within n * 2^-46 of the sum of the terms'
    magnitudes (the bound quoted for the residual pass: ~1e-13 of |b| for
    rows of a few hundred terms), where a plain float32 sum is ~2^-24.
(The device kernel is compared with the FP64 pass on the GPU in
tests/test_gpu_mixed.py.)
"""
from fractions import Fraction

import numpy as np
import pytest

f32 = np.float32


def split_bits(v: float):
    """dd_from_bits: hi = sign, exponent and top 23 stored mantissa bits;
    lo = the remaining 29 bits as a float."""
    b = np.array([v], np.float64).view(np.uint64)[0]
    sign = -1.0 if b >> 63 else 1.0
    e11 = int((b >> 52) & 0x7FF)
    if e11 - 1023 + 127 <= 0:
        return f32(0), f32(0)
    hb = np.uint64(b & ~np.uint64(0x1FFFFFFF))          # truncate the low 29 mantissa bits
    hi = f32(np.array([hb], np.uint64).view(np.float64)[0])   # exact: 24 significant bits
    rem = int(b & 0x1FFFFFFF)
    lo = f32(sign * rem * 2.0 ** (e11 - 1075)) if rem else f32(0)
    return hi, lo


def fma32(a, b, c):
    return f32(np.float64(a) * np.float64(b) + np.float64(c))


def dd_fma(acc, a, b):
    """acc += a b (acc, a, b: (hi, lo) float32 pairs), as the kernel does."""
    ahi, alo = a
    bhi, blo = b
    p = f32(ahi * bhi)
    e = fma32(ahi, bhi, -p)
    e = fma32(ahi, blo, e)
    e = fma32(alo, bhi, e)
    s = f32(acc[0] + p)
    bv = f32(s - acc[0])
    err = f32(f32(acc[0] - f32(s - bv)) + f32(p - bv))
    return s, f32(acc[1] + f32(err + e))


def exact(x) -> Fraction:
    return Fraction(float(x))


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_split_is_truncation_within_2_pow_47(seed):
    rng = np.random.default_rng(seed)
    vals = rng.standard_normal(2000) * np.exp(rng.uniform(-30, 30, 2000))
    for v in vals:
        hi, lo = split_bits(float(v))
        assert abs(float(hi)) <= abs(v)                                   # truncation toward zero
        err = abs(exact(hi) + exact(lo) - exact(v))
        assert err <= Fraction(2) ** -47 * abs(exact(v))


@pytest.mark.parametrize("n", [64, 600])
def test_dd_dot_product_error_bound(n):
    rng = np.random.default_rng(n)
    a = rng.standard_normal(n) * np.exp(rng.uniform(-3, 3, n))
    b = rng.standard_normal(n) * np.exp(rng.uniform(-3, 3, n))
    acc = (f32(0), f32(0))
    plain = f32(0)
    for x, y in zip(a, b):
        xs, ys = split_bits(float(x)), split_bits(float(y))
        acc = dd_fma(acc, xs, ys)
        plain = f32(plain + f32(xs[0] * ys[0]))
    truth = sum(exact(x) * exact(y) for x, y in zip(a, b))
    scale = sum(abs(exact(x) * exact(y)) for x, y in zip(a, b))
    err = abs(exact(acc[0]) + exact(acc[1]) - truth)
    assert err <= n * Fraction(2) ** -46 * scale, float(err / scale)
    # a plain float32 accumulation is some 5 orders of magnitude worse
    assert abs(exact(plain) - truth) > 100 * err
