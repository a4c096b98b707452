"""The FP32-pair arithmetic of the fp64x form (hodlr3d_gb300/csrc/matvec_gemv.cu:
mac, merge, value), restated with numpy float32 on the CPU and checked against
exact rational sums: dot products of FP64 data reach ~1e-14 of sum |a x|, the
accuracy the GPU tests ask of the fp64x products.  The fused multiply-add is
emulated in float64, which is exact for the product's error term (a float32
product fits in 48 bits and its rounding error is a float32)."""
from fractions import Fraction

import numpy as np

f32 = np.float32


def fma(a, b, c):
    return f32(np.float64(a) * np.float64(b) + np.float64(c))


def two_sum(s, p):
    t = f32(s + p)
    bb = f32(t - s)
    return t, f32(f32(s - f32(t - bb)) + f32(p - bb))


def mac(s, c, v, lo, xh, xl):
    p = f32(v * xh)
    e = fma(v, xh, -p)              # v xh = p + e exactly
    s, err = two_sum(s, p)
    return s, f32(c + f32(err + fma(v, xl, fma(lo, xh, e))))


def merge(s, c, s2, c2):
    s, err = two_sum(s, s2)
    return s, f32(f32(c + c2) + err)


def pair(v):
    hi = f32(v)
    return hi, f32(np.float64(v) - np.float64(hi))


def test_pair_dot_products_reach_fp64_accuracy():
    rng = np.random.default_rng(0)
    for n, scale in ((64, 1.0), (1024, 1e-3), (4096, 1e5)):
        a = rng.standard_normal(n) * scale
        x = rng.standard_normal(n)
        # two lanes, merged at the end (as a warp's butterfly does)
        acc = [(f32(0), f32(0)), (f32(0), f32(0))]
        for i in range(n):
            v, lo = pair(a[i])
            xh, xl = pair(x[i])
            s, c = acc[i % 2]
            acc[i % 2] = mac(s, c, v, lo, xh, xl)
        s, c = merge(*acc[0], *acc[1])
        got = float(s) + float(c)
        exact = sum(Fraction(float(ai)) * Fraction(float(xi)) for ai, xi in zip(a, x))
        scale_sum = float(sum(abs(Fraction(float(ai)) * Fraction(float(xi))) for ai, xi in zip(a, x)))
        assert abs(got - float(exact)) <= 1e-13 * scale_sum, (n, got, float(exact))


def test_two_sum_is_error_free():
    rng = np.random.default_rng(1)
    for _ in range(2000):
        s, p = f32(rng.standard_normal() * 10.0 ** int(rng.integers(-8, 8))), f32(rng.standard_normal())
        t, err = two_sum(s, p)
        assert Fraction(float(t)) + Fraction(float(err)) == Fraction(float(s)) + Fraction(float(p))
