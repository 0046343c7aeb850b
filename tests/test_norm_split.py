"""The split behind the recomputed residual's norm in the mixed solver
(`k_outer_residual<false, true>`, `peps_mg_gb300/csrc/pmg_mixed.cu`), restated on the host:
r = r32 + rl, r32 the round-to-nearest FP32 value (the kernel's FP32 copy), rl read from the
29 mantissa bits the rounding dropped, both scaled by 2^nexp; (r32 + rl)^2 is formed as the
FP32 product w^2, its FMA rounding error and 2 w rl.  Checked against exact rational arithmetic
on seeded values over the FP32 normal range: each squared term to 2^-45 relative, and a sum of
many terms, accumulated with two-sum as the kernel does, to 1e-11 relative.
"""
from fractions import Fraction

import numpy as np


def low_part_scaled(v, nexp):
    """f64_low_part_scaled: (v - fl32(v)) 2^nexp rounded to FP32, from the encoding."""
    bits = int(np.float64(v).view(np.uint64))
    e = ((bits >> 52) & 0x7FF) - 1023
    k = e - 52 + nexp
    if e < -126 or e > 127 or k < -126 or k > 127:
        return np.float32(0.0)
    m = bits & ((1 << 52) - 1)
    hi = m >> 29
    rem = m & 0x1FFFFFFF
    up = rem > 0x10000000 or (rem == 0x10000000 and (hi & 1))
    q = rem - 0x20000000 if up else rem
    d = np.float32(q) * np.float32(2.0 ** k)
    return -d if bits >> 63 else d


def f32(x):
    return np.float32(x)


def two_sum(a, b):
    s = f32(a + b)
    bb = f32(s - a)
    return s, f32(f32(a - f32(s - bb)) + f32(b - bb))


def fma32(a, b, c):
    """FP32 fused multiply-add: the exact a b + c rounded once (via Fraction)."""
    return np.float32(float(Fraction(float(a)) * Fraction(float(b)) + Fraction(float(c))))


def square_terms(v, nexp):
    w = f32(f32(v) * f32(2.0 ** nexp))
    wl = low_part_scaled(v, nexp)
    p = f32(w * w)
    pe = fma32(w, w, -p)
    pe = fma32(f32(2.0 * w), wl, pe)
    return p, pe


def test_square_of_each_value():
    rng = np.random.default_rng(17)
    for _ in range(3000):
        mag = 10.0 ** rng.uniform(-12, 8)
        v = float(rng.uniform(-1, 1) * mag)
        nexp = int(np.floor(-np.log2(mag))) + int(rng.integers(-3, 4))
        p, pe = square_terms(v, nexp)
        exact = (Fraction(v) * Fraction(2) ** nexp) ** 2
        got = Fraction(float(p)) + Fraction(float(pe))
        assert abs(got - exact) <= exact * Fraction(1, 2 ** 45), v


def test_rounding_direction_of_the_low_part():
    # values exactly half-way between two FP32 numbers (ties to even) and just beside them
    base = float(np.float32(1.2345678))
    ulp = float(np.spacing(np.float32(base)))
    for v in (base + ulp / 2, base + ulp / 2 * (1 + 2 ** -20), base + ulp / 2 * (1 - 2 ** -20), base + 1.5 * ulp,
              -(base + ulp / 2)):
        r32 = np.float32(v)
        low = low_part_scaled(v, 0)
        assert Fraction(float(r32)) + Fraction(float(low)) == Fraction(v), v


def test_norm_of_many_values():
    rng = np.random.default_rng(5)
    vals = rng.normal(size=4000) * 10.0 ** rng.uniform(-3, 1, size=4000) * 1e-9
    nexp = 30
    S = f32(0.0)
    Sl = f32(0.0)
    for v in vals:
        p, pe = square_terms(float(v), nexp)
        S, t = two_sum(S, p)
        Sl = f32(Sl + f32(t + pe))
    got = (Fraction(float(S)) + Fraction(float(Sl))) / Fraction(2) ** (2 * nexp)
    exact = sum(Fraction(float(v)) ** 2 for v in vals)
    assert abs(got - exact) <= exact * Fraction(1, 10 ** 11)
