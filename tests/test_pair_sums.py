"""The FP32 pair sums behind the mixed path's moment partials (CPU): the
axis-1 projection accumulates, per thread, sums of d, jj d and jj^2 d over
its run of FP32 increments d as unevaluated pairs hi + lo (Knuth's two-sum;
the FMA residual of w x for the integer weights) and takes FP64 only once.
Restated here in numpy float32 with the same operation order, the pair sums
are checked against exact rational sums: the error stays within a few units
of 2^-44 of the sum of |terms|, far below the 1e-12 conservation bound."""
from __future__ import annotations

from fractions import Fraction

import numpy as np
import pytest

f32 = np.float32


def _two_sum_add(hi, lo, x):
    s = f32(hi + x)
    bp = f32(s - hi)
    err = f32(f32(hi - f32(s - bp)) + f32(x - bp))
    return s, f32(lo + err)


def _fma_residual(w, x, p):
    # exact w x - p (w x and p are FP32; the product is exact in FP64)
    return f32(float(w) * float(x) - float(p))


def _pair_sum(terms, weights):
    hi, lo = f32(0), f32(0)
    for w, x in zip(weights, terms):
        p = f32(f32(w) * x)
        hi, lo = _two_sum_add(hi, lo, p)
        lo = f32(lo + _fma_residual(f32(w), x, p))
    return float(hi) + float(lo)


@pytest.mark.parametrize("seed", range(6))
@pytest.mark.parametrize("order", [0, 1, 2])
def test_pair_sums_exact_to_2e44(seed, order):
    rng = np.random.default_rng(seed)
    jg = 6
    # increments of mixed sign and spread magnitude, as FP32 numbers
    d = (rng.standard_normal(jg) * 10.0 ** rng.uniform(-6, -2, jg)).astype(np.float32)
    w = [float(jj ** order) for jj in range(jg)]
    got = _pair_sum(d, w)
    exact = sum(Fraction(wi) * Fraction(float(x)) for wi, x in zip(w, d))
    mag = sum(abs(Fraction(wi) * Fraction(float(x))) for wi, x in zip(w, d))
    assert abs(Fraction(got) - exact) <= Fraction(8, 2 ** 44) * mag


def test_plain_fp32_sum_is_not_enough():
    """The same sums in plain FP32 miss by ~1e-8 of the terms, the reason
    for the pairs."""
    rng = np.random.default_rng(7)
    worst = 0.0
    for _ in range(50):
        d = (rng.standard_normal(6) * 10.0 ** rng.uniform(-6, -2, 6)).astype(np.float32)
        s = f32(0)
        for x in d:
            s = f32(s + x)
        exact = sum(Fraction(float(x)) for x in d)
        mag = sum(abs(Fraction(float(x))) for x in d)
        worst = max(worst, float(abs(Fraction(float(s)) - exact) / mag))
    assert worst > 2.0 ** -30
