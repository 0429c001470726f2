"""The double-float phase reduction of the mixed summators (mixed.cu),
restated in numpy FP32 arithmetic and checked against exact rationals (CPU).

Per dimension the kernel splits kappa = k / 2 pi and x into FP32 hi + lo
parts, forms pr = kh*xh with its exact error e = fma(kh, xh, -pr), keeps the
fraction pr - rint(pr) in a running FP32 sum `a`, and adds the small terms
kh*xl + kl*xh + e into `b` with FMAs; at the end th + tl = (a - rint(a)) + b
as a normalised FP32 pair.  The phase of the reference (src/field.rs:57, the
FP64 dot product k.x) is compared in turns with exact rational arithmetic.

Bounds checked: |theta| * 2^-46 turns while every dimension's product is at
least one turn; up to 2^-24 turns where one of several products is smaller
(the FP32 sum of fractions with different quanta rounds).
"""
from fractions import Fraction

import numpy as np
import pytest

F32 = np.float32
# 2 pi to 100 digits
TWO_PI = Fraction("6.283185307179586476925286766559005768394338798750211641949889184615632812572417997256069650684234136")
K_INV_2PI = 0.15915494309189535                      # fl(1 / (2 pi)), as the mode table uses


def _fma32(a, b, c):
    return F32(float(a) * float(b) + float(c))


def _kernel_phase(k, x):
    """th + tl of the mixed kernel for one point and one mode."""
    a = F32(0.0)
    b = F32(0.0)
    for kd, xd in zip(k, x):
        kap = kd * K_INV_2PI
        kh = F32(kap)
        kl = F32(kap - float(kh))
        xh = F32(xd)
        xl = F32(xd - float(xh))
        pr = F32(kh * xh)
        e = _fma32(kh, xh, -float(pr))
        a = F32(a + F32(pr - np.rint(pr)))
        b = _fma32(kh, xl, _fma32(kl, xh, float(F32(e + b))))
    a2 = F32(a - np.rint(a))
    th = F32(a2 + b)
    tl = F32(b - F32(th - a2))
    return Fraction(float(th)) + Fraction(float(tl))


def _cases(seed, n):
    rng = np.random.default_rng(seed)
    for _ in range(n):
        d = int(rng.integers(1, 4))
        k = rng.standard_normal(d) * 10.0 ** rng.uniform(-1.0, 3.5)
        x = rng.uniform(-1000.0, 1000.0, d)
        yield k, x


def _error(k, x):
    exact = sum(Fraction(float(kd)) * Fraction(float(xd)) for kd, xd in zip(k, x)) / TWO_PI
    err = _kernel_phase(k, x) - (exact - round(exact))
    err -= round(err)
    return abs(float(err))


@pytest.mark.parametrize("seed", [0, 1])
def test_phase_reduction_bounds(seed):
    worst_big, worst_small, n_small = 0.0, 0.0, 0
    for k, x in _cases(seed, 1200):
        turns = np.abs(k * x) / (2.0 * np.pi)
        err = _error(k, x)
        if turns.min() >= 1.0 or len(k) == 1:
            worst_big = max(worst_big, err / max(1.0, turns.sum()))
        else:
            worst_small = max(worst_small, err)
            n_small += 1
    assert worst_big <= 2.0 ** -46
    assert n_small > 0 and worst_small <= 2.0 ** -24


def test_one_dimension_at_large_phase():
    """|k.x| near 1e6 rad: the reduced phase still holds ~2^-29 turns."""
    rng = np.random.default_rng(9)
    errs = [_error(np.array([k]), np.array([x]))
            for k, x in zip(rng.uniform(900.0, 1100.0, 300), rng.uniform(900.0, 1000.0, 300))]
    assert max(errs) <= 2.0 ** -28
