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
(the FP32 sum of fractions with different quanta rounds).  Then the whole
per-term arithmetic, restated over a 2-D field, against the oracle: the
error budget of the form and the share of it the phase rounding takes.
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


# ---------------------------------------------------------------------------
# the whole per-term arithmetic of the mixed kernel, vectorised over points
# and modes: phase as above, sincos_turns_reduced (tests/test_dfturns_cpu.py
# restates it), weights rotated by the quarter-turn count, the FP32 term
# fmaf(w.x, c1, w.y * s1); the compensated tile sums are taken as exact
# ---------------------------------------------------------------------------
def _fma_arr(a, b, c):
    return (np.asarray(a, np.float64) * np.asarray(b, np.float64)
            + np.asarray(c, np.float64)).astype(F32)


def _mixed_field(cov, z1, z2, pos, exact_phase=False):
    from test_dfturns_cpu import _constants, _sincos_reduced
    kS, kC, kRound, kTwoPi = _constants()
    kap = cov * K_INV_2PI
    kh = kap.astype(F32)
    kl = (kap - kh.astype(np.float64)).astype(F32)
    xh = pos.astype(F32)
    xl = (pos - xh.astype(np.float64)).astype(F32)
    shape = (pos.shape[1], cov.shape[1])
    a = np.zeros(shape, F32)
    b = np.zeros(shape, F32)
    for d in range(cov.shape[0]):
        KH, KL = np.broadcast_to(kh[d][None, :], shape), np.broadcast_to(kl[d][None, :], shape)
        XH, XL = np.broadcast_to(xh[d][:, None], shape), np.broadcast_to(xl[d][:, None], shape)
        pr = (KH * XH).astype(F32)
        e = _fma_arr(KH, XH, -pr)
        a = (a + (pr - np.rint(pr)).astype(F32)).astype(F32)
        b = _fma_arr(KH, XL, _fma_arr(KL, XH, (e + b).astype(F32)))
    a2 = (a - np.rint(a)).astype(F32)
    th = (a2 + b).astype(F32)
    tl = (b - (th - a2)).astype(F32)
    if exact_phase:
        turns = (cov.T @ pos).T / (2.0 * np.pi)
        turns -= np.rint(turns)
        th = turns.astype(F32)
        tl = (turns - th.astype(np.float64)).astype(F32)
    s1, c1, q, _ = _sincos_reduced(th, tl, kS, kC, kRound, kTwoPi)
    z1f, z2f = z1.astype(F32), z2.astype(F32)
    rot = [(z1f, z2f), (z2f, -z1f), (-z1f, -z2f), (-z2f, z1f)]
    wx = np.select([q == k for k in range(4)], [np.broadcast_to(r[0], shape) for r in rot])
    wy = np.select([q == k for k in range(4)], [np.broadcast_to(r[1], shape) for r in rot])
    z12 = _fma_arr(wx, c1, (wy.astype(F32) * s1).astype(F32))
    return z12.astype(np.float64).sum(axis=1)


def test_mixed_arithmetic_error_budget():
    """A 2-D field like the 1e5-point x 1000-mode workload (positions in
    [0, 100]^2, Gaussian spectrum l = 10): the restated arithmetic stays well
    inside the form's 1e-6 bar, and an exact phase would remove a visible part
    of the max error (the sub-turn rounding of the fractions' sum)."""
    import oracle
    rng = np.random.default_rng(0)
    pos = rng.uniform(0.0, 100.0, (2, 600))
    cov = rng.normal(0.0, np.sqrt(2.0) / 10.0, (2, 500))
    z1, z2 = rng.standard_normal(500), rng.standard_normal(500)
    ref = oracle.summator(cov, z1, z2, pos, num_threads=1)
    rms = float(np.sqrt(np.mean(ref ** 2)))
    e = _mixed_field(cov, z1, z2, pos) - ref
    e_exact = _mixed_field(cov, z1, z2, pos, exact_phase=True) - ref
    assert float(np.sqrt(np.mean(e ** 2))) / rms <= 1.5e-7
    assert float(np.abs(e).max()) / rms <= 5e-7
    assert float(np.sqrt(np.mean(e_exact ** 2))) < 0.9 * float(np.sqrt(np.mean(e ** 2)))
