"""The phase arithmetic of dfturns.cuh, restated in numpy (CPU).

The mixed summators (mixed.cu) take sin and cos of phases held in turns:
whole turns and quarter turns drop out exactly, then polynomials fitted for
this project give sin(2 pi f) and cos(2 pi f) on |f| <= 1/8, and a first-order
term corrects for the phase's low part.  The coefficients are read from the
header itself, so these tests pin the committed constants:

* the polynomials' error on |f| <= 1/8, evaluated as the kernel does (FP32
  Horner steps with fused multiply-adds), against FP64 sin/cos;
* the quarter-turn reduction of sincos_turns_reduced (exact reduced
  argument, rotation by q quarter turns from the low bits of the rounding
  sum) over phases of several turns, with the low-part correction.
"""
import os
import re

import numpy as np
import pytest

from conftest import ROOT

F32 = np.float32
HEADER = os.path.join(ROOT, "gstools-core_gb300", "csrc", "dfturns.cuh")


def _constants():
    text = open(HEADER).read()
    vals = dict((k, float(v)) for k, v in re.findall(r"\b(k[SC][0-4]|kRoundF|kTwoPiF)\s*=\s*([-0-9.eE+]+)f", text))
    return ([vals[f"kS{i}"] for i in range(5)], [vals[f"kC{i}"] for i in range(5)],
            vals["kRoundF"], vals["kTwoPiF"])


def _fma(a, b, c):
    """fmaf on FP32 arrays (the product is exact in FP64; the sum rounds twice
    at worst, far below the bounds tested)."""
    return (np.asarray(a, np.float64) * np.asarray(b, np.float64) + np.asarray(c, np.float64)).astype(F32)


def _horner(k, x):
    acc = np.full_like(x, F32(k[4]))
    for c in (k[3], k[2], k[1], k[0]):
        acc = _fma(acc, x, np.full_like(x, F32(c)))
    return acc


def _sincos_reduced(th, tl, kS, kC, kRound, kTwoPi):
    """sincos_turns_reduced: returns (s1, c1, q mod 4)."""
    qf = _fma(th, np.full_like(th, F32(4.0)), np.full_like(th, F32(kRound)))
    q = (qf - F32(kRound)).astype(F32)
    f = _fma(q, np.full_like(q, F32(-0.25)), th)
    f2 = (f * f).astype(F32)
    s = (_horner(kS, f2) * f).astype(F32)
    c = _horner(kC, f2)
    tw = (tl * F32(kTwoPi)).astype(F32)
    s1 = _fma(tw, c, s)
    c1 = _fma(-tw, s, c)
    return s1, c1, qf.view(np.int32) & 3, f


def test_polynomials_on_the_eighth_turn():
    kS, kC, _, _ = _constants()
    f = np.linspace(-0.125, 0.125, 1_000_001).astype(F32)
    f2 = (f * f).astype(F32)
    s = (_horner(kS, f2) * f).astype(F32).astype(np.float64)
    c = _horner(kC, f2).astype(np.float64)
    x = 2.0 * np.pi * f.astype(np.float64)
    assert np.abs(s - np.sin(x)).max() <= 8.7e-8
    assert np.abs(c - np.cos(x)).max() <= 5.8e-8


def test_quarter_turn_reduction():
    kS, kC, kRound, kTwoPi = _constants()
    rng = np.random.default_rng(3)
    th = rng.uniform(-4.0, 4.0, 400_000).astype(F32)
    tl = (rng.uniform(-1.0, 1.0, th.size) * 2.0 ** -26).astype(F32)
    s1, c1, q, f = _sincos_reduced(th, tl, kS, kC, kRound, kTwoPi)
    assert np.abs(f).max() <= 0.125
    # f is the exact remainder: th = q/4 + f
    qn = np.rint(4.0 * th.astype(np.float64))
    assert np.array_equal(f.astype(np.float64), th.astype(np.float64) - qn / 4.0)
    assert np.array_equal(q, (qn.astype(np.int64) & 3).astype(np.int32))
    # rotate by q quarter turns, as the callers do
    rot = {0: (s1, c1), 1: (c1, -s1), 2: (-s1, -c1), 3: (-c1, s1)}
    sin_q = np.select([q == k for k in range(4)], [rot[k][0] for k in range(4)])
    cos_q = np.select([q == k for k in range(4)], [rot[k][1] for k in range(4)])
    phase = 2.0 * np.pi * (th.astype(np.float64) + tl.astype(np.float64))
    assert np.abs(sin_q - np.sin(phase)).max() <= 1.5e-7
    assert np.abs(cos_q - np.cos(phase)).max() <= 1.5e-7


@pytest.mark.parametrize("name", ["kRoundF", "kTwoPiF"])
def test_named_constants(name):
    _, _, kRound, kTwoPi = _constants()
    if name == "kRoundF":
        assert kRound == 1.5 * 2.0 ** 23
    else:
        assert kTwoPi == float(F32(2.0 * np.pi))
