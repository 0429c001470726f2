"""The operand slicing of the x5 tensor-core form, restated in numpy (CPU).

The kernel (separable_tc.cu: slice3x2 for the rows F, gtab_x5_entry for
the columns G) represents each FP32 factor by f16 slices so that the
leading product F1*G1 is an integer multiple of a fixed unit:

  F / W (|F/W| <= 1), in units of 2^15:
      F1 = 2^15 * rint(F/W * 2^(bF-1)) / 2^(bF-1)   (bF-bit integer grid)
      F2 = f16(F/W * 2^15 - F1),  F3 = f16(F/W * 2^15 - F1 - F2)
  G (|G| <= 1), in units of 2^15:
      G1 = 32 * rint(G * 2^10)                     (11-bit integer grid)
      G2 = f16(G * 2^15 - G1)

Checked here: F1 and G1 are exact in f16 and every product F1*G1 is an
integer number of counts of 2^(30-(bF-1)-10), at most 2^(bF+9) of them (the
exactness of the main sum rests on both); F's slices hold it to about
2^-(bF+21) of W and G's to 2^-22, so G's representation bounds the form's
error per term; and the G grid can widen by one bit but not two before its
leading slice stops being exact in f16 (the width is traded against bF
under the main sum's 2^23-count limit).
"""
import numpy as np
import pytest

F32, F16 = np.float32, np.float16


def _fma32(a, b, c):
    """fmaf on FP32 arrays: the FP32 product is exact in FP64."""
    return (a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64)).astype(F32)


def _slice_f(x, W, bF):
    ls = F32(2.0 ** (bF - 1) / W)
    lu = F32(2.0 ** 15 / 2.0 ** (bF - 1))
    ku = F32(2.0 ** 15 / W)
    s1 = (np.rint(x * ls) * lu).astype(F32)
    r = _fma32(x, np.full_like(x, ku), -s1)
    h1 = s1.astype(F16)
    h2 = r.astype(F16)
    h3 = (r - h2.astype(F32)).astype(F16)
    return s1, h1, h2, h3


def _slice_g(g, lead_bits=11):
    gs = F32(2.0 ** (lead_bits - 1))
    gu = F32(2.0 ** 15 / 2.0 ** (lead_bits - 1))
    g1 = (np.rint(g * gs) * gu).astype(F32)
    h1 = g1.astype(F16)
    h2 = (g * F32(2.0 ** 15) - g1).astype(F16)
    return g1, h1, h2


@pytest.mark.parametrize("bF", [3, 5, 8, 9])
def test_f_slices(bF):
    rng = np.random.default_rng(bF)
    W = 8.0
    x = rng.uniform(-W, W, 200_000).astype(F32)
    s1, h1, h2, h3 = _slice_f(x, W, bF)
    assert np.array_equal(h1.astype(F32), s1)                       # F1 exact in f16
    rec = (h1.astype(np.float64) + h2.astype(np.float64) + h3.astype(np.float64)) * W / 2.0 ** 15
    err = np.max(np.abs(rec - x.astype(np.float64))) / W
    assert err <= 2.0 ** -(bF + 21)


def test_g_slices_set_the_error_budget():
    rng = np.random.default_rng(11)
    g = rng.uniform(-1.0, 1.0, 400_000).astype(F32)
    g1, h1, h2 = _slice_g(g)
    assert np.array_equal(h1.astype(F32), g1)                       # G1 exact in f16
    rec = (h1.astype(np.float64) + h2.astype(np.float64)) / 2.0 ** 15
    err = np.abs(rec - g.astype(np.float64))
    assert err.max() <= 2.0 ** -22 * 1.0001
    assert err.max() >= 2.0 ** -23                                  # the bound is reached
    # f16 holds integers up to 2^11 exactly: a 12-bit grid still fits, 13 bits do not
    g1b, h1b, _ = _slice_g(g, lead_bits=12)
    assert np.array_equal(h1b.astype(F32), g1b)
    g1c, h1c, _ = _slice_g(g, lead_bits=13)
    assert not np.array_equal(h1c.astype(F32), g1c)


@pytest.mark.parametrize("bF", [3, 9])
def test_leading_products_are_whole_counts(bF):
    rng = np.random.default_rng(100 + bF)
    W = 4.0
    s1, _, _, _ = _slice_f(rng.uniform(-W, W, 4096).astype(F32), W, bF)
    g1, _, _ = _slice_g(rng.uniform(-1.0, 1.0, 4096).astype(F32))
    count = 2.0 ** (30 - (bF - 1) - 10)
    prod = s1.astype(np.float64)[:, None] * g1.astype(np.float64)[None, :]
    n = prod / count
    assert np.array_equal(n, np.rint(n))
    assert np.abs(n).max() <= 2.0 ** (bF + 9)
