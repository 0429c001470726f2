"""The operand slicing of the x5 tensor-core form, restated in numpy (CPU).

The kernel (separable_tc.cu: slice3x2 for the rows F, gtab_x5_entry for
the columns G) represents each FP32 factor by f16 slices so that the
leading product F1*G1 is an integer multiple of a fixed unit:

  F / W (|F/W| <= 1), in units of 2^15:
      F1 = 2^15 * rint(F/W * 2^(bF-1)) / 2^(bF-1)   (bF-bit integer grid)
      F2 = f16(F/W * 2^15 - F1),  F3 = f16(F/W * 2^15 - F1 - F2)
  G (|G| <= 1), in units of 2^15:
      G1 = 16 * rint(G * 2^11)                     (12-bit integer grid)
      G2 = f16(G * 2^15 - G1)

Checked here: F1 and G1 are exact in f16 and every product F1*G1 is an
integer number of counts of 2^(30-(bF-1)-11), at most 2^(bF+10) of them (the
exactness of the main sum rests on both); F's slices hold it to about
2^-(bF+21) of W and G's to 2^-24; the G grid is the widest whose leading
slice f16 holds exactly (13 bits are not); and, on a small grid, the form's
representation error (slices of FP32 factors, leading sum exact, the rest
in FP64) stays within the RMS and max bars the GPU tests hold the kernel to,
with the 12-bit G grid about 1.6 times tighter than an 11-bit one.
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


def _slice_g(g, lead_bits=12):
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
    assert err.max() <= 2.0 ** -24 * 1.0001
    assert err.max() >= 2.0 ** -25                                  # the bound is reached
    # f16 holds integers up to 2^11 exactly: 13 bits no longer fit
    g1c, h1c, _ = _slice_g(g, lead_bits=13)
    assert not np.array_equal(h1c.astype(F32), g1c)


@pytest.mark.parametrize("bF", [3, 9])
def test_leading_products_are_whole_counts(bF):
    rng = np.random.default_rng(100 + bF)
    W = 4.0
    s1, _, _, _ = _slice_f(rng.uniform(-W, W, 4096).astype(F32), W, bF)
    g1, _, _ = _slice_g(rng.uniform(-1.0, 1.0, 4096).astype(F32))
    count = 2.0 ** (30 - (bF - 1) - 11)
    prod = s1.astype(np.float64)[:, None] * g1.astype(np.float64)[None, :]
    n = prod / count
    assert np.array_equal(n, np.rint(n))
    assert np.abs(n).max() <= 2.0 ** (bF + 10)


def _lead_bits_f(typ, lead_bits_g):
    """bF as the normaliser picks it: 6 sigma of the main sum below 2^23 counts."""
    bf = int(np.floor(23 + 2 - lead_bits_g - np.log2(max(typ, 1.0))))
    return min(max(bf, 3), 9)


def _emulated_errors(incompr, lead_bits_g, shape=(3, 40, 40), n=1024, seed=5):
    """Error of the x5 representation on a 3-D grid, relative to the field RMS.

    Rows F = (z1 - i z2) e^{i kx x} e^{i ky y} rounded to FP32 (the on-chip
    product), columns G = w e^{i kz z} rounded to FP32 (the table), each
    sliced as above; the sliced products summed in FP64 (the main sum is
    exact on the device, the cross sums are drained long before FP32
    rounding matters)."""
    rng = np.random.default_rng(seed)
    cov = rng.normal(0.0, np.sqrt(2.0) / 8.0, (3, n))
    z1, z2 = rng.standard_normal(n), rng.standard_normal(n)
    ax = [np.arange(s, dtype=np.float64) for s in shape]
    s = z1 - 1j * z2
    W = 2.0 ** np.ceil(np.log2(np.abs(s).max()))
    bf = _lead_bits_f(6.0 * np.sqrt((np.abs(s) ** 2).sum() / 2.0) / W, lead_bits_g)
    ex, ey, ez = (np.exp(1j * np.outer(a, k)) for a, k in zip(ax, cov))
    k2 = (cov ** 2).sum(0)

    def fs(v):
        return sum(h.astype(np.float64) for h in _slice_f(v, W, bf)[1:]) * W / 2.0 ** 15

    def gs(v):
        return sum(h.astype(np.float64) for h in _slice_g(v, lead_bits_g)[1:]) / 2.0 ** 15

    errs, refs = [], []
    for c in (range(3) if incompr else [None]):
        w = np.ones(n) if c is None else (float(c == 0) - cov[c] * cov[0] / k2)
        G = w[None, :] * ez
        Gq = gs(G.real.astype(F32)) - 1j * gs((-G.imag).astype(F32))
        for a in range(shape[0]):
            F = (s * ex[a])[None, :] * ey
            Ff = F.astype(np.complex64)
            got = fs(Ff.real) @ Gq.real.T - fs(Ff.imag) @ Gq.imag.T
            ref = (F @ G.T).real
            errs.append((got - ref).ravel())
            refs.append(ref.ravel())
    e, r = np.concatenate(errs), np.concatenate(refs)
    rms = np.sqrt(np.mean(r ** 2))
    return float(np.sqrt(np.mean(e ** 2)) / rms), float(np.abs(e).max() / rms)


@pytest.mark.parametrize("incompr", [False, True])
def test_emulated_error_budget(incompr):
    rms12, max12 = _emulated_errors(incompr, 12)
    rms11, _ = _emulated_errors(incompr, 11)
    assert rms12 <= 1.5e-7 and max12 <= 1e-6
    assert rms11 / rms12 >= 1.4
