"""The leading-grid bound and the exact output conversion of the x5 form,
restated in numpy (CPU).

The kernel (separable_tc.cu: wnorm_block, x5_lead_bound) bounds the leading
products of a run of n modes by

    B(bF) = 2049 (2^(bF-1) (1 + 2^-21) S1 + 0.7072 n),
    S1 = sum_j |w_j| / W over those modes,  W = 2^e > max_j |w_j|,

counts (leading grid 2^(bF-1)); its checks at chunk boundaries rest on this:
no partial sum inside a chunk moves further from the boundary's value than
B over the chunk's modes, in any mode order and at any grid point.  Checked
here on integer grids built as the kernel builds them: random, coherent and
equal-magnitude weights, the largest partial sum over every prefix of
several mode orders stays within B.  The output conversion i32_to_f64_pow2
(integer operations only: count of leading zeros and 32-bit funnel shifts)
is restated and compared with exact scaling.
"""
import numpy as np
import pytest

TWO24 = 2.0 ** 24


def lead_bound(bf, s1, n):
    return 2049.0 * (2.0 ** (bf - 1) * (1.0 + 2.0 ** -21) * s1 + 0.7072 * n)


def pick_bf(w):
    """The widest grid whose bound over all the modes stays within 2^24
    counts (so every partial sum of a run of them does), W, S1."""
    mx = np.abs(w).max()
    e = int(np.frexp(mx)[1]) if mx > 0 else 0
    W = 2.0 ** e
    s1 = np.abs(w).sum() / W * (1 + 1e-12)
    bf = 9
    while bf > 3 and lead_bound(bf, s1, len(w)) > TWO24:
        bf -= 1
    return bf, lead_bound(bf, s1, len(w)) > TWO24, W, s1


def lead_counts(w, phase_rows, g, bf, W):
    """Integer leading products of the rows F = w e^{i phase} (one row per
    phase vector) against columns G (unit modulus or less), counts per mode."""
    F = (w[None, :] * np.exp(1j * phase_rows)).astype(np.complex64)
    Gc = g.astype(np.complex64)
    iF_re = np.rint(F.real / W * 2.0 ** (bf - 1))
    iF_im = np.rint(F.imag / W * 2.0 ** (bf - 1))
    iG_re = np.rint(Gc.real * 2.0 ** 11)
    iG_im = np.rint(-Gc.imag * 2.0 ** 11)
    # F[b, 2j] G[c, 2j] + F[b, 2j+1] G[c, 2j+1] with G = (Re C, -Im C)
    return iF_re[:, None, :] * iG_re[None, :, :] + iF_im[:, None, :] * iG_im[None, :, :]


@pytest.mark.parametrize("kind", ["random", "coherent", "equal"])
def test_partial_sums_stay_within_the_bound(kind):
    rng = np.random.default_rng({"random": 1, "coherent": 2, "equal": 3}[kind])
    n = 1500
    if kind == "random":
        w = rng.standard_normal(n) - 1j * rng.standard_normal(n)
    elif kind == "coherent":
        w = np.ones(n, dtype=complex)
    else:
        w = 0.999 * np.exp(1j * rng.uniform(0, 2 * np.pi, n))
    bf, over, W, s1 = pick_bf(w)
    assert not over
    bound = lead_bound(bf, s1, n)
    assert bound <= TWO24
    # rows at phase 0 (in phase: the coherent extreme) and random phases
    rows = np.vstack([np.zeros(n), rng.uniform(0, 2 * np.pi, (3, n))])
    g = np.vstack([np.ones(n), np.exp(1j * rng.uniform(0, 2 * np.pi, (3, n)))])
    c = lead_counts(w, rows, g, bf, W)
    worst = 0.0
    for order in [np.arange(n), rng.permutation(n), np.argsort(-np.abs(w))]:
        worst = max(worst, np.abs(np.cumsum(c[:, :, order], axis=2)).max())
    assert worst <= bound
    if kind == "coherent":
        # the bound is tight to its rounding allowance for in-phase weights
        assert worst >= 0.75 * bound


def i32_to_f64_pow2(v, q):
    """separable_tc.cu i32_to_f64_pow2: clz, funnel shifts, exponent bits."""
    u = v & 0xFFFFFFFF
    sign = u & 0x80000000
    a = ((-v) & 0xFFFFFFFF) if v < 0 else v
    lz = 32 - a.bit_length()
    sh = lz + 21
    if sh >= 32:
        mhi, mlo = (a << (sh - 32)) & 0xFFFFFFFF, 0
    else:
        mhi, mlo = (a >> (32 - sh)) & 0xFFFFFFFF, (a << sh) & 0xFFFFFFFF
    hi = sign | (((1023 + 31 - lz + q) & 0xFFF) << 20) | (mhi & 0xFFFFF)
    if a == 0:
        hi, mlo = sign, 0
    if v == -(2 ** 31):
        return float("nan")
    return float(np.array((hi << 32) | mlo, dtype=np.uint64).view(np.float64))


def test_int_to_f64_conversion_is_exact():
    rng = np.random.default_rng(5)
    vals = [0, 1, -1, 2, 3, -3, 2 ** 20, 2 ** 20 - 1, 2 ** 30, -(2 ** 30) - 7,
            2 ** 31 - 1] + list(rng.integers(-2 ** 31 + 1, 2 ** 31, 2000))
    for q in (-40, -20, -1, 0, 7):
        for v in vals:
            assert i32_to_f64_pow2(int(v), q) == np.ldexp(float(v), q)
    assert np.isnan(i32_to_f64_pow2(-(2 ** 31), 0))          # the NaN sentinel


def test_fixed_point_output_keeps_the_main_sum_exact():
    """T = rint(M * 2^(bF-14)) + rint(C * 2^(bF-14)): the main sum M (whole
    counts of 2^(20-bF)) enters exactly as 64 per count; the cross total C is
    rounded to 1/64 count.  The FP32 sum M + C that this replaces rounds at
    the field's magnitude."""
    rng = np.random.default_rng(6)
    bf = 5
    counts = rng.integers(-2 ** 24 + 1, 2 ** 24, 5000)
    M = (counts * 2.0 ** (20 - bf)).astype(np.float32)
    assert np.array_equal(M.astype(np.float64), counts * 2.0 ** (20 - bf))
    C = (rng.standard_normal(5000) * 2.0 ** (20 - bf) * 2.0 ** 18).astype(np.float32)
    s = np.float32(2.0 ** (bf - 14))
    T = np.rint(M * s).astype(np.int64) + np.rint(C * s).astype(np.int64)
    assert np.all(np.abs(T) < 2 ** 31)
    exact = (M.astype(np.float64) + C.astype(np.float64)) * 2.0 ** (bf - 14)
    assert np.abs(T - exact).max() <= 0.5
    f32 = (M + C).astype(np.float64) * 2.0 ** (bf - 14)
    assert np.abs(f32 - exact).max() > 8.0       # FP32 rounding: many 1/64 counts
