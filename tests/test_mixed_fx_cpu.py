"""The integer phase of the mixed form (mixed_fx.cu), restated in numpy (CPU).

For unstructured points the kernel forms kappa.x (kappa = k / 2 pi) modulo one
turn in 32-bit integer arithmetic: per dimension the coordinate as a 61-bit
fixed-point integer X' = rint(x 2^s) + 2^60 = Xh 2^29 + Xl, the mode's
B = kappa 2^(61 - s) as BI + BF 2^-32 with BI biased by 2^31, and

    theta = c_point + sum_d lo32(BI' Xh) + hi32(BF Xh) + hi32(BI' * 8 Xl)

(mod 2^32, units of 2^-32 turn), with the per-point constant c_point taking
out the bias (and adding 2^27 + 16, which centres and rounds the remainder)
and a per-mode constant phi folded into the mode's table.  When every mode of
a call has |BI| < 2^20, the kernel forms sum_d BI Xl 2^-29 instead as a
chain of FP32 fused multiply-adds of the signed BI and fl(Xl 2^-29) into the
mantissa of 1.5 2^23, rounded to an integer; that form is restated here as
well.
Restated here with the same unsigned 32-bit operations and compared with the
exact rational phase of the FP64 inputs (Python integers): within 4 units
(2^-30 turns) in 1-3 dimensions, heavy-tailed wave numbers and coordinates of
either sign.  Then the table and polynomial evaluation of the term (the remainder read
from the phase word's bits as the mantissa of a float in [1, 2)), the sums of
eight modes' terms, and a whole field against the oracle at the form's 1e-6
bar, in FP32 as the kernel computes it.
"""
from fractions import Fraction

import numpy as np
import pytest

import oracle

U32 = 0xFFFFFFFF
INV2PI = 0.15915494309189535            # fl(1 / (2 pi)), as dfturns.cuh


def scale(maxabs):
    e = int(np.frexp(maxabs)[1]) if maxabs > 0 else 0
    return 60 - e


def point_words(x, s, small=False):
    """(Xh, 8 Xl or fl(Xl 2^-29), per-point constant part) of one coordinate."""
    X = int(np.rint(np.ldexp(x, s)))
    Xp = X + (1 << 60)
    h, l = Xp >> 29, Xp & ((1 << 29) - 1)
    if small:
        return h, np.float32(np.float32(l) * np.float32(2.0 ** -29)), ((h & 1) << 31) & U32
    return h, (l << 3) & U32, (4 * l + ((h & 1) << 31)) & U32


MAGIC_BITS = 0x4B400000          # bits of 1.5 2^23
TILE = 128                       # modes per accumulation tile
SMALL_BI = 1 << 20


def small_products(bis_biased, xlfs):
    """round(sum_d BI Xl 2^-29) + 0x4B400000 as the kernel's chain of FP32
    fused multiply-adds leaves it (each step exact in FP64 before its one
    rounding to FP32)."""
    v = np.float32(12582912.0)
    for bi_biased, xlf in zip(bis_biased, xlfs):
        bi = np.float32(int(bi_biased) - (1 << 31))
        v = np.float32(np.float64(bi) * np.float64(xlf) + np.float64(v))
    return int(v.view(np.uint32))


def mode_words(k, s):
    """(BI', BF, phi part) of one wave-number component, as fx_mode_entry."""
    B = np.ldexp(k * INV2PI, 61 - s)
    assert abs(B) < 2 ** 31
    bq = int(np.rint(np.ldexp(B, 32)))
    bi, bf = bq >> 32, bq & U32
    return (bi + (1 << 31)) & U32, bf, Fraction((bq >> 1) & U32) + Fraction(bq & 1, 2)


def fx_theta(k, x, dim, small=False):
    """theta + 2^27 + 16 (uint32) of one point*mode and the per-mode phi (exact)."""
    s = [scale(abs(x[d])) for d in range(dim)]
    c = (0x08000000 + 16 + dim) & U32
    t = 0
    phi = Fraction(0)
    bis, xls = [], []
    for d in range(dim):
        h, xl, cd = point_words(x[d], s[d], small)
        bi, bf, ph = mode_words(k[d], s[d])
        c = (c - cd) & U32
        bis.append(bi)
        xls.append(xl)
        if not small:
            t = (t + ((bi * xl) >> 32)) & U32
        t = (t + ((bf * h) >> 32)) & U32
        t = (t + bi * h) & U32
        phi += ph
    if small:
        t = (t + small_products(bis, xls) - MAGIC_BITS) & U32
    return (t + c) & U32, phi


def exact_turns(k, x, dim):
    """kappa.x in turns, exactly, from the FP64 values (kappa rounded as the
    kernel rounds it: fl(k * fl(1/2pi)))."""
    return sum(Fraction(float(np.float64(k[d]) * INV2PI)) * Fraction(float(x[d]))
               for d in range(dim))


@pytest.mark.parametrize("small", [False, True])
@pytest.mark.parametrize("dim", [1, 2, 3])
def test_integer_phase_within_four_units(dim, small):
    rng = np.random.default_rng(dim)
    worst = 0.0
    for _ in range(3000):
        ext = 10.0 ** rng.uniform(-2, 4)
        x = rng.uniform(-ext, ext, dim)
        k = rng.standard_normal(dim) / np.sqrt(rng.chisquare(1)) * 10.0 ** rng.uniform(-2, 1)
        s = [scale(abs(x[d])) for d in range(dim)]
        lim = SMALL_BI if small else 2 ** 31
        if any(abs(np.ldexp(k[d] * INV2PI, 61 - s[d])) >= lim - 1 for d in range(dim)):
            continue
        t, phi = fx_theta(k, x, dim, small)
        # t = kappa.x + phi + 2^27 + 16 (table centring, remainder rounding),
        # modulo one turn
        want = (exact_turns(k, x, dim) * 2 ** 32 + phi + 2 ** 27 + 16) % (2 ** 32)
        err = float((Fraction(t) - want + 2 ** 31) % (2 ** 32) - 2 ** 31)
        worst = max(worst, abs(err))
    assert worst <= 4.0, worst


PI8 = np.pi / 8
# the kernel's minimax coefficients (FP32) of sin(r pi/8) / r and cos(r pi/8)
# as polynomials in r^2, |r| <= 1/2
S1, S3, S5 = (np.float32(v) for v in (0.39269909262657166, -0.01009317860007286,
                                      7.771774107823148e-05))
C0, C2, C4 = (np.float32(v) for v in (1.0, -0.07710610330104828, 0.000988987972959876))


def fma32(a, b, c):
    """FP32 fused multiply-add: the product of two floats is exact in FP64."""
    return np.float32(np.float64(a) * np.float64(b) + np.float64(c))


def fx_term(t, tab):
    """The term of one point*mode from its phase word t = theta + 2^27 + 16."""
    f32 = np.float32
    m = t >> 28
    r = f32(np.uint32(0x3F800000 | ((t >> 5) & 0x7FFFFF)).view(np.float32) - f32(1.5))
    r2 = f32(r * r)
    sn = f32(r * fma32(r2, fma32(r2, S5, S3), S1))
    cs = fma32(r2, fma32(r2, C4, C2), C0)
    return fma32(tab[0][m], cs, -f32(tab[1][m] * sn))


def test_polynomials_within_their_bound():
    """The FP32 coefficients, evaluated exactly, stay within 6e-9 of sin and
    cos over |r| <= 1/2 (sixteenths of a turn)."""
    r = np.linspace(-0.5, 0.5, 200001)
    u = r * r
    sn = r * (np.float64(S1) + u * (np.float64(S3) + u * np.float64(S5)))
    cs = np.float64(C0) + u * (np.float64(C2) + u * np.float64(C4))
    assert np.max(np.abs(sn - np.sin(PI8 * r))) < 6e-9
    assert np.max(np.abs(cs - np.cos(PI8 * r))) < 6e-9


def test_remainder_float_and_polynomials():
    """The remainder float is exact, within 2^-28 turn of the phase's
    remainder, and the FP32 evaluation gives e^{i theta} within the FP32
    table entries' rounding."""
    rng = np.random.default_rng(5)
    t = rng.integers(0, 2 ** 32, 20000, dtype=np.uint64).astype(np.uint32)
    m = t >> 28
    rem = (t.astype(np.int64) & ((1 << 28) - 1)) - 2 ** 27 - 16     # theta - m 2^28
    r = (np.uint32(0x3F800000) | ((t >> 5) & 0x7FFFFF)).view(np.float32).astype(np.float64) - 1.5
    assert np.all(np.abs(r * 2 ** 28 - rem) <= 16)                   # units of 2^-32 turn
    theta = (m.astype(np.float64) * 2 ** 28 + rem) * (2 * np.pi / 2 ** 32)
    tab = (np.cos(np.arange(16) * np.pi / 8).astype(np.float32),
           np.sin(np.arange(16) * np.pi / 8).astype(np.float32))
    # T = e^{2 pi i m/16}: Re(T e^{ir}) = cos(theta); T = -i e^{...}: sin(theta)
    got_c = np.array([fx_term(int(v), tab) for v in t])
    tab_s = (tab[1], -tab[0])
    got_s = np.array([fx_term(int(v), tab_s) for v in t])
    assert np.max(np.abs(got_c - np.cos(theta))) < 3e-7          # FP32 table entries
    assert np.max(np.abs(got_s - np.sin(theta))) < 3e-7


def fx_field(cov, z1, z2, pos):
    """The kernel's arithmetic for a scalar field, FP32 where the kernel
    uses FP32 (table, polynomial, sums of eight modes, Kahan tile sums,
    double-float total)."""
    dim, n = cov.shape
    P = pos.shape[1]
    s = [scale(np.abs(pos[d]).max()) for d in range(dim)]
    out = np.empty(P)
    f32 = np.float32
    tabs, words = [], []
    small = all(abs(int(mode_words(cov[d, j], s[d])[0]) - (1 << 31)) < SMALL_BI
                for d in range(dim) for j in range(n))
    for j in range(n):
        ws = [mode_words(cov[d, j], s[d]) for d in range(dim)]
        phi = float(sum(w[2] for w in ws) % (2 ** 32))
        ang = (np.arange(16) * 2.0 ** 28 - phi) * (2 * np.pi / 2 ** 32)
        tr = (z1[j] * np.cos(ang) + z2[j] * np.sin(ang)).astype(f32)
        ti = (z1[j] * np.sin(ang) - z2[j] * np.cos(ang)).astype(f32)
        tabs.append((tr, ti))
        words.append(ws)
    for p in range(P):
        pw = [point_words(pos[d, p], s[d], small) for d in range(dim)]
        c = (0x08000000 + 16 + dim) & U32
        for d in range(dim):
            c = (c - pw[d][2]) & U32
        hi = lo = f32(0)
        for t0 in range(0, n, TILE):
            acc = cmp = f32(0)
            terms = []
            for j in range(t0, min(n, t0 + TILE)):
                t = c
                if small:
                    t = (t + small_products([words[j][d][0] for d in range(dim)],
                                            [pw[d][1] for d in range(dim)]) - MAGIC_BITS) & U32
                for d in range(dim):
                    bi, bf, _ = words[j][d]
                    if not small:
                        t = (t + ((bi * pw[d][1]) >> 32)) & U32
                    t = (t + ((bf * pw[d][0]) >> 32)) & U32
                    t = (t + bi * pw[d][0]) & U32
                terms.append(fx_term(t, tabs[j]))
            if len(terms) == TILE:        # a full tile: groups of eight modes
                groups = []
                for q in range(0, TILE, 8):
                    pairs = [f32(terms[q + 2 * k] + terms[q + 2 * k + 1]) for k in range(4)]
                    pend = f32(f32(pairs[0] + pairs[1]) + pairs[2])
                    groups.append(f32(pend + pairs[3]))
            else:                         # the last, shorter tile: pairs
                groups = [terms[q] if q + 1 == len(terms) else f32(terms[q] + terms[q + 1])
                          for q in range(0, len(terms), 2)]
            for a in groups:
                y = f32(a - cmp)
                tt = f32(acc + y)
                cmp = f32(f32(tt - acc) - y)
                acc = tt
            sm = f32(hi + acc)
            bb = f32(sm - hi)
            e = f32(f32(hi - f32(sm - bb)) + f32(acc - bb))
            hi, lo = sm, f32(lo + e - cmp)
        out[p] = float(hi) + float(lo)
    return out


@pytest.mark.parametrize("extent", [1000.0, 2e6])
def test_field_against_the_oracle(extent):
    """A heavy-tailed field; at the larger extent some |BI| reach 2^20 and
    the field takes the integer high products."""
    rng = np.random.default_rng(11)
    n, P = 200, 300
    cov = rng.standard_normal((3, n)) / np.sqrt(rng.chisquare(1, n)) / 5.0   # heavy tails
    z1, z2 = rng.standard_normal(n), rng.standard_normal(n)
    pos = rng.uniform(0, extent, (3, P))
    ref = oracle.summator(cov, z1, z2, pos)
    got = fx_field(cov, z1, z2, pos)
    err = np.abs(got - ref).max() / np.sqrt(np.mean(ref ** 2))
    assert err <= 1e-6, err

