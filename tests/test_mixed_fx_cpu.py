"""The integer phase of the mixed form (mixed_fx.cu), restated in numpy (CPU).

For unstructured points the kernel forms kappa.x (kappa = k / 2 pi) modulo one
turn in 32-bit integer arithmetic: per dimension the coordinate as a 61-bit
fixed-point integer X' = rint(x 2^s) + 2^60 = Xh 2^29 + Xl, the mode's
B = kappa 2^(61 - s) as BI + BF 2^-32 with BI biased by 2^31, and

    theta = c_point + sum_d lo32(BI' Xh) + hi32(BF Xh) + hi32(BI' * 8 Xl)

(mod 2^32, units of 2^-32 turn), with the per-point constant c_point taking
out the bias and a per-mode constant phi folded into the mode's table.
Restated here with the same unsigned 32-bit operations and compared with the
exact rational phase of the FP64 inputs (Python integers): within 4 units
(2^-30 turns) in 1-3 dimensions, heavy-tailed wave numbers and coordinates of
either sign.  Then the table and polynomial evaluation of the term, and a
whole field against the oracle at the form's 1e-6 bar, in FP32 as the kernel
computes it.
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


def point_words(x, s):
    """(Xh, 8 Xl, per-point constant part) of one coordinate."""
    X = int(np.rint(np.ldexp(x, s)))
    Xp = X + (1 << 60)
    h, l = Xp >> 29, Xp & ((1 << 29) - 1)
    return h, (l << 3) & U32, (4 * l + ((h & 1) << 31)) & U32


def mode_words(k, s):
    """(BI', BF, phi part) of one wave-number component, as fx_mode_entry."""
    B = np.ldexp(k * INV2PI, 61 - s)
    assert abs(B) < 2 ** 31
    bq = int(np.rint(np.ldexp(B, 32)))
    bi, bf = bq >> 32, bq & U32
    return (bi + (1 << 31)) & U32, bf, Fraction((bq >> 1) & U32) + Fraction(bq & 1, 2)


def fx_theta(k, x, dim):
    """theta + 2^27 (uint32) of one point*mode and the per-mode phi (exact)."""
    s = [scale(abs(x[d])) for d in range(dim)]
    c = (0x08000000 + dim) & U32
    t = 0
    phi = Fraction(0)
    for d in range(dim):
        h, x8l, cd = point_words(x[d], s[d])
        bi, bf, ph = mode_words(k[d], s[d])
        c = (c - cd) & U32
        t = (t + ((bi * x8l) >> 32)) & U32
        t = (t + ((bf * h) >> 32)) & U32
        t = (t + bi * h) & U32
        phi += ph
    return (t + c) & U32, phi


def exact_turns(k, x, dim):
    """kappa.x in turns, exactly, from the FP64 values (kappa rounded as the
    kernel rounds it: fl(k * fl(1/2pi)))."""
    return sum(Fraction(float(np.float64(k[d]) * INV2PI)) * Fraction(float(x[d]))
               for d in range(dim))


@pytest.mark.parametrize("dim", [1, 2, 3])
def test_integer_phase_within_four_units(dim):
    rng = np.random.default_rng(dim)
    worst = 0.0
    for _ in range(3000):
        ext = 10.0 ** rng.uniform(-2, 4)
        x = rng.uniform(-ext, ext, dim)
        k = rng.standard_normal(dim) / np.sqrt(rng.chisquare(1)) * 10.0 ** rng.uniform(-2, 1)
        s = [scale(abs(x[d])) for d in range(dim)]
        if any(abs(np.ldexp(k[d] * INV2PI, 61 - s[d])) >= 2 ** 31 for d in range(dim)):
            continue
        t, phi = fx_theta(k, x, dim)
        # t = kappa.x + phi + 2^27 (table centring), modulo one turn
        want = (exact_turns(k, x, dim) * 2 ** 32 + phi + 2 ** 27) % (2 ** 32)
        err = float((Fraction(t) - want + 2 ** 31) % (2 ** 32) - 2 ** 31)
        worst = max(worst, abs(err))
    assert worst <= 4.0, worst


def fx_field(cov, z1, z2, pos):
    """The kernel's arithmetic for a scalar field, FP32 where the kernel
    uses FP32 (table, polynomial, Kahan tile sums, double-float total)."""
    dim, n = cov.shape
    P = pos.shape[1]
    s = [scale(np.abs(pos[d]).max()) for d in range(dim)]
    out = np.empty(P)
    f32 = np.float32
    rad = f32(np.float32(2 * np.pi) / np.float32(2 ** 36))
    tabs, words = [], []
    for j in range(n):
        ws = [mode_words(cov[d, j], s[d]) for d in range(dim)]
        phi = float(sum(w[2] for w in ws) % (2 ** 32))
        ang = (np.arange(16) * 2.0 ** 28 - phi) * (2 * np.pi / 2 ** 32)
        tr = (z1[j] * np.cos(ang) + z2[j] * np.sin(ang)).astype(f32)
        ti = (z1[j] * np.sin(ang) - z2[j] * np.cos(ang)).astype(f32)
        tabs.append((tr, ti))
        words.append(ws)
    for p in range(P):
        pw = [point_words(pos[d, p], s[d]) for d in range(dim)]
        c = (0x08000000 + dim) & U32
        for d in range(dim):
            c = (c - pw[d][2]) & U32
        hi = lo = f32(0)
        acc = cmp = f32(0)
        for j in range(n):
            t = c
            for d in range(dim):
                bi, bf, _ = words[j][d]
                t = (t + ((bi * pw[d][1]) >> 32)) & U32
                t = (t + ((bf * pw[d][0]) >> 32)) & U32
                t = (t + bi * pw[d][0]) & U32
            m = t >> 28
            u = np.uint32(((t << 4) ^ 0x80000000) & U32).view(np.int32)
            rr = f32(f32(u) * rad)
            r2 = f32(rr * rr)
            sn = f32(rr * r2 * f32(f32(r2 * f32(1 / 120)) + f32(-1 / 6)) + rr)
            cs = f32(r2 * f32(r2 * f32(r2 * f32(-1 / 720) + f32(1 / 24)) + f32(-0.5)) + f32(1))
            term = f32(tabs[j][0][m] * cs - tabs[j][1][m] * sn)
            y = f32(term - cmp)
            tt = f32(acc + y)
            cmp = f32(f32(tt - acc) - y)
            acc = tt
            if j % 32 == 31 or j == n - 1:
                sm = f32(hi + acc)
                bb = f32(sm - hi)
                e = f32(f32(hi - f32(sm - bb)) + f32(acc - bb))
                hi, lo = sm, f32(lo + e - cmp)
                acc = cmp = f32(0)
        out[p] = float(hi) + float(lo)
    return out


def test_field_against_the_oracle():
    rng = np.random.default_rng(11)
    n, P = 200, 300
    cov = rng.standard_normal((3, n)) / np.sqrt(rng.chisquare(1, n)) / 5.0   # heavy tails
    z1, z2 = rng.standard_normal(n), rng.standard_normal(n)
    pos = rng.uniform(0, 1000, (3, P))
    ref = oracle.summator(cov, z1, z2, pos)
    got = fx_field(cov, z1, z2, pos)
    err = np.abs(got - ref).max() / np.sqrt(np.mean(ref ** 2))
    assert err <= 1e-6, err

