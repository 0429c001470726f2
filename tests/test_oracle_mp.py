"""The oracle against an independent high-precision evaluation (CPU).

The reference's own known answers (tests/test_oracle.py) pin the oracle for
2-D fields with few modes.  Here the same formulas are evaluated in
multiple-precision arithmetic (mpmath, 200 bits) for d = 1, 2, 3, Gaussian
and heavy-tailed (Student-t, nu = 1) spectra with phases beyond 1e4:

* the phase is the reference's FP64 dot product, formed in Python floats in
  the reference's order (((0 + k0 x0) + k1 x1) + k2 x2, no FMA;
  src/field.rs:57, src/short_vec.rs:30-33), so both sides see the same phase;
* cos, sin, z1 cos + z2 sin and the sum over modes are then taken exactly;
* the incompressible weights are formed in Python floats as the reference
  forms them (src/field.rs:138-152).

The oracle (FP64, glibc cos/sin, sequential sums) must agree within the
FP64 rounding bound of its own operations: 2^-52 times (three roundings per
term of the term magnitudes plus one per partial sum of the partial sums),
with an extra rounding per product for the weighted components.
"""
import numpy as np
import pytest

import oracle

mpmath = pytest.importorskip("mpmath")

mpmath.mp.prec = 200
U = 2.0 ** -52


def _inputs(seed, dim, n, p, heavy):
    rng = np.random.default_rng(seed)
    if heavy:
        cov = rng.standard_normal((dim, n)) / np.sqrt(rng.chisquare(1, n)) / 2.0
    else:
        cov = rng.normal(0.0, 0.5, (dim, n))
    z1, z2 = rng.standard_normal(n), rng.standard_normal(n)
    half = 1000.0 if heavy else 100.0
    pos = rng.uniform(-half, half, (dim, p))
    return cov, z1, z2, pos


def _phase(k, x):
    ph = 0.0
    for kd, xd in zip(k, x):
        ph = ph + kd * xd                  # Python floats: IEEE FP64, no FMA
    return ph


def _terms(cov, z1, z2, x):
    """Exact z1 cos + z2 sin per mode at the point x (mpf), and their sizes."""
    out, mags = [], []
    for j in range(cov.shape[1]):
        ph = mpmath.mpf(_phase(cov[:, j], x))
        c, s = mpmath.cos(ph), mpmath.sin(ph)
        out.append(mpmath.mpf(z1[j]) * c + mpmath.mpf(z2[j]) * s)
        mags.append(abs(z1[j] * float(c)) + abs(z2[j] * float(s)))
    return out, mags


@pytest.mark.parametrize("dim", [1, 2, 3])
@pytest.mark.parametrize("heavy", [False, True])
def test_summator_against_high_precision(dim, heavy):
    cov, z1, z2, pos = _inputs(10 * dim + heavy, dim, 48, 16, heavy)
    got = oracle.summator(cov, z1, z2, pos, num_threads=1)
    for i in range(pos.shape[1]):
        terms, mags = _terms(cov, z1, z2, pos[:, i])
        exact, partial_sizes, acc = mpmath.mpf(0), 0.0, mpmath.mpf(0)
        for t in terms:
            acc += t
            partial_sizes += abs(float(acc))
        exact = acc
        bound = U * (3.0 * sum(mags) + partial_sizes)
        assert abs(got[i] - float(exact)) <= bound, (i, got[i], float(exact), bound)


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("heavy", [False, True])
def test_summator_incompr_against_high_precision(dim, heavy):
    cov, z1, z2, pos = _inputs(100 + 10 * dim + heavy, dim, 40, 12, heavy)
    got = oracle.summator_incompr(cov, z1, z2, pos, num_threads=1)
    n = cov.shape[1]
    # weights as the reference forms them, in FP64 (src/field.rs:138-152)
    w = np.zeros((dim, n))
    for j in range(n):
        k = cov[:, j]
        k_2 = k[0] / _phase(k, k)
        w[0, j] = 1.0 - k[0] * k_2
        for c in range(1, dim):
            w[c, j] = -(k[c] * k_2)
    for i in range(pos.shape[1]):
        terms, mags = _terms(cov, z1, z2, pos[:, i])
        for c in range(dim):
            acc, partial_sizes, size = mpmath.mpf(0), 0.0, 0.0
            for j, t in enumerate(terms):
                acc += mpmath.mpf(w[c, j]) * t
                partial_sizes += abs(float(acc))
                size += abs(w[c, j]) * mags[j]
            bound = U * (4.0 * size + partial_sizes)
            assert abs(got[c, i] - float(acc)) <= bound, (c, i, got[c, i], float(acc), bound)


def test_heavy_tail_phases_are_large():
    """The heavy-tailed cases above do reach large phases."""
    cov, _, _, pos = _inputs(31, 3, 48, 16, True)
    ph = np.abs(cov.T @ pos)
    assert ph.max() > 1e4


@pytest.mark.parametrize("dim", [1, 2, 3])
def test_summator_fourier_against_high_precision(dim):
    """sum_j f_j (z1_j cos + z2_j sin) (src/field.rs:219-249), one more
    rounding per term for the spectrum factor."""
    cov, z1, z2, pos = _inputs(200 + dim, dim, 40, 12, False)
    sf = np.random.default_rng(dim).uniform(0.1, 2.0, cov.shape[1])
    got = oracle.summator_fourier(sf, cov, z1, z2, pos, num_threads=1)
    for i in range(pos.shape[1]):
        terms, mags = _terms(cov, z1, z2, pos[:, i])
        acc, partial_sizes = mpmath.mpf(0), 0.0
        for j, t in enumerate(terms):
            acc += mpmath.mpf(sf[j]) * t
            partial_sizes += abs(float(acc))
        bound = U * (4.0 * float(np.dot(sf, mags)) + partial_sizes)
        assert abs(got[i] - float(acc)) <= bound, (i, got[i], float(acc), bound)
