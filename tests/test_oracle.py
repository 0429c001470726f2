"""The CPU oracle against the reference's own known answers (CPU only).

Pins oracle/field_oracle.c to src/field.rs's test module:
  test_summate_2d          :359-382  exact
  test_summate_fourier_2d  :334-357  exact
  test_summate_incompr_2d  :384-430  assert_ulps_eq!(max_ulps = 6)
then checks the layout, threading and dimension handling the reference has.
"""
import numpy as np
import pytest

import oracle
from conftest import ulps_eq


def test_summate_golden_exact(goldens):
    g = goldens
    out = oracle.summator(g["setup.cov_samples"], g["setup.z_1"], g["setup.z_2"], g["setup.pos"])
    assert out.shape == (8,)
    # bit for bit, like the reference's assert_eq!
    assert out.tobytes() == g["expected.summate"].tobytes()


def test_summate_fourier_golden_exact(goldens):
    g = goldens
    out = oracle.summator_fourier(g["fourier.spectrum_factor"], g["fourier.modes"],
                                  g["fourier.z_1"], g["fourier.z_2"], g["fourier.pos"])
    assert out.tobytes() == g["expected.summate_fourier"].tobytes()


@pytest.mark.parametrize("threads", [None, 1, 4])
def test_summate_incompr_golden_ulps(goldens, threads):
    g = goldens
    out = oracle.summator_incompr(g["setup.cov_samples"], g["setup.z_1"], g["setup.z_2"],
                                  g["setup.pos"], num_threads=threads)
    exp = g["expected.summate_incompr"]
    assert out.shape == exp.shape == (3, 8)
    bad = [(i, j) for i in range(3) for j in range(8) if not ulps_eq(out[i, j], exp[i, j], 6)]
    assert not bad, bad


def test_summate_threads_bit_identical():
    rng = np.random.default_rng(1)
    cov = rng.normal(0, 1.0, (3, 257))
    z1, z2 = rng.standard_normal(257), rng.standard_normal(257)
    pos = rng.uniform(-50, 50, (3, 1001))
    a = oracle.summator(cov, z1, z2, pos)
    b = oracle.summator(cov, z1, z2, pos, num_threads=7)
    assert a.tobytes() == b.tobytes()


def test_summate_strided_views_identical():
    """Any strides: F-order, transposed copies and sliced views give the same bits."""
    rng = np.random.default_rng(2)
    cov = rng.normal(0, 0.3, (2, 100))
    z1, z2 = rng.standard_normal(100), rng.standard_normal(100)
    pos = rng.uniform(0, 100, (2, 300))
    ref = oracle.summator(cov, z1, z2, pos)
    covf, posf = np.asfortranarray(cov), np.asfortranarray(pos)
    assert oracle.summator(covf, z1, z2, posf).tobytes() == ref.tobytes()
    big = np.zeros((2, 600))
    big[:, ::2] = pos
    zz1 = np.zeros(200)
    zz1[::2] = z1
    assert oracle.summator(cov, zz1[::2], z2, big[:, ::2]).tobytes() == ref.tobytes()
    assert oracle.summator(cov.T.copy().T, z1, z2, pos.T.copy().T).tobytes() == ref.tobytes()


@pytest.mark.parametrize("dim", [1, 2, 3])
def test_summate_matches_numpy_float64(dim):
    rng = np.random.default_rng(10 + dim)
    n, p = 64, 200
    cov = rng.normal(0, 0.5, (dim, n))
    z1, z2 = rng.standard_normal(n), rng.standard_normal(n)
    pos = rng.uniform(-20, 20, (dim, p))
    ph = cov.T @ pos                       # (n, p)
    ref = (z1[:, None] * np.cos(ph) + z2[:, None] * np.sin(ph)).sum(axis=0)
    out = oracle.summator(cov, z1, z2, pos)
    np.testing.assert_allclose(out, ref, rtol=0, atol=1e-12 * max(1.0, np.sqrt(np.mean(ref ** 2))))


@pytest.mark.parametrize("dim", [2, 3])
def test_incompr_matches_numpy_float64(dim):
    rng = np.random.default_rng(20 + dim)
    n, p = 150, 100
    cov = rng.normal(0, 0.5, (dim, n))
    z1, z2 = rng.standard_normal(n), rng.standard_normal(n)
    pos = rng.uniform(-20, 20, (dim, p))
    ph = cov.T @ pos
    z12 = z1[:, None] * np.cos(ph) + z2[:, None] * np.sin(ph)          # (n, p)
    kk = (cov ** 2).sum(axis=0)
    proj = -cov * (cov[0] / kk)[None, :]                                # (d, n)
    proj[0] += 1.0
    ref = proj @ z12
    for threads in (None, 3):
        out = oracle.summator_incompr(cov, z1, z2, pos, num_threads=threads)
        np.testing.assert_allclose(out, ref, rtol=0, atol=1e-12 * np.sqrt(np.mean(ref ** 2)))


def test_incompr_divergence_free_in_spectral_space():
    """Each mode's projector p(k) = e1 - k k0/|k|^2 is orthogonal to k."""
    rng = np.random.default_rng(5)
    cov = rng.normal(0, 1, (3, 40))
    kk = (cov ** 2).sum(axis=0)
    proj = -cov * (cov[0] / kk)[None, :]
    proj[0] += 1.0
    assert np.max(np.abs((proj * cov).sum(axis=0))) < 1e-14


def test_incompr_rejects_other_dims():
    rng = np.random.default_rng(0)
    for dim in (1, 4):
        with pytest.raises(ValueError):
            oracle.summator_incompr(rng.normal(size=(dim, 5)), np.ones(5), np.ones(5),
                                    rng.normal(size=(dim, 3)))


def test_empty_inputs():
    cov = np.zeros((3, 0))
    z = np.zeros(0)
    pos = np.ones((3, 4))
    assert np.array_equal(oracle.summator(cov, z, z, pos), np.zeros(4))
    assert oracle.summator(np.ones((3, 2)), np.ones(2), np.ones(2), np.zeros((3, 0))).shape == (0,)
    assert np.array_equal(oracle.summator_incompr(cov, z, z, pos), np.zeros((3, 4)))
