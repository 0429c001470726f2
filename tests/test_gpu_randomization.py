"""The normalised field of a randomization-method generator (GPU tests).

GSTools' generators wrap the summators in an affine step (a scale of the
summed modes, a mean).  ``randomization_field`` folds the scale into z1, z2
and adds the offset in place; checked against the oracle's sum scaled and
shifted the same way, on points and on a flattened mesh (routed to the
separable forms), for the plain bar (1e-12) and at tolerance 1e-6.
"""
import os

import numpy as np
import pytest

import oracle
from conftest import rel_err

pytestmark = pytest.mark.gpu
NT = os.cpu_count() or 1


def _case(seed, dim, n, p):
    rng = np.random.default_rng(seed)
    cov = rng.normal(0.0, 0.4, (dim, n))
    return cov, rng.standard_normal(n), rng.standard_normal(n), rng.uniform(-30, 30, (dim, p))


@pytest.mark.parametrize("tol,bar", [(None, 1e-12), (1e-6, 1e-6)])
def test_scalar_rand_meth(gsc, tol, bar):
    cov, z1, z2, pos = _case(1, 3, 700, 20000)
    var, mean = 2.5, -1.75
    scale = np.sqrt(var / cov.shape[1])
    out = gsc.randomization_field(cov, z1, z2, pos, scale, mean, tolerance=tol)
    ref = scale * oracle.summator(cov, z1, z2, pos, num_threads=NT) + mean
    # error relative to the scaled field's own spread
    assert float(np.max(np.abs(out - ref))) / float(np.std(ref)) <= bar


@pytest.mark.parametrize("tol,bar", [(None, 1e-12), (1e-6, 1e-6)])
def test_incompr_rand_meth_on_a_mesh(gsc, tol, bar):
    rng = np.random.default_rng(2)
    cov = rng.normal(0.0, 0.3, (3, 400))
    z1, z2 = rng.standard_normal(400), rng.standard_normal(400)
    axes = [np.linspace(0, 30, 24), np.linspace(-5, 5, 20), np.linspace(2, 9, 32)]
    pos = np.ascontiguousarray(np.array(np.meshgrid(*axes, indexing="ij")).reshape(3, -1))
    u_mean, var = 0.8, 1.3
    scale = u_mean * np.sqrt(var / cov.shape[1])
    out = gsc.randomization_field(cov, z1, z2, pos, scale, u_mean, incompr=True, tolerance=tol,
                                  timing=True)
    assert out.shape == (3, pos.shape[1]) and out.flags.f_contiguous
    ref = scale * oracle.summator_incompr(cov, z1, z2, pos, num_threads=NT)
    ref[0] += u_mean
    dev = ref - np.array([[u_mean], [0.0], [0.0]])
    assert float(np.max(np.abs(out - ref))) / float(np.sqrt(np.mean(dev ** 2))) <= bar
    names = {k for k, _ in gsc.last_timings()}
    assert ("sep_f64_dmma" if tol is None else "sep_tc_f16x5") in names


def test_zero_offset_and_unit_scale_is_summate(gsc):
    cov, z1, z2, pos = _case(3, 2, 300, 5000)
    a = gsc.randomization_field(cov, z1, z2, pos, 1.0)
    b = gsc.summate(cov, z1, z2, pos)
    assert np.array_equal(a, b)
