"""Positions and modes read in place from host memory (GPU tests).

Where the GPU reads pageable host memory coherently (cudaDevAttrPageableMemoryAccess,
GB300's host link), host-array calls leave C-ordered positions and dense
modes where they are: the point kernels read the positions in place and the
record kernel the modes; other layouts go through the pinned staging.  Both
routes feed the same kernels the same values, so their results must agree
bit for bit; a seeded subset of points is also checked against the oracle at
the form's bar (reference src/field.rs:37-65, :97-182).
"""
import os

import numpy as np
import pytest

import oracle
from conftest import rel_err

pytestmark = pytest.mark.gpu
NT = os.cpu_count() or 1


def _case(seed, n, p):
    rng = np.random.default_rng(seed)
    cov = rng.standard_normal((3, n)) / np.sqrt(rng.chisquare(1, n)) / 5.0
    z1, z2 = rng.standard_normal(n), rng.standard_normal(n)
    pos = rng.uniform(0.0, 1000.0, (3, p))
    return cov, z1, z2, pos


@pytest.mark.parametrize("form,bar", [("mixed", 1e-6), ("plain", 1e-12)])
@pytest.mark.parametrize("kind", ["scalar", "incompr"])
@pytest.mark.parametrize("p", [300, 20_000, 1 << 22])     # 7 KB, 480 KB and 96 MiB of positions
def test_positions_in_place_match_staged(gsc, form, bar, kind, p):
    cov, z1, z2, pos = _case(5, 64, p)
    assert pos.flags.c_contiguous and cov.flags.c_contiguous
    staged = np.asfortranarray(pos)                   # rows not contiguous: staged
    fn = gsc.summate_incompr if kind == "incompr" else gsc.summate
    got = fn(cov, z1, z2, pos, form=form)
    ref = fn(cov, z1, z2, staged, form=form)
    assert np.array_equal(got, ref, equal_nan=True)
    # modes in a strided layout go through the staging as well
    zz = np.empty((z1.size, 2))
    zz[:, 0], zz[:, 1] = z1, z2                       # z1, z2 with a stride of 2
    ref_m = fn(np.asfortranarray(cov), zz[:, 0], zz[:, 1], staged, form=form)
    assert np.array_equal(got, ref_m, equal_nan=True)
    idx = np.sort(np.random.default_rng(6).choice(pos.shape[1], min(p, 4096), replace=False))
    sub = np.ascontiguousarray(pos[:, idx])
    if kind == "incompr":
        want = oracle.summator_incompr(cov, z1, z2, sub, num_threads=NT)
        err = rel_err(got[:, idx], want)
    else:
        want = oracle.summator(cov, z1, z2, sub, num_threads=NT)
        err = rel_err(got[idx], want)
    assert err <= bar, f"{form} {kind}: {err:.3e}"
