"""Tuned launches of the mixed kernel (GPU test).

A mixed-form call of at least 2^26 point*modes whose shape bucket has no
cache entry times nine candidate launches (2, 4 or 8 points per thread x 4, 8
or 16 target blocks per SM for the mode splits) on its own data and keeps the
fastest; later calls of the bucket reuse it.  Checked: the tuned call, the
cached call and the untuned default (tune mode 0) all stay within the mixed
form's bar against the oracle (1e-6 of the field RMS), the winner is one of
the candidates and lands in the cache file.
"""
import os

import numpy as np
import pytest

import oracle
from conftest import rel_err

pytestmark = pytest.mark.gpu


def test_tuned_mixed_call_within_its_bar(gsc, tmp_path):
    import ctypes
    from gstools_core import _native
    lib = _native.lib
    path = tmp_path / "tune.txt"
    assert lib.gsc_tune_cache_open(str(path).encode()) == 0
    assert lib.gsc_tune_set_mode(2) == 0
    rng = np.random.default_rng(21)
    P, N = 1 << 20, 2048
    cov = rng.standard_normal((3, N)) / np.sqrt(rng.chisquare(1, N)) / 5.0
    z1, z2 = rng.standard_normal(N), rng.standard_normal(N)
    pos = rng.uniform(0.0, 300.0, (3, P))
    idx = np.sort(rng.choice(P, 4096, replace=False))
    ref = oracle.summator(cov, z1, z2, np.ascontiguousarray(pos[:, idx]),
                          num_threads=os.cpu_count())
    try:
        for mode in (2, 1, 0):                    # tune, cached, fixed default
            assert lib.gsc_tune_set_mode(mode) == 0
            got = gsc.summate(cov, z1, z2, pos, form="mixed")
            err = rel_err(got[idx], ref)
            print(f"mode {mode}: {err:.3e}")
            assert err <= 1e-6
    finally:
        lib.gsc_tune_set_mode(2)
        lib.gsc_tune_cache_open(None)
    text = path.read_text()
    line = [l for l in text.splitlines() if "|mixed|d3s|p21|n12" in l]
    assert len(line) == 1
    R, W = (int(x) for x in line[0].split("\t")[1].split()[:2])
    assert R in (2, 4, 8) and W in (4, 8, 16)
