"""Result arrays from the pinned host pool (GPU tests).

Host-array calls return new arrays, as the reference does (src/lib.rs:47,
64); from 64 KiB up their memory is a pinned block of the library's pool,
handed back when the array and all its views are gone.  Checked here: the
results are right (against the oracle), a dropped result's block is reused
by the next call of that size, a surviving view keeps its block (a later
call does not overwrite it), Fortran-ordered incompressible results keep
their layout, and the pool's bookkeeping (stats, trim, foreign pointers).
"""
import gc
import os

import numpy as np
import pytest

import oracle
from conftest import rel_err

pytestmark = pytest.mark.gpu
NT = os.cpu_count() or 1


def _case(seed, dim=3, n=64, p=300_000):
    rng = np.random.default_rng(seed)
    return (rng.normal(0.0, 0.3, (dim, n)), rng.standard_normal(n), rng.standard_normal(n),
            rng.uniform(-20.0, 20.0, (dim, p)))


def test_results_come_from_the_pool_and_are_reused(gsc):
    cov, z1, z2, pos = _case(1)
    gc.collect()
    before = gsc.host_pool_stats()
    a = gsc.summate(cov, z1, z2, pos, form="plain")
    assert rel_err(a, oracle.summator(cov, z1, z2, pos, num_threads=NT)) <= 1e-12
    live = gsc.host_pool_stats()["live_bytes"]
    assert live >= before["live_bytes"] + a.nbytes
    ptr = a.ctypes.data
    del a
    gc.collect()
    assert gsc.host_pool_stats()["live_bytes"] == before["live_bytes"]
    b = gsc.summate(cov, z1, z2, pos, form="plain")
    assert b.ctypes.data == ptr                       # the same block, reused
    assert rel_err(b, oracle.summator(cov, z1, z2, pos, num_threads=NT)) <= 1e-12


def test_views_keep_their_block(gsc):
    cov, z1, z2, pos = _case(2)
    a = gsc.summate(cov, z1, z2, pos, form="mixed")
    view = a[::3]
    saved = view.copy()
    del a
    gc.collect()
    cov2, z12, z22, pos2 = _case(3)
    b = gsc.summate(cov2, z12, z22, pos2, form="mixed")
    assert np.array_equal(view, saved)
    assert not np.shares_memory(view, b)


def test_incompr_and_structured_results(gsc):
    cov, z1, z2, pos = _case(4, dim=3, n=50, p=200_000)
    v = gsc.summate_incompr(cov, z1, z2, pos, form="plain")
    assert v.shape == (3, pos.shape[1]) and v.flags.f_contiguous
    assert rel_err(v, oracle.summator_incompr(cov, z1, z2, pos, num_threads=NT)) <= 1e-12
    axes = tuple(np.arange(s, dtype=np.float64) for s in (16, 96, 128))
    flat = np.ascontiguousarray(np.array(np.meshgrid(*axes, indexing="ij")).reshape(3, -1))
    s = gsc.summate_structured(cov, z1, z2, axes, form="sep_f16x5")
    assert rel_err(s, oracle.summator(cov, z1, z2, flat, num_threads=NT)) <= 1e-6
    si = gsc.summate_incompr_structured(cov, z1, z2, axes, form="sep_f16x5")
    assert rel_err(si, oracle.summator_incompr(cov, z1, z2, flat, num_threads=NT)) <= 1e-6


def test_small_results_are_plain_arrays(gsc):
    cov, z1, z2, pos = _case(5, p=1000)          # 8 KB: below the pool's 64 KiB
    gc.collect()
    before = gsc.host_pool_stats()["live_bytes"]
    a = gsc.summate(cov, z1, z2, pos, form="plain")
    assert gsc.host_pool_stats()["live_bytes"] == before
    assert a.flags.owndata


def test_pool_bookkeeping(gsc):
    import ctypes
    from gstools_core import _native
    cov, z1, z2, pos = _case(6)
    a = gsc.summate(cov, z1, z2, pos, form="plain")
    del a
    gc.collect()
    assert gsc.host_pool_stats()["cached_bytes"] > 0
    gsc.host_pool_trim()
    assert gsc.host_pool_stats()["cached_bytes"] == 0
    foreign = np.empty(16)
    assert _native.lib.gsc_host_free(ctypes.c_void_p(foreign.ctypes.data)) == _native.GSC_ERR_INVALID
    ptr = ctypes.c_void_p()
    assert _native.lib.gsc_host_alloc(0, ctypes.byref(ptr)) == _native.GSC_ERR_INVALID


@pytest.mark.parametrize("incompr,shape", [
    (False, (160, 128, 64)),      # 160 row tiles, tensor-store epilogue
    (True, (200, 128, 64)),       # 200 row tiles x 3 components of 64
    (False, (160, 128, 63)),      # odd rows: plain-store epilogue
    (True, (80, 256, 45)),        # 160 row tiles, components of 45 columns
])
def test_wave_launches_with_overlapped_copies(gsc, incompr, shape):
    """More row tiles than one wave: the tensor-core GEMM runs one launch per
    wave and each wave's rows are copied into the pinned result while the
    next wave computes; the assembled field equals the oracle's."""
    rng = np.random.default_rng(7 + incompr + shape[2])
    n = 40
    cov = rng.normal(0.0, 0.3, (3, n))
    z1, z2 = rng.standard_normal(n), rng.standard_normal(n)
    axes = tuple(0.5 * np.arange(s, dtype=np.float64) for s in shape)
    flat = np.ascontiguousarray(np.array(np.meshgrid(*axes, indexing="ij")).reshape(3, -1))
    if incompr:
        got = gsc.summate_incompr_structured(cov, z1, z2, axes, form="sep_f16x5")
        ref = oracle.summator_incompr(cov, z1, z2, flat, num_threads=NT)
    else:
        got = gsc.summate_structured(cov, z1, z2, axes, form="sep_f16x5")
        ref = oracle.summator(cov, z1, z2, flat, num_threads=NT)
    assert got.shape == ref.shape
    # The form's error is about 1e-7 of the field RMS (RMS over points); the
    # max over the millions of values here is a 6-8 sigma statistic of that:
    # 4.6e-7 to 8.5e-7 on these four cases (1.03e-6 on the 45-column case
    # before the G grid took its twelfth bit).
    err = np.asarray(got, dtype=np.float64) - ref
    rms = float(np.sqrt(np.mean(ref ** 2)))
    assert float(np.sqrt(np.mean(err ** 2))) / rms <= 2e-7
    assert rel_err(got, ref) <= 1e-6


def test_host_calls_time_their_copies(gsc):
    """With timing on, a host-array call reports its host-device copies
    (copy_h2d, copy_d2h) beside its kernels.  A point call whose result is
    a pinned pool block has its kernels write the result in place (no copy
    back); with a small, pageable result it copies the result back."""
    cov, z1, z2, pos = _case(9)
    small = np.ascontiguousarray(pos[:, :1000])            # 8 KB result: pageable
    for call, d2h in ((lambda: gsc.summate(cov, z1, z2, pos, form="mixed", timing=True), False),
                      (lambda: gsc.summate(cov, z1, z2, small, form="mixed", timing=True), True),
                      (lambda: gsc.summate_structured(cov, z1, z2, (np.arange(8.0),) * 3,
                                                      form="sep_f64", timing=True), True),
                      (lambda: gsc.summate_batch([{"cov": cov, "z1": z1, "z2": z2, "pos": pos}] * 2,
                                                 form="plain", timing=True), True)):
        call()
        call()                                   # a batch plan is reused on the second call
        t = dict(gsc.last_timings())
        assert "copy_h2d" in t and t["copy_h2d"] >= 0
        assert ("copy_d2h" in t) == d2h and t.get("copy_d2h", 0.0) >= 0
        assert any(not k.startswith("copy_") for k in t)
