"""Failure detection of the pipelined kernels, exercised without a GPU fault
(GPU test).

A one-CTA kernel waits, with the bounded wait the tensor-core pipelines use,
on an mbarrier that nothing ever completes.  The wait must give up after its
limit, record its code in the device status word and return; the host must
read the status as GSC_ERR_KERNEL, clear it, and the device must go on
computing correct fields.
"""
import os
import time

import numpy as np
import pytest

import oracle
from conftest import rel_err

pytestmark = pytest.mark.gpu


def test_timed_out_wait_reports_and_the_device_stays_usable(gsc):
    from gstools_core import _native
    lib = _native.lib
    t0 = time.monotonic()
    rc = lib.gsc_selftest_wait_timeout(-1, 20000)          # 20 ms limit
    elapsed = time.monotonic() - t0
    assert rc == _native.GSC_ERR_KERNEL
    assert b"status 1" in lib.gsc_last_error()
    assert elapsed < 5.0
    gsc.device_status()                                     # cleared: no error now
    # the same context computes correctly afterwards (tensor-core form)
    rng = np.random.default_rng(5)
    cov = rng.normal(0.0, 0.3, (3, 300))
    z1, z2 = rng.standard_normal(300), rng.standard_normal(300)
    axes = tuple(np.arange(n, dtype=np.float64) for n in (9, 40, 50))
    pos = np.ascontiguousarray(np.array(np.meshgrid(*axes, indexing="ij")).reshape(3, -1))
    ref = oracle.summator(cov, z1, z2, pos, num_threads=os.cpu_count() or 1)
    out = gsc.summate_structured(cov, z1, z2, axes, form="sep_f16x5")
    assert rel_err(out, ref) <= 1e-6


def test_selftest_rejects_limits_out_of_range(gsc):
    from gstools_core import _native
    assert _native.lib.gsc_selftest_wait_timeout(-1, 10) == _native.GSC_ERR_INVALID
    assert _native.lib.gsc_selftest_wait_timeout(-1, 10 ** 9) == _native.GSC_ERR_INVALID


def _scalar_case(seed, dim=3, n=200, p=5000):
    rng = np.random.default_rng(seed)
    cov = rng.normal(0.0, 0.3, (dim, n))
    z1, z2 = rng.standard_normal(n), rng.standard_normal(n)
    pos = rng.uniform(-20.0, 20.0, (dim, p))
    return cov, z1, z2, pos


@pytest.mark.parametrize("countdown", [0, 1])
def test_allocation_failure_is_reported_and_recovered(gsc, countdown):
    """An out-of-memory in any of a call's buffer allocations (injected on
    the host, the same path a failing cudaMalloc takes) raises MemoryError;
    the next call allocates again and computes the right field."""
    from gstools_core import _native
    lib = _native.lib
    cov, z1, z2, pos = _scalar_case(11)
    ref = oracle.summator(cov, z1, z2, pos, num_threads=os.cpu_count() or 1)
    gsc.release_buffers()                      # the next call must allocate
    assert lib.gsc_selftest_fail_alloc(countdown) == 0
    try:
        with pytest.raises(MemoryError, match="injected allocation failure"):
            gsc.summate(cov, z1, z2, pos, form="plain")
    finally:
        lib.gsc_selftest_fail_alloc(-1)
    out = gsc.summate(cov, z1, z2, pos, form="plain")
    assert rel_err(out, ref) <= 1e-12


def test_batch_plan_allocation_failure(gsc):
    """A plan whose device memory cannot be had is not made (no partial plan
    leaks); the same items then make a working plan."""
    torch = pytest.importorskip("torch")
    from gstools_core import _native
    lib = _native.lib
    items = []
    for s in range(3):
        cov, z1, z2, pos = _scalar_case(20 + s, n=100 + s, p=3000 + s)
        items.append({"cov": cov, "z1": z1, "z2": z2, "pos": pos})
    dev = [{k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in it.items()}
           for it in items]
    for d in dev:
        d["out"] = torch.empty(d["pos"].shape[1], dtype=torch.float64, device="cuda")
    for countdown in (0, 2):
        assert lib.gsc_selftest_fail_alloc(countdown) == 0
        try:
            with pytest.raises(MemoryError, match="injected allocation failure"):
                gsc.Batch(dev, form="plain", points_per_thread=4, tile_modes=8, units_per_block=4)
        finally:
            lib.gsc_selftest_fail_alloc(-1)
    with gsc.Batch(dev, form="plain", points_per_thread=4, tile_modes=8, units_per_block=4) as b:
        b.run()
        torch.cuda.synchronize()
    for it, d in zip(items, dev):
        ref = oracle.summator(it["cov"], it["z1"], it["z2"], it["pos"])
        assert rel_err(d["out"].cpu().numpy(), ref) <= 1e-12


def test_release_buffers_keeps_results(gsc):
    """Released between calls of every host-array path, the library
    reallocates and gives bit-identical results."""
    cov, z1, z2, pos = _scalar_case(31, dim=2, n=300, p=20000)
    a = gsc.summate(cov, z1, z2, pos, form="mixed")
    ai = gsc.summate_incompr(cov, z1, z2, pos, form="plain")
    gsc.release_buffers()
    assert np.array_equal(a, gsc.summate(cov, z1, z2, pos, form="mixed"))
    gsc.release_buffers()
    assert np.array_equal(ai, gsc.summate_incompr(cov, z1, z2, pos, form="plain"))
    axes = (np.arange(64.0), np.arange(96.0))
    s = gsc.summate_structured(cov, z1, z2, axes, form="sep_f16x5")
    gsc.release_buffers()
    assert np.array_equal(s, gsc.summate_structured(cov, z1, z2, axes, form="sep_f16x5"))
    gsc.release_buffers()
    gsc.release_buffers()                     # twice in a row is harmless
