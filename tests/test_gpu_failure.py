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
