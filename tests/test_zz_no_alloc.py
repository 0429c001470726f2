"""The allocation-free entry point gsc_summate_dev_noalloc (GPU test).

Callers that may not have a library allocate device memory (a host whose own
allocator owns the GPU, a real-time loop, a plug-in host with its own arena)
use this entry point: it keeps its per-mode tables in a fixed array inside the
library instead of allocating.  This file checks, through the C ABI, that it
returns what the allocating entry point gsc_summate_dev returns and what the
oracle (the CPU restatement of the reference's summator) returns, within the
plain FP64 bar of 1e-12 of the field RMS, on two calls in a row -- the second
call reuses the array the first one filled.  Both calls run with the
library's allocation-failure injection armed, so any allocation of a library
buffer would fail them, and the second call leaves the device's free memory
unchanged.  It also checks that the entry point refuses more modes than the
array holds.  It is named to run last in the suite.
"""
import ctypes
import os

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

TOL = 1e-12
MAX_MODES = 1024


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _case(seed, dim, n, p):
    rng = np.random.default_rng(seed)
    cov = rng.normal(0.0, 0.4, (dim, n))
    z1, z2 = rng.standard_normal(n), rng.standard_normal(n)
    pos = rng.uniform(-60.0, 60.0, (dim, p))
    return cov, z1, z2, pos


def test_noalloc_matches_allocating_entry_point_and_oracle(native_lib):
    torch = pytest.importorskip("torch")
    import oracle
    from gstools_core import _native
    lib = _native.lib
    stream = torch.cuda.current_stream()
    opts = _native.make_opts(stream=stream.cuda_stream)
    # two calls in a row, the same kernels (the first one loads them)
    cases = [(3, 700, 50000), (3, MAX_MODES, 7777)]
    for call, (dim, n, p) in enumerate(cases):
        host = _case(call, dim, n, p)
        cov, z1, z2, pos = (_dev(torch, a) for a in host)
        ref = torch.empty(p, dtype=torch.float64, device="cuda")
        got = torch.full((p,), float("nan"), dtype=torch.float64, device="cuda")
        args = (cov.data_ptr(), z1.data_ptr(), z2.data_ptr(), pos.data_ptr(), dim, n, p)
        _native.check(lib.gsc_summate_dev(*args, ref.data_ptr(), ctypes.byref(opts)))
        stream.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        # the next allocation of any library buffer would fail as out of memory
        assert lib.gsc_selftest_fail_alloc(0) == 0
        try:
            rc = lib.gsc_summate_dev_noalloc(*args, got.data_ptr(), ctypes.byref(opts))
        finally:
            lib.gsc_selftest_fail_alloc(-1)
        _native.check(rc)
        stream.synchronize()
        if call > 0:            # the device is warm: the call took no device memory
            assert torch.cuda.mem_get_info()[0] == free_before
        got_h = got.cpu().numpy()
        err = rel_err(got_h, ref.cpu().numpy())
        assert err <= TOL, f"call {call}: {err:.3e} against gsc_summate_dev"
        want = oracle.summator(*host, num_threads=os.cpu_count())
        err_o = rel_err(got_h, want)
        assert err_o <= TOL, f"call {call}: {err_o:.3e} against the oracle"


def test_noalloc_refuses_more_modes_than_its_array_holds(native_lib):
    torch = pytest.importorskip("torch")
    from gstools_core import _native
    lib = _native.lib
    cov, z1, z2, pos = (_dev(torch, a) for a in _case(9, 3, MAX_MODES + 1, 100))
    out = torch.empty(100, dtype=torch.float64, device="cuda")
    rc = lib.gsc_summate_dev_noalloc(cov.data_ptr(), z1.data_ptr(), z2.data_ptr(),
                                     pos.data_ptr(), 3, MAX_MODES + 1, 100, out.data_ptr(),
                                     None)
    assert rc == _native.GSC_ERR_INVALID
    assert b"at most 1024 modes" in lib.gsc_last_error()
