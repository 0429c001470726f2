"""The allocation-free entry point gsc_summate_dev_noalloc (GPU test).

Callers that may not have a library allocate device memory (a host whose own
allocator owns the GPU, a real-time loop, a plug-in host with its own arena)
use this entry point: it keeps its per-mode tables in a fixed array inside the
library instead of allocating.  This file checks, through the C ABI, that it
returns what the allocating entry point gsc_summate_dev returns (within the
plain FP64 bar of 1e-12 of the field RMS) on two calls in a row -- the second
call reuses the array the first one filled -- and that it refuses more modes
than the array holds.  It is named to run last in the suite.
"""
import ctypes

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


def test_noalloc_matches_allocating_entry_point(native_lib):
    torch = pytest.importorskip("torch")
    from gstools_core import _native
    lib = _native.lib
    stream = torch.cuda.current_stream()
    opts = _native.make_opts(stream=stream.cuda_stream)
    cases = [(3, 700, 50000), (2, MAX_MODES, 7777)]     # two calls in a row
    for seed, (dim, n, p) in enumerate(cases):
        cov, z1, z2, pos = (_dev(torch, a) for a in _case(seed, dim, n, p))
        ref = torch.empty(p, dtype=torch.float64, device="cuda")
        got = torch.full((p,), float("nan"), dtype=torch.float64, device="cuda")
        args = (cov.data_ptr(), z1.data_ptr(), z2.data_ptr(), pos.data_ptr(), dim, n, p)
        _native.check(lib.gsc_summate_dev(*args, ref.data_ptr(), ctypes.byref(opts)))
        _native.check(lib.gsc_summate_dev_noalloc(*args, got.data_ptr(), ctypes.byref(opts)))
        stream.synchronize()
        err = rel_err(got.cpu().numpy(), ref.cpu().numpy())
        assert err <= TOL, f"call {seed}: {err:.3e}"


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
