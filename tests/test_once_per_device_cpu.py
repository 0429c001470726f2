"""Per-device kernel set-up, on the CPU (no device is touched).

Launch attributes such as the dynamic shared-memory limit belong to the
device that was current when cudaFuncSetAttribute ran.  Every launch path of
the library therefore sets them up through one registry keyed by (kernel,
device): a process with two GPUs configures each kernel on each of them,
and threads whose first calls race set each pair up once.  The registry is
driven here through gsc_selftest_once_per_device with stand-in kernels and
device ordinals; every pair's set-up fails once before it succeeds, as a
transient error would, and must then run exactly once more.
"""
import ctypes

import pytest


@pytest.mark.parametrize("n_devices,n_keys,n_threads", [(1, 1, 1), (2, 3, 1), (4, 8, 16),
                                                        (8, 24, 32), (64, 64, 64)])
def test_each_kernel_is_set_up_once_per_device(native_lib, n_devices, n_keys, n_threads):
    from gstools_core import _native
    setups = ctypes.c_int64(-1)
    rc = _native.lib.gsc_selftest_once_per_device(n_devices, n_keys, n_threads,
                                                  ctypes.byref(setups))
    assert rc == _native.GSC_OK, _native.lib.gsc_last_error()
    assert setups.value == n_devices * n_keys


def test_selftest_rejects_out_of_range_arguments(native_lib):
    from gstools_core import _native
    setups = ctypes.c_int64(0)
    for args in ((0, 1, 1), (1, 0, 1), (1, 1, 0), (65, 1, 1), (1, 65, 1), (1, 1, 65)):
        assert _native.lib.gsc_selftest_once_per_device(*args, ctypes.byref(setups)) == \
            _native.GSC_ERR_INVALID
