"""ctypes binding of ``libgstools_core_gb300.so`` (the C ABI in
``include/gstools_core_gb300.h``).

The library is loaded when the package is imported.  If it has not been
built, the import fails: there is no CPU implementation behind this package.
"""
from __future__ import annotations

import ctypes

import numpy as np
import os

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libgstools_core_gb300.so")

GSC_OK = 0
GSC_ERR_INVALID = 1
GSC_ERR_DIM = 2
GSC_ERR_CUDA = 3
GSC_ERR_NO_DEVICE = 4
GSC_ERR_NOMEM = 5
GSC_ERR_KERNEL = 6

GSC_FLAG_TIMING = 1

FORMS = {
    "auto": 0,
    "plain": 1,
    "plain_libm": 2,
    "sep_f16x3": 3,
    "sep_bf16x3": 4,
    "sep_f16x5": 5,
    "mixed": 6,
    "mixed_f64phase": 7,
    "sep_f64": 8,
}


class GscOpts(ctypes.Structure):
    _fields_ = [
        ("struct_size", ctypes.c_int32),
        ("form", ctypes.c_int32),
        ("device", ctypes.c_int32),
        ("flags", ctypes.c_int32),
        ("stream", ctypes.c_void_p),
        ("tolerance", ctypes.c_double),
    ]


def make_opts(form="auto", device=-1, flags=0, stream=None, tolerance=0.0) -> GscOpts:
    if isinstance(form, str):
        if form not in FORMS:
            raise ValueError(f"unknown form {form!r}; choose from {sorted(FORMS)}")
        form = FORMS[form]
    return GscOpts(ctypes.sizeof(GscOpts), int(form), int(device), int(flags),
                   ctypes.c_void_p(stream or 0), float(tolerance))


class GscBatchItem(ctypes.Structure):
    _fields_ = [
        ("dim", ctypes.c_int32),
        ("kind", ctypes.c_int32),
        ("n_modes", ctypes.c_int64),
        ("n_points", ctypes.c_int64),
        ("cov", ctypes.c_void_p),
        ("z1", ctypes.c_void_p),
        ("z2", ctypes.c_void_p),
        ("spectrum_factor", ctypes.c_void_p),
        ("pos", ctypes.c_void_p),
        ("out", ctypes.c_void_p),
    ]


# The same layout as a numpy structured type, so that a list of many items is
# filled by columns instead of one ctypes structure at a time.
BATCH_ITEM_DTYPE = np.dtype([("dim", "<i4"), ("kind", "<i4"), ("n_modes", "<i8"),
                             ("n_points", "<i8"), ("cov", "<u8"), ("z1", "<u8"), ("z2", "<u8"),
                             ("spectrum_factor", "<u8"), ("pos", "<u8"), ("out", "<u8")],
                            align=True)


class GscBatchConfig(ctypes.Structure):
    _fields_ = [
        ("struct_size", ctypes.c_int32),
        ("points_per_thread", ctypes.c_int32),
        ("tile_modes", ctypes.c_int32),
        ("units_per_block", ctypes.c_int32),
        ("form", ctypes.c_int32),
        ("blocks", ctypes.c_int32),
        ("units", ctypes.c_int64),
        ("max_splits", ctypes.c_int32),
        ("tuned", ctypes.c_int32),
        ("tune_ms", ctypes.c_double),
        ("work", ctypes.c_double),
    ]


BATCH_KINDS = {"scalar": 0, "incompr": 1, "fourier": 2}
SPECTRA = {"gaussian": 0, "exponential": 1}


class GscSampleItem(ctypes.Structure):
    _fields_ = [
        ("spectrum", ctypes.c_int32),
        ("dim", ctypes.c_int32),
        ("n_modes", ctypes.c_int64),
        ("len_scale", ctypes.c_double),
        ("realization", ctypes.c_int64),
        ("cov", ctypes.c_void_p),
        ("z1", ctypes.c_void_p),
        ("z2", ctypes.c_void_p),
    ]


def make_batch_config(points_per_thread=0, tile_modes=0, units_per_block=0) -> GscBatchConfig:
    return GscBatchConfig(ctypes.sizeof(GscBatchConfig), int(points_per_thread), int(tile_modes),
                          int(units_per_block))


# name -> (restype, argtypes); every symbol declared in the public header
_P, _I64, _I32 = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32
_OPTS = ctypes.POINTER(GscOpts)
SIGNATURES = {
    "gsc_version": (ctypes.c_char_p, []),
    "gsc_last_error": (ctypes.c_char_p, []),
    "gsc_device_count": (ctypes.c_int, [ctypes.POINTER(_I32)]),
    "gsc_last_timings": (ctypes.c_int, [_P, _P, _I32]),
    "gsc_last_timeline": (ctypes.c_int, [_P, _P, _P, _I32]),
    "gsc_kernel_name": (ctypes.c_char_p, [_I32]),
    "gsc_summate_f64": (ctypes.c_int, [_P, _I64, _I64, _P, _I64, _P, _I64, _P, _I64, _I64,
                                       _I64, _I64, _I64, _P, _I64, _OPTS]),
    "gsc_summate_dev": (ctypes.c_int, [_P, _P, _P, _P, _I64, _I64, _I64, _P, _OPTS]),
    "gsc_summate_incompr_f64": (ctypes.c_int, [_P, _I64, _I64, _P, _I64, _P, _I64, _P, _I64,
                                               _I64, _I64, _I64, _I64, _P, _I64, _I64, _OPTS]),
    "gsc_summate_incompr_dev": (ctypes.c_int, [_P, _P, _P, _P, _I64, _I64, _I64, _P, _OPTS]),
    "gsc_device_status": (ctypes.c_int, [_I32]),
    "gsc_summate_dev_noalloc": (ctypes.c_int, [_P, _P, _P, _P, _I64, _I64, _I64, _P, _OPTS]),
    "gsc_summate_structured_f64": (ctypes.c_int, [_P, _I64, _I64, _P, _I64, _P, _I64, _I64, _I64,
                                                  _P, _I64, _I64, _P, _I64, _I64, _P, _I64, _I64,
                                                  _P, _OPTS]),
    "gsc_summate_structured_dev": (ctypes.c_int, [_P, _P, _P, _I64, _I64, _P, _I64, _P, _I64,
                                                  _P, _I64, _P, _OPTS]),
    "gsc_summate_incompr_structured_f64": (ctypes.c_int, [_P, _I64, _I64, _P, _I64, _P, _I64,
                                                          _I64, _I64, _P, _I64, _I64, _P, _I64,
                                                          _I64, _P, _I64, _I64, _P, _OPTS]),
    "gsc_summate_incompr_structured_dev": (ctypes.c_int, [_P, _P, _P, _I64, _I64, _P, _I64, _P,
                                                          _I64, _P, _I64, _P, _OPTS]),
    "gsc_summate_fourier_f64": (ctypes.c_int, [_P, _I64, _P, _I64, _I64, _P, _I64, _P, _I64,
                                               _P, _I64, _I64, _I64, _I64, _I64, _P, _I64,
                                               _OPTS]),
    "gsc_summate_fourier_dev": (ctypes.c_int, [_P, _P, _P, _P, _P, _I64, _I64, _I64, _P, _OPTS]),
    "gsc_summate_fourier_structured_f64": (ctypes.c_int, [_P, _I64, _P, _I64, _I64, _P, _I64,
                                                          _P, _I64, _I64, _I64, _P, _I64, _I64,
                                                          _P, _I64, _I64, _P, _I64, _I64, _P,
                                                          _OPTS]),
    "gsc_summate_fourier_structured_dev": (ctypes.c_int, [_P, _P, _P, _P, _I64, _I64, _P, _I64,
                                                          _P, _I64, _P, _I64, _P, _OPTS]),
    "gsc_batch_create": (ctypes.c_int, [ctypes.POINTER(GscBatchItem), _I64, _OPTS,
                                        ctypes.POINTER(GscBatchConfig),
                                        ctypes.POINTER(ctypes.c_void_p)]),
    "gsc_batch_run": (ctypes.c_int, [_P, _P]),
    "gsc_batch_run_graph": (ctypes.c_int, [_P, _P]),
    "gsc_batch_get_config": (ctypes.c_int, [_P, ctypes.POINTER(GscBatchConfig)]),
    "gsc_batch_destroy": (ctypes.c_int, [_P]),
    "gsc_summate_batch_f64": (ctypes.c_int, [ctypes.POINTER(GscBatchItem), _I64, _OPTS,
                                             ctypes.POINTER(GscBatchConfig)]),
    "gsc_last_batch_config": (ctypes.c_int, [_I32, ctypes.POINTER(GscBatchConfig)]),
    "gsc_sample_modes_batch_dev": (ctypes.c_int, [ctypes.POINTER(GscSampleItem), _I64,
                                                  ctypes.c_uint64, _OPTS]),
    "gsc_sample_modes_dev": (ctypes.c_int, [_I32, _I32, _I64, ctypes.c_double, ctypes.c_uint64,
                                            _I64, _P, _P, _P, _OPTS]),
    "gsc_sample_modes_f64": (ctypes.c_int, [_I32, _I32, _I64, ctypes.c_double, ctypes.c_uint64,
                                            _I64, _P, _P, _P, _OPTS]),
    "gsc_selftest_wait_timeout": (ctypes.c_int, [_I32, _I64]),
    "gsc_selftest_pipe_rates": (ctypes.c_int, [_I32, ctypes.POINTER(ctypes.c_double)]),
    "gsc_selftest_fail_alloc": (ctypes.c_int, [_I32]),
    "gsc_selftest_detect_grid": (ctypes.c_int, [_P, _I64, _I64, _I64, _I64,
                                                ctypes.POINTER(ctypes.c_int64)]),
    "gsc_selftest_once_per_device": (ctypes.c_int, [_I32, _I32, _I32, ctypes.POINTER(_I64)]),
    "gsc_selftest_batch_queue": (ctypes.c_int, [ctypes.POINTER(GscBatchItem), _I64, _I32,
                                                ctypes.POINTER(GscBatchConfig), _I32, _I32]),
    "gsc_tune_cache_open": (ctypes.c_int, [ctypes.c_char_p]),
    "gsc_tune_cache_size": (ctypes.c_int, [ctypes.POINTER(ctypes.c_int64)]),
    "gsc_tune_cache_get": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(ctypes.c_int32)]),
    "gsc_tune_cache_put": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(ctypes.c_int32)]),
    "gsc_tune_cache_clear": (ctypes.c_int, []),
    "gsc_tune_set_mode": (ctypes.c_int, [_I32]),
    "gsc_release_buffers": (ctypes.c_int, [_I32]),
    "gsc_host_alloc": (ctypes.c_int, [_I64, ctypes.POINTER(ctypes.c_void_p)]),
    "gsc_host_free": (ctypes.c_int, [ctypes.c_void_p]),
    "gsc_host_pool_trim": (ctypes.c_int, []),
    "gsc_host_pool_stats": (ctypes.c_int, [ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64)]),
}


def _load():
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            f"gstools_core: native library {LIB_PATH} is not built; run "
            "`python -c 'import __graft_entry__ as g; g.build()'` or "
            "`python gstools-core_gb300/gsc_build.py` (there is no CPU fallback)")
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


lib = _load()


class GscError(RuntimeError):
    """A CUDA-side failure reported by the native library."""


def check(rc: int) -> None:
    if rc == GSC_OK:
        return
    msg = (lib.gsc_last_error() or b"").decode(errors="replace")
    if rc in (GSC_ERR_INVALID, GSC_ERR_DIM):
        raise ValueError(msg)
    if rc == GSC_ERR_NOMEM:
        raise MemoryError(msg)
    raise GscError(f"[status {rc}] {msg}")


def device_count() -> int:
    n = _I32(0)
    check(lib.gsc_device_count(ctypes.byref(n)))
    return int(n.value)


def last_timings(cap: int = 64):
    """[(kernel_name, ms), ...] of the last call made with GSC_FLAG_TIMING."""
    ids = (_I32 * cap)()
    ms = (ctypes.c_double * cap)()
    n = lib.gsc_last_timings(ids, ms, cap)
    return [(lib.gsc_kernel_name(ids[i]).decode(), float(ms[i])) for i in range(n)]


def last_timeline(cap: int = 256):
    """[(kernel_name, start_ms, ms), ...] of the last call made with
    GSC_FLAG_TIMING: each record's start after the first record's start (all
    of the call's streams on one clock) and its duration."""
    ids = (_I32 * cap)()
    st = (ctypes.c_double * cap)()
    ms = (ctypes.c_double * cap)()
    n = lib.gsc_last_timeline(ids, st, ms, cap)
    return [(lib.gsc_kernel_name(ids[i]).decode(), float(st[i]), float(ms[i])) for i in range(n)]
