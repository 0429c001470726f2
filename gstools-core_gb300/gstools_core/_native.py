"""ctypes binding of ``libgstools_core_gb300.so`` (the C ABI in
``include/gstools_core_gb300.h``).

The library is loaded when the package is imported.  If it has not been
built, the import fails: there is no CPU implementation behind this package.
"""
from __future__ import annotations

import ctypes
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


# name -> (restype, argtypes); every symbol declared in the public header
_P, _I64, _I32 = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32
_OPTS = ctypes.POINTER(GscOpts)
SIGNATURES = {
    "gsc_version": (ctypes.c_char_p, []),
    "gsc_last_error": (ctypes.c_char_p, []),
    "gsc_device_count": (ctypes.c_int, [ctypes.POINTER(_I32)]),
    "gsc_last_timings": (ctypes.c_int, [_P, _P, _I32]),
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
