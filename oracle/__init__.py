"""CPU oracle for the spectral random-field summators (test infrastructure).

This package is the CHECKER for the GPU library, not part of the product:
only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg import it.  It wraps ``field_oracle.c``, a C restatement of the
reference's ``src/field.rs`` (``summator`` :37-65, ``summator_incompr``
:97-182, ``summator_fourier`` :219-249), compiled with ``-ffp-contract=off``
and calling glibc ``cos``/``sin`` so that it reproduces the reference's
known answers bit for bit (see tests/test_oracle.py).

Every function takes numpy float64 arrays with arbitrary strides, like the
reference's ``PyReadonlyArray`` arguments, and returns a new array shaped
like the reference's result.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, "field_oracle.c")
_OUT_DIR = os.path.join(_HERE, "_build")
_LIB_PATH = os.path.join(_OUT_DIR, "libfield_oracle.so")

# -ffp-contract=off: Rust never fuses a*b+c, and GCC on aarch64 would.
CFLAGS = ["-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-pthread"]

_lock = threading.Lock()
_lib = None


def build(force: bool = False) -> str:
    """Compile ``field_oracle.c`` into ``oracle/_build/libfield_oracle.so``."""
    os.makedirs(_OUT_DIR, exist_ok=True)
    if (not force and os.path.exists(_LIB_PATH)
            and os.path.getmtime(_LIB_PATH) >= os.path.getmtime(_SRC)):
        return _LIB_PATH
    tmp = _LIB_PATH + f".tmp{os.getpid()}"
    subprocess.run(["gcc", *CFLAGS, "-o", tmp, _SRC, "-lm"], check=True)
    os.replace(tmp, _LIB_PATH)
    return _LIB_PATH


def _load():
    global _lib
    with _lock:
        if _lib is None:
            lib = ctypes.CDLL(build())
            P, I64, INT = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int
            lib.orc_summator.argtypes = [P, I64, I64, P, I64, P, I64, P, I64, I64,
                                         I64, I64, I64, P, I64, INT]
            lib.orc_summator_fourier.argtypes = [P, I64, P, I64, I64, P, I64, P, I64,
                                                 P, I64, I64, I64, I64, I64, P, I64, INT]
            lib.orc_summator_incompr.argtypes = [P, I64, I64, P, I64, P, I64, P, I64, I64,
                                                 I64, I64, I64, P, I64, I64, INT]
            for f in (lib.orc_summator, lib.orc_summator_fourier, lib.orc_summator_incompr):
                f.restype = INT
            _lib = lib
    return _lib


def _view(a: np.ndarray, ndim: int):
    if not isinstance(a, np.ndarray) or a.dtype != np.float64 or a.ndim != ndim:
        raise TypeError(f"expected a float64 ndarray with {ndim} dims")
    es = a.itemsize
    strides = tuple(s // es for s in a.strides)
    return a.ctypes.data, strides


def _check(rc: int):
    if rc == 3:
        raise ValueError("Only two- and three-dimensional problems are supported.")
    if rc != 0:
        raise RuntimeError(f"oracle failed with status {rc}")


def _nthreads(num_threads):
    return 1 if num_threads is None else int(num_threads)


def summator(cov_samples, z1, z2, pos, num_threads=None) -> np.ndarray:
    """src/field.rs:37-65.  ``num_threads`` None means sequential."""
    cp, (cs_d, cs_n) = _view(cov_samples, 2)
    z1p, (z1s,) = _view(z1, 1)
    z2p, (z2s,) = _view(z2, 1)
    pp, (ps_d, ps_p) = _view(pos, 2)
    d, n = cov_samples.shape
    if pos.shape[0] != d or z1.shape[0] != n or z2.shape[0] != n:
        raise ValueError("shape mismatch")
    p = pos.shape[1]
    out = np.empty(p, dtype=np.float64)
    _check(_load().orc_summator(cp, cs_d, cs_n, z1p, z1s, z2p, z2s, pp, ps_d, ps_p,
                                d, n, p, out.ctypes.data, 1, _nthreads(num_threads)))
    return out


def summator_fourier(spectrum_factor, modes, z1, z2, pos, num_threads=None) -> np.ndarray:
    """src/field.rs:219-249."""
    sp, (sfs,) = _view(spectrum_factor, 1)
    mp, (ms_d, ms_n) = _view(modes, 2)
    z1p, (z1s,) = _view(z1, 1)
    z2p, (z2s,) = _view(z2, 1)
    pp, (ps_d, ps_p) = _view(pos, 2)
    d, n = modes.shape
    if (pos.shape[0] != d or z1.shape[0] != n or z2.shape[0] != n
            or spectrum_factor.shape[0] != n):
        raise ValueError("shape mismatch")
    p = pos.shape[1]
    out = np.empty(p, dtype=np.float64)
    _check(_load().orc_summator_fourier(sp, sfs, mp, ms_d, ms_n, z1p, z1s, z2p, z2s,
                                        pp, ps_d, ps_p, d, n, p, out.ctypes.data, 1,
                                        _nthreads(num_threads)))
    return out


def summator_incompr(cov_samples, z1, z2, pos, num_threads=None) -> np.ndarray:
    """src/field.rs:97-182.  Returns (dim, n_points); None means one fold split."""
    cp, (cs_d, cs_n) = _view(cov_samples, 2)
    z1p, (z1s,) = _view(z1, 1)
    z2p, (z2s,) = _view(z2, 1)
    pp, (ps_d, ps_p) = _view(pos, 2)
    d, n = cov_samples.shape
    if pos.shape[0] != d or z1.shape[0] != n or z2.shape[0] != n:
        raise ValueError("shape mismatch")
    p = pos.shape[1]
    out = np.empty((d, p), dtype=np.float64)
    _check(_load().orc_summator_incompr(cp, cs_d, cs_n, z1p, z1s, z2p, z2s, pp, ps_d, ps_p,
                                        d, n, p, out.ctypes.data, p, 1,
                                        _nthreads(num_threads)))
    return out
