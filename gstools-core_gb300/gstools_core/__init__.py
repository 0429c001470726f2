"""gstools_core -- GB300 (sm_103a) drop-in for GSTools-Core's field summators.

Mirrors the Python module that GSTools-Core's PyO3 layer exposes
(reference ``src/lib.rs:29-65``):

    summate(cov_samples, z1, z2, pos, num_threads=None) -> ndarray (n_points,)
    summate_incompr(cov_samples, z1, z2, pos, num_threads=None)
        -> ndarray (dim, n_points), Fortran ordered like the reference
    summate_fourier(spectrum_factor, modes, z1, z2, pos, num_threads=None)
        -> ndarray (n_points,)                      (src/lib.rs:67-84)
    __version__

Same argument names, dtypes, shapes and return values.  The work runs on the
GPU through the C ABI of ``include/gstools_core_gb300.h``; there is no CPU
path.  Differences from the reference, all at its failure points:

* a shape mismatch or an unsupported dimension raises ``ValueError``
  (the reference panics, and its release build aborts the process);
* ``num_threads`` is validated like PyO3's ``Option<usize>`` and otherwise
  ignored: GPU parallelism is not set by a thread count.

Keyword-only extensions (not in the reference): ``form`` selects a
computation form and ``tolerance`` the error budget that ``form="auto"``
may spend (default 1e-12 of the field RMS, the plain FP64 bar).
"""
from __future__ import annotations

import ctypes
import operator

import numpy as np

from . import _native
from ._native import GscError, device_count, last_timeline, last_timings

__all__ = ["summate", "summate_incompr", "summate_fourier", "randomization_field", "summate_device",
           "summate_incompr_device", "summate_fourier_device",
           "summate_structured", "summate_incompr_structured", "summate_fourier_structured",
           "summate_structured_device", "summate_incompr_structured_device",
           "summate_fourier_structured_device", "Batch", "summate_batch", "last_batch_config",
           "sample_modes", "sample_modes_batch_device",
           "device_status", "release_buffers", "host_pool_stats", "host_pool_trim",
           "device_count", "last_timings", "last_timeline", "GscError", "__version__"]

__version__ = "1.1.0"          # the reference crate version this mirrors (Cargo.toml:3)
native_version = _native.lib.gsc_version().decode()


# ---------------------------------------------------------------------------
# argument extraction with PyO3/numpy's error behaviour
# ---------------------------------------------------------------------------
_F64 = np.dtype(np.float64)


def _array(obj, name: str, ndim: int) -> np.ndarray:
    if type(obj) is np.ndarray and obj.ndim == ndim and obj.dtype is _F64:
        return obj                       # the common case, checked first
    if not isinstance(obj, np.ndarray):
        raise TypeError(f"argument '{name}': '{type(obj).__name__}' object cannot be "
                        f"converted to 'PyArray<T, D>'")
    if obj.ndim != ndim:
        raise TypeError(f"argument '{name}': dimensionality mismatch:\n from={obj.ndim}, to={ndim}")
    if obj.dtype != np.float64:
        raise TypeError(f"argument '{name}': type mismatch:\n from={obj.dtype}, to=float64")
    return obj


def _num_threads(num_threads) -> None:
    if num_threads is None:
        return
    try:
        n = operator.index(num_threads)
    except TypeError:
        raise TypeError(f"argument 'num_threads': '{type(num_threads).__name__}' object "
                        "cannot be interpreted as an integer") from None
    if n < 0:
        raise OverflowError("argument 'num_threads': can't convert negative int to unsigned")


def _assert_eq(left: int, right: int) -> None:
    if left != right:
        raise ValueError(f"assertion `left == right` failed\n  left: {left}\n right: {right}")


def _strides(a: np.ndarray):
    return tuple(s // a.itemsize for s in a.strides)


_POOL_MIN_BYTES = 1 << 16

_CHAR = ctypes.c_char
_ADDRESS = ctypes.addressof


def _ptr(a: np.ndarray) -> int:
    """Address of an array's data.  Through the buffer protocol where the
    array exports a writable C-contiguous buffer (about a third of the cost
    of ``a.ctypes.data``, which an ensemble call pays several times per
    realization); ``a.ctypes.data`` for any other array."""
    try:
        return _ADDRESS(_CHAR.from_buffer(a))
    except (TypeError, ValueError, BufferError):
        return a.ctypes.data


def _result(shape, order="C") -> np.ndarray:
    """A new float64 result array.  From 64 KiB up its memory comes from the
    library's pool of pinned host blocks, which takes the block back when the
    array and every view of it are gone: repeated calls reuse resident pages
    instead of faulting in fresh ones (the result is still a new array each
    call, as the reference returns)."""
    return _result_ptr(shape, order)[0]


def _result_ptr(shape, order="C"):
    """_result and the address of its data (known here without asking the
    array, which costs about a microsecond per call)."""
    n = 1
    for s in shape if isinstance(shape, tuple) else (shape,):
        n *= int(s)
    nbytes = 8 * n
    if nbytes >= _POOL_MIN_BYTES:
        ptr = ctypes.c_void_p()
        if _native.lib.gsc_host_alloc(nbytes, ctypes.byref(ptr)) == 0:
            return np.asarray(_PoolBlock(ptr.value, shape, order)), ptr.value
    a = np.empty(shape, dtype=np.float64, order=order)
    return a, a.ctypes.data


class _PoolBlock:
    """Owner of a pinned pool block, exposed to numpy as a float64 array
    (the array's base): the block returns to the pool when the last array
    or view referring to it is gone."""
    __slots__ = ("ptr", "__array_interface__")
    _free = _native.lib.gsc_host_free

    def __init__(self, ptr, shape, order):
        shape = tuple(shape) if isinstance(shape, tuple) else (int(shape),)
        strides = None
        if order == "F" and len(shape) > 1:
            strides, step = [], 8
            for s in shape:
                strides.append(step)
                step *= int(s)
            strides = tuple(strides)
        self.ptr = ptr
        self.__array_interface__ = {"data": (ptr, False), "shape": shape, "typestr": "<f8",
                                    "strides": strides, "version": 3}

    def __del__(self):
        if self.ptr:
            try:
                _PoolBlock._free(self.ptr)
            except Exception:      # interpreter teardown: the OS reclaims the block
                pass
            self.ptr = None


def host_pool_stats() -> dict:
    """Bytes of pinned result memory handed out and cached by the pool."""
    live, cached = ctypes.c_int64(), ctypes.c_int64()
    _native.check(_native.lib.gsc_host_pool_stats(ctypes.byref(live), ctypes.byref(cached)))
    return {"live_bytes": live.value, "cached_bytes": cached.value}


def host_pool_trim() -> None:
    """Releases the pool's cached (free) pinned blocks."""
    _native.check(_native.lib.gsc_host_pool_trim())


def _opts(form, tolerance, timing, device=-1, stream=None):
    flags = _native.GSC_FLAG_TIMING if timing else 0
    return _native.make_opts(form=form, device=device, flags=flags, stream=stream,
                             tolerance=tolerance or 0.0)


def _prepare(cov_samples, z1, z2, pos, num_threads, cov_name="cov_samples"):
    cov = _array(cov_samples, cov_name, 2)
    z1 = _array(z1, "z1", 1)
    z2 = _array(z2, "z2", 1)
    pos = _array(pos, "pos", 2)
    _num_threads(num_threads)
    # the reference's asserts, in its order (src/field.rs:44-46, 104-106)
    _assert_eq(cov.shape[0], pos.shape[0])
    _assert_eq(cov.shape[1], z1.shape[0])
    _assert_eq(cov.shape[1], z2.shape[0])
    return cov, z1, z2, pos


# ---------------------------------------------------------------------------
# reference API
# ---------------------------------------------------------------------------
def summate(cov_samples, z1, z2, pos, num_threads=None, *, form="auto", tolerance=None,
            timing=False, device=-1):
    """Scalar randomization method (reference ``src/field.rs:37-65``).

    u[p] = sum_j z1[j] cos(k_j . x_p) + z2[j] sin(k_j . x_p)
    with k_j = cov_samples[:, j] and x_p = pos[:, p].
    """
    cov, z1, z2, pos = _prepare(cov_samples, z1, z2, pos, num_threads)
    dim, n = cov.shape
    p = pos.shape[1]
    out, out_ptr = _result_ptr(p)
    cs, zs1, zs2, ps = _strides(cov), _strides(z1), _strides(z2), _strides(pos)
    o = _opts(form, tolerance, timing, device)
    _native.check(_native.lib.gsc_summate_f64(
        _ptr(cov), cs[0], cs[1], _ptr(z1), zs1[0], _ptr(z2), zs2[0],
        _ptr(pos), ps[0], ps[1], dim, n, p, out_ptr, 1, ctypes.byref(o)))
    return out


def summate_incompr(cov_samples, z1, z2, pos, num_threads=None, *, form="auto", tolerance=None,
                    timing=False, device=-1):
    """Incompressible vector field (reference ``src/field.rs:97-182``).

    u[i, p] = sum_j p_i(k_j) (z1[j] cos(k_j . x_p) + z2[j] sin(k_j . x_p)),
    p(k) = e_1 - k k_0 / |k|^2; dim must be 2 or 3.  Returns a
    Fortran-ordered (dim, n_points) array, as the reference does.
    """
    cov, z1, z2, pos = _prepare(cov_samples, z1, z2, pos, num_threads)
    dim, n = cov.shape
    if dim not in (2, 3):
        raise ValueError("Only two- and three-dimensional problems are supported.")
    p = pos.shape[1]
    out, out_ptr = _result_ptr((dim, p), order="F")
    cs, zs1, zs2, ps = _strides(cov), _strides(z1), _strides(z2), _strides(pos)
    os_ = _strides(out)
    o = _opts(form, tolerance, timing, device)
    _native.check(_native.lib.gsc_summate_incompr_f64(
        _ptr(cov), cs[0], cs[1], _ptr(z1), zs1[0], _ptr(z2), zs2[0],
        _ptr(pos), ps[0], ps[1], dim, n, p, out_ptr, os_[0], os_[1],
        ctypes.byref(o)))
    return out


def summate_fourier(spectrum_factor, modes, z1, z2, pos, num_threads=None, *, form="auto",
                    tolerance=None, timing=False, device=-1):
    """Fourier method (reference ``src/field.rs:219-249``).

    u[p] = sum_j sf[j] (z1[j] cos(k_j . x_p) + z2[j] sin(k_j . x_p))
    with k_j = modes[:, j] (the equidistant Fourier grid) and sf the spectrum
    factor sqrt(2 S(k_j dk)).
    """
    sf = _array(spectrum_factor, "spectrum_factor", 1)
    modes, z1, z2, pos = _prepare(modes, z1, z2, pos, num_threads, "modes")
    dim, n = modes.shape
    # the reference zips sf with the mode columns, which asserts equal length
    _assert_eq(sf.shape[0], n)
    p = pos.shape[1]
    out, out_ptr = _result_ptr(p)
    ms, zs1, zs2, ps = _strides(modes), _strides(z1), _strides(z2), _strides(pos)
    o = _opts(form, tolerance, timing, device)
    _native.check(_native.lib.gsc_summate_fourier_f64(
        _ptr(sf), _strides(sf)[0], _ptr(modes), ms[0], ms[1], _ptr(z1),
        zs1[0], _ptr(z2), zs2[0], _ptr(pos), ps[0], ps[1], dim, n, p,
        out_ptr, 1, ctypes.byref(o)))
    return out


# ---------------------------------------------------------------------------
# device-resident API (arrays exposing __cuda_array_interface__, e.g. torch)
# ---------------------------------------------------------------------------
def _cuda_view(obj, name: str, shape):
    iface = getattr(obj, "__cuda_array_interface__", None)
    if iface is None:
        raise TypeError(f"argument '{name}': expected a CUDA array (__cuda_array_interface__)")
    if iface["typestr"] != "<f8":
        raise TypeError(f"argument '{name}': type mismatch:\n from={iface['typestr']}, to=<f8")
    if tuple(iface["shape"]) != tuple(shape):
        raise ValueError(f"argument '{name}': shape {tuple(iface['shape'])} != {tuple(shape)}")
    strides = iface.get("strides")
    if strides is not None:
        expect, acc = [], 8
        for s in reversed(shape):
            expect.append(acc)
            acc *= s
        if tuple(strides) != tuple(reversed(expect)) and int(np.prod(shape)) > 1:
            raise ValueError(f"argument '{name}': must be C-contiguous")
    return iface["data"][0]


def _dev_shapes(cov_samples, pos):
    cs = cov_samples.__cuda_array_interface__["shape"]
    ps = pos.__cuda_array_interface__["shape"]
    if len(cs) != 2 or len(ps) != 2:
        raise TypeError("cov_samples and pos must be 2-D")
    _assert_eq(cs[0], ps[0])
    return cs[0], cs[1], ps[1]


def summate_device(cov_samples, z1, z2, pos, out, *, form="auto", tolerance=None, stream=None,
                   timing=False, device=-1):
    """``summate`` on device-resident, C-contiguous float64 arrays; writes
    ``out`` (n_points,) and returns without synchronising ``stream``."""
    dim, n, p = _dev_shapes(cov_samples, pos)
    args = [_cuda_view(cov_samples, "cov_samples", (dim, n)), _cuda_view(z1, "z1", (n,)),
            _cuda_view(z2, "z2", (n,)), _cuda_view(pos, "pos", (dim, p))]
    o = _opts(form, tolerance, timing, device, stream)
    _native.check(_native.lib.gsc_summate_dev(*args, dim, n, p,
                                              _cuda_view(out, "out", (p,)), ctypes.byref(o)))
    return out


def summate_incompr_device(cov_samples, z1, z2, pos, out, *, form="auto", tolerance=None,
                           stream=None, timing=False, device=-1):
    """``summate_incompr`` on device arrays; ``out`` is (dim, n_points), C order."""
    dim, n, p = _dev_shapes(cov_samples, pos)
    args = [_cuda_view(cov_samples, "cov_samples", (dim, n)), _cuda_view(z1, "z1", (n,)),
            _cuda_view(z2, "z2", (n,)), _cuda_view(pos, "pos", (dim, p))]
    o = _opts(form, tolerance, timing, device, stream)
    _native.check(_native.lib.gsc_summate_incompr_dev(
        *args, dim, n, p, _cuda_view(out, "out", (dim, p)), ctypes.byref(o)))
    return out


def randomization_field(cov_samples, z1, z2, pos, scale, offset=0.0, *, incompr=False,
                        form="auto", tolerance=None, timing=False, device=-1):
    """The normalised field a randomization-method generator returns from
    these modes: ``offset + scale * summate(...)`` for a scalar field, and
    ``offset * e_1 + scale * summate_incompr(...)`` with ``incompr=True``
    (extension; no reference counterpart).

    This is the affine step GSTools' generators wrap around the summators.
    ``RandMeth`` scales the summed modes by ``sqrt(var / mode_no)``, and the
    mean of the spatial random field is added after. ``IncomprRandMeth``
    adds a mean velocity along e_1 to a scaled sum. Pass those as ``scale``
    and ``offset``. The scale multiplies z1 and z2 before the sum, so every
    computation form, including the separable ones that flattened meshes
    are routed to, computes the scaled field directly: one rounding per
    mode, within every form's bar. The offset is added to the result in
    place. A nugget is left to the caller: it is random, drawn by the
    caller's generator.
    """
    z1 = _array(z1, "z1", 1)
    z2 = _array(z2, "z2", 1)
    s = float(scale)
    fn = summate_incompr if incompr else summate
    out = fn(cov_samples, z1 * s, z2 * s, pos, form=form, tolerance=tolerance, timing=timing,
             device=device)
    off = float(offset)
    if off != 0.0:
        if incompr:
            out[0] += off
        else:
            out += off
    return out


# ---------------------------------------------------------------------------
# structured grids (extension: the reference's callers expand the mesh)
# ---------------------------------------------------------------------------
def _axes_host(axes, dim):
    if not isinstance(axes, (list, tuple)) or len(axes) != dim:
        raise ValueError(f"axes must be a sequence of {dim} 1-D float64 arrays")
    out = []
    for i, a in enumerate(axes):
        out.append(_array(a, f"axes[{i}]", 1))
    while len(out) < 3:
        out.append(None)
    return out


def _structured_host(fn, cov_samples, z1, z2, axes, num_threads, form, tolerance, timing,
                     device, incompr, spectrum_factor=None):
    sf = None if spectrum_factor is None else _array(spectrum_factor, "spectrum_factor", 1)
    cov = _array(cov_samples, "cov_samples" if sf is None else "modes", 2)
    z1 = _array(z1, "z1", 1)
    z2 = _array(z2, "z2", 1)
    _num_threads(num_threads)
    dim, n = cov.shape
    _assert_eq(cov.shape[1], z1.shape[0])
    _assert_eq(cov.shape[1], z2.shape[0])
    if sf is not None:
        _assert_eq(sf.shape[0], n)
    ax = _axes_host(axes, dim)
    if incompr and dim not in (2, 3):
        raise ValueError("Only two- and three-dimensional problems are supported.")
    npts = 1
    for a in ax[:dim]:
        npts *= a.shape[0]
    out = _result((dim, npts) if incompr else npts)
    args = []
    for a in ax:
        if a is None:
            args += [None, 0, 0]
        else:
            args += [a.ctypes.data, a.shape[0], _strides(a)[0]]
    cs, zs1, zs2 = _strides(cov), _strides(z1), _strides(z2)
    o = _opts(form, tolerance, timing, device)
    lead = [] if sf is None else [sf.ctypes.data, _strides(sf)[0]]
    _native.check(fn(*lead, cov.ctypes.data, cs[0], cs[1], z1.ctypes.data, zs1[0],
                     z2.ctypes.data, zs2[0], dim, n, *args, out.ctypes.data, ctypes.byref(o)))
    return out


def summate_structured(cov_samples, z1, z2, axes, num_threads=None, *, form="auto",
                       tolerance=None, timing=False, device=-1):
    """``summate`` on the structured grid ``meshgrid(*axes, indexing="ij")``.

    Equal to ``summate(cov_samples, z1, z2, pos)`` with
    ``pos = np.array(np.meshgrid(*axes, indexing="ij")).reshape(dim, -1)``
    (the flattening GSTools uses for structured meshes), but the grid is never
    expanded: with ``form="sep_f16x5"`` (or ``form="auto"`` and
    ``tolerance >= 1e-6``) the sum runs as a separable complex contraction on
    the tensor cores with max error below 1e-6 of the field RMS;
    ``form="sep_f16x3"`` (``tolerance >= 1e-5``) is faster and less exact.
    Returns a flat (n_points,) array.
    """
    return _structured_host(_native.lib.gsc_summate_structured_f64, cov_samples, z1, z2, axes,
                            num_threads, form, tolerance, timing, device, False)


def summate_incompr_structured(cov_samples, z1, z2, axes, num_threads=None, *, form="auto",
                               tolerance=None, timing=False, device=-1):
    """``summate_incompr`` on a structured grid; returns (dim, n_points), C order."""
    return _structured_host(_native.lib.gsc_summate_incompr_structured_f64, cov_samples, z1,
                            z2, axes, num_threads, form, tolerance, timing, device, True)


def summate_fourier_structured(spectrum_factor, modes, z1, z2, axes, num_threads=None, *,
                               form="auto", tolerance=None, timing=False, device=-1):
    """``summate_fourier`` on the structured grid ``meshgrid(*axes, indexing="ij")``
    (flat (n_points,) result); the forms are those of ``summate_structured``."""
    return _structured_host(_native.lib.gsc_summate_fourier_structured_f64, modes, z1, z2, axes,
                            num_threads, form, tolerance, timing, device, False, spectrum_factor)


def _structured_dev(fn, cov_samples, z1, z2, axes, out, form, tolerance, stream, timing,
                    device, incompr, spectrum_factor=None):
    cs = cov_samples.__cuda_array_interface__["shape"]
    if len(cs) != 2:
        raise TypeError("cov_samples must be 2-D")
    dim, n = cs
    if not isinstance(axes, (list, tuple)) or len(axes) != dim:
        raise ValueError(f"axes must be a sequence of {dim} CUDA arrays")
    args, npts = [], 1
    for i, a in enumerate(axes):
        la = a.__cuda_array_interface__["shape"]
        if len(la) != 1:
            raise TypeError(f"axes[{i}] must be 1-D")
        args += [_cuda_view(a, f"axes[{i}]", (la[0],)), la[0]]
        npts *= la[0]
    while len(args) < 6:
        args += [None, 0]
    shape = (dim, npts) if incompr else (npts,)
    o = _opts(form, tolerance, timing, device, stream)
    lead = [] if spectrum_factor is None else [_cuda_view(spectrum_factor, "spectrum_factor", (n,))]
    _native.check(fn(*lead, _cuda_view(cov_samples, "cov_samples", (dim, n)),
                     _cuda_view(z1, "z1", (n,)),
                     _cuda_view(z2, "z2", (n,)), dim, n, *args, _cuda_view(out, "out", shape),
                     ctypes.byref(o)))
    return out


def summate_structured_device(cov_samples, z1, z2, axes, out, *, form="auto", tolerance=None,
                              stream=None, timing=False, device=-1):
    """``summate_structured`` on device arrays; writes ``out`` (n_points,)."""
    return _structured_dev(_native.lib.gsc_summate_structured_dev, cov_samples, z1, z2, axes,
                           out, form, tolerance, stream, timing, device, False)


def summate_incompr_structured_device(cov_samples, z1, z2, axes, out, *, form="auto",
                                      tolerance=None, stream=None, timing=False, device=-1):
    """``summate_incompr_structured`` on device arrays; ``out`` is (dim, n_points)."""
    return _structured_dev(_native.lib.gsc_summate_incompr_structured_dev, cov_samples, z1, z2,
                           axes, out, form, tolerance, stream, timing, device, True)


def summate_fourier_device(spectrum_factor, modes, z1, z2, pos, out, *, form="auto",
                           tolerance=None, stream=None, timing=False, device=-1):
    """``summate_fourier`` on device arrays; writes ``out`` (n_points,)."""
    dim, n, p = _dev_shapes(modes, pos)
    args = [_cuda_view(spectrum_factor, "spectrum_factor", (n,)),
            _cuda_view(modes, "modes", (dim, n)), _cuda_view(z1, "z1", (n,)),
            _cuda_view(z2, "z2", (n,)), _cuda_view(pos, "pos", (dim, p))]
    o = _opts(form, tolerance, timing, device, stream)
    _native.check(_native.lib.gsc_summate_fourier_dev(*args, dim, n, p,
                                                      _cuda_view(out, "out", (p,)),
                                                      ctypes.byref(o)))
    return out


def summate_fourier_structured_device(spectrum_factor, modes, z1, z2, axes, out, *, form="auto",
                                      tolerance=None, stream=None, timing=False, device=-1):
    """``summate_fourier_structured`` on device arrays; writes ``out`` (n_points,)."""
    return _structured_dev(_native.lib.gsc_summate_fourier_structured_dev, modes, z1, z2, axes,
                           out, form, tolerance, stream, timing, device, False, spectrum_factor)


# ---------------------------------------------------------------------------
# batched ensembles (extension: GSTools calls summate once per realization)
# ---------------------------------------------------------------------------
def _config_dict(c) -> dict:
    names = {v: k for k, v in _native.FORMS.items()}
    return {"form": names.get(c.form, c.form), "points_per_thread": c.points_per_thread,
            "tile_modes": c.tile_modes, "units_per_block": c.units_per_block,
            "blocks": c.blocks, "units": c.units, "max_splits": c.max_splits,
            "tuned": bool(c.tuned), "tune_ms": c.tune_ms, "work": c.work}


def _batch_kind(item) -> str:
    kind = item.get("kind", "scalar")
    if kind not in _native.BATCH_KINDS:
        raise ValueError(f"unknown item kind {kind!r}; choose from {sorted(_native.BATCH_KINDS)}")
    return kind


class Batch:
    """An ensemble of realizations planned for one persistent launch.

    ``items`` is a sequence of dicts of device arrays (``__cuda_array_interface__``,
    C-contiguous float64): ``cov`` (dim, n_modes) -- the mode grid ``modes``
    for Fourier items --, ``z1``, ``z2`` (n_modes), ``pos`` (dim, n_points),
    ``out`` ((n_points,) or (dim, n_points) for ``kind="incompr"``), optional
    ``kind`` ("scalar", "incompr", "fourier") and ``spectrum_factor``
    (n_modes, Fourier).  Each item computes what ``summate`` /
    ``summate_incompr`` / ``summate_fourier`` computes for it.

    Construction tunes the launch configuration on the ensemble's own data
    (writing scratch values into the outputs) unless ``points_per_thread``,
    ``tile_modes`` (FP64 form) and ``units_per_block`` are all given or an
    ensemble of the same shape was tuned before.  ``run`` enqueues one run;
    ``run_graph`` replays a CUDA graph of it.  The arrays stay bound to the
    plan: update their contents in place between runs.
    """

    def __init__(self, items, *, form="auto", tolerance=None, device=-1, timing=False,
                 points_per_thread=0, tile_modes=0, units_per_block=0):
        self._handle = None
        self._keep = list(items)
        arr = (_native.GscBatchItem * max(1, len(self._keep)))()
        for i, it in enumerate(self._keep):
            kind = _batch_kind(it)
            cov = it["modes"] if kind == "fourier" and "modes" in it else it["cov"]
            cs = cov.__cuda_array_interface__["shape"]
            ps = it["pos"].__cuda_array_interface__["shape"]
            if len(cs) != 2 or len(ps) != 2:
                raise TypeError(f"item {i}: cov and pos must be 2-D")
            dim, n = cs
            _assert_eq(dim, ps[0])
            p = ps[1]
            shape = (dim, p) if kind == "incompr" else (p,)
            sf = None
            if kind == "fourier":
                sf = _cuda_view(it["spectrum_factor"], "spectrum_factor", (n,))
            arr[i] = _native.GscBatchItem(
                dim, _native.BATCH_KINDS[kind], n, p, _cuda_view(cov, "cov", (dim, n)),
                _cuda_view(it["z1"], "z1", (n,)), _cuda_view(it["z2"], "z2", (n,)), sf,
                _cuda_view(it["pos"], "pos", (dim, p)), _cuda_view(it["out"], "out", shape))
        o = _opts(form, tolerance, timing, device)
        cfg = _native.make_batch_config(points_per_thread, tile_modes, units_per_block)
        h = ctypes.c_void_p()
        _native.check(_native.lib.gsc_batch_create(arr, len(self._keep), ctypes.byref(o),
                                                    ctypes.byref(cfg), ctypes.byref(h)))
        self._handle = h

    def run(self, stream=None):
        """Enqueues one run on ``stream`` (an int CUDA stream handle; None =
        the legacy default stream); does not synchronise."""
        _native.check(_native.lib.gsc_batch_run(self._handle, stream or None))

    def run_graph(self, stream=None):
        """As ``run``, by replaying a CUDA graph captured on the first call."""
        _native.check(_native.lib.gsc_batch_run_graph(self._handle, stream or None))

    @property
    def config(self) -> dict:
        c = _native.make_batch_config()
        _native.check(_native.lib.gsc_batch_get_config(self._handle, ctypes.byref(c)))
        return _config_dict(c)

    def close(self):
        if self._handle:
            _native.lib.gsc_batch_destroy(self._handle)
            self._handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def summate_batch(items, *, form="auto", tolerance=None, device=-1, timing=False,
                  points_per_thread=0, tile_modes=0, units_per_block=0):
    """Host-array ensemble: ``items`` as for ``Batch`` but numpy float64
    arrays (any layout; copied dense), without ``out``.  Returns the list of
    fields: (n_points,) per scalar or Fourier item, (dim, n_points) C order
    per incompressible item."""
    keep, outs = [], []
    cols = [[] for _ in range(10)]       # the gsc_batch_item fields, by column
    (c_dim, c_kind, c_n, c_p, c_cov, c_z1, c_z2, c_sf, c_pos, c_out) = cols
    for it in items:
        kind = _batch_kind(it)
        cov = np.ascontiguousarray(_array(it["modes"] if kind == "fourier" and "modes" in it
                                          else it["cov"], "cov", 2))
        z1 = np.ascontiguousarray(_array(it["z1"], "z1", 1))
        z2 = np.ascontiguousarray(_array(it["z2"], "z2", 1))
        pos = np.ascontiguousarray(_array(it["pos"], "pos", 2))
        dim, n = cov.shape
        _assert_eq(dim, pos.shape[0])
        _assert_eq(n, z1.shape[0])
        _assert_eq(n, z2.shape[0])
        p = pos.shape[1]
        sf = None
        if kind == "fourier":
            sf = np.ascontiguousarray(_array(it["spectrum_factor"], "spectrum_factor", 1))
            _assert_eq(sf.shape[0], n)
        out, out_ptr = _result_ptr((dim, p) if kind == "incompr" else p)
        keep += [cov, z1, z2, pos, sf]
        outs.append(out)
        c_dim.append(dim)
        c_kind.append(_native.BATCH_KINDS[kind])
        c_n.append(n)
        c_p.append(p)
        c_cov.append(_ptr(cov))
        c_z1.append(_ptr(z1))
        c_z2.append(_ptr(z2))
        c_sf.append(0 if sf is None else _ptr(sf))
        c_pos.append(_ptr(pos))
        c_out.append(out_ptr)
    arr = np.zeros(max(1, len(outs)), dtype=_native.BATCH_ITEM_DTYPE)
    if outs:
        for name, col in zip(_native.BATCH_ITEM_DTYPE.names, cols):
            arr[name] = col
    o = _opts(form, tolerance, timing, device)
    cfg = _native.make_batch_config(points_per_thread, tile_modes, units_per_block)
    _native.check(_native.lib.gsc_summate_batch_f64(
        arr.ctypes.data_as(ctypes.POINTER(_native.GscBatchItem)), len(outs), ctypes.byref(o),
        ctypes.byref(cfg)))
    return outs


def last_batch_config(device=-1) -> dict:
    """Configuration of the plan that the last ``summate_batch`` call used."""
    c = _native.make_batch_config()
    _native.check(_native.lib.gsc_last_batch_config(device, ctypes.byref(c)))
    return _config_dict(c)


# ---------------------------------------------------------------------------
# on-device spectral sampling (extension: GSTools draws these on the host)
# ---------------------------------------------------------------------------
def _spectrum(name) -> int:
    if name not in _native.SPECTRA:
        raise ValueError(f"unknown spectrum {name!r}; choose from {sorted(_native.SPECTRA)}")
    return _native.SPECTRA[name]


def sample_modes(spectrum, dim, n_modes, len_scale, seed, realization=0, *, device=-1):
    """Draws (cov_samples, z1, z2) for one realization on the GPU.

    spectrum "gaussian": k ~ N(0, 2 / len_scale^2) per component;
    "exponential": k = g / |n| / len_scale (multivariate Student-t, one
    degree of freedom).  z1, z2 ~ N(0, 1).  Values depend only on (seed,
    realization, mode): Philox4x32-10 counters.  Returns host arrays
    (dim, n_modes), (n_modes,), (n_modes,)."""
    cov = np.empty((int(dim), int(n_modes)), dtype=np.float64)
    z1 = np.empty(int(n_modes), dtype=np.float64)
    z2 = np.empty(int(n_modes), dtype=np.float64)
    o = _opts("auto", None, False, device)
    _native.check(_native.lib.gsc_sample_modes_f64(
        _spectrum(spectrum), int(dim), int(n_modes), float(len_scale), int(seed) & (2**64 - 1),
        int(realization), cov.ctypes.data, z1.ctypes.data, z2.ctypes.data, ctypes.byref(o)))
    return cov, z1, z2


def sample_modes_batch_device(items, seed, *, stream=None, device=-1, timing=False):
    """Draws many realizations in one launch into device arrays: each item a
    dict with "spectrum", "len_scale", "realization" and CUDA arrays "cov"
    (dim, n_modes), "z1", "z2" (n_modes,).  Does not synchronise."""
    arr = (_native.GscSampleItem * max(1, len(items)))()
    for i, it in enumerate(items):
        shape = it["cov"].__cuda_array_interface__["shape"]
        if len(shape) != 2:
            raise TypeError(f"item {i}: cov must be 2-D")
        dim, n = shape
        arr[i] = _native.GscSampleItem(
            _spectrum(it["spectrum"]), dim, n, float(it["len_scale"]), int(it.get("realization", i)),
            _cuda_view(it["cov"], "cov", (dim, n)), _cuda_view(it["z1"], "z1", (n,)),
            _cuda_view(it["z2"], "z2", (n,)))
    o = _opts("auto", None, timing, device, stream)
    _native.check(_native.lib.gsc_sample_modes_batch_dev(arr, len(items),
                                                         int(seed) & (2**64 - 1), ctypes.byref(o)))


def release_buffers(device=-1) -> None:
    """Frees the scratch and staging memory the library keeps on ``device``
    between calls (and the cached plan of ``summate_batch``); the next call
    allocates again.  Plans held as ``Batch`` objects stay."""
    _native.check(_native.lib.gsc_release_buffers(device))


def device_status(device=-1) -> None:
    """Raises GscError if a kernel of an earlier device-array call on ``device``
    reported a failed pipeline wait, a mixed-form call met a wave number past
    its integer phase range, or an explicit ``form="sep_f16x5"`` call met
    inputs past the bound of its exact leading sum (the output of that call is
    invalid; form "auto" recomputes such calls on an FP64 form).  The report
    is cleared once raised."""
    _native.check(_native.lib.gsc_device_status(device))
