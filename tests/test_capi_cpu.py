"""The C-ABI library and the gstools_core host logic, without a GPU.

Checks that libgstools_core_gb300.so loads and exports every function the
public header declares, and that the Python layer reproduces the reference's
argument handling (src/lib.rs:33-65: PyReadonlyArray extraction errors,
Option<usize> num_threads, the shape asserts of src/field.rs:44-46).
No compute call is made unless a GPU is present.
"""
import ctypes
import glob
import os
import re

import numpy as np
import pytest

from conftest import ROOT


def _declared_symbols():
    names = []
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"^[A-Za-z_][\w \*]*?\b(gsc_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = _declared_symbols()
    for n in ("gsc_summate_f64", "gsc_summate_incompr_f64", "gsc_summate_dev",
              "gsc_summate_incompr_dev", "gsc_last_error", "gsc_version"):
        assert n in names


def test_library_exports_every_declared_symbol(native_lib):
    lib = ctypes.CDLL(native_lib)
    missing = [n for n in _declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header(gsc):
    from gstools_core import _native
    assert set(_declared_symbols()) == set(_native.SIGNATURES)


def test_version(gsc):
    assert gsc.__version__ == "1.1.0"
    assert gsc.native_version.startswith("1.1.0")


def _args(dim=3, n=10, p=8):
    rng = np.random.default_rng(0)
    return (rng.normal(size=(dim, n)), rng.normal(size=n), rng.normal(size=n),
            rng.normal(size=(dim, p)))


@pytest.mark.parametrize("fn", ["summate", "summate_incompr"])
def test_type_errors_like_pyo3(gsc, fn):
    f = getattr(gsc, fn)
    cov, z1, z2, pos = _args()
    with pytest.raises(TypeError, match="cov_samples"):
        f(cov.tolist(), z1, z2, pos)
    with pytest.raises(TypeError, match="type mismatch"):
        f(cov.astype(np.float32), z1, z2, pos)
    with pytest.raises(TypeError, match="dimensionality mismatch"):
        f(cov, z1[:, None], z2, pos)
    with pytest.raises(TypeError, match="pos"):
        f(cov, z1, z2, pos.astype(np.int64))
    with pytest.raises(TypeError):
        f(cov, z1, z2, pos, 2.5)
    with pytest.raises(OverflowError):
        f(cov, z1, z2, pos, -1)


@pytest.mark.parametrize("fn", ["summate", "summate_incompr"])
def test_shape_asserts_raise_value_error(gsc, fn):
    f = getattr(gsc, fn)
    cov, z1, z2, pos = _args()
    with pytest.raises(ValueError, match="left: 3\n right: 2"):
        f(cov, z1, z2, pos[:2])
    with pytest.raises(ValueError, match="left: 10\n right: 9"):
        f(cov, z1[:9], z2, pos)
    with pytest.raises(ValueError, match="left: 10\n right: 11"):
        f(cov, z1, np.zeros(11), pos)


def test_incompr_dimension_error(gsc):
    for dim in (1, 4):
        cov, z1, z2, pos = _args(dim=dim)
        with pytest.raises(ValueError, match="two- and three-dimensional"):
            gsc.summate_incompr(cov, z1, z2, pos)


def test_empty_points_need_no_device(gsc):
    cov, z1, z2, _ = _args()
    out = gsc.summate(cov, z1, z2, np.zeros((3, 0)))
    assert out.shape == (0,) and out.dtype == np.float64
    out = gsc.summate_incompr(cov, z1, z2, np.zeros((3, 0)))
    assert out.shape == (3, 0)


def test_abi_validation_without_device(native_lib):
    """Bad arguments are rejected before any CUDA call, with a message."""
    from gstools_core import _native
    lib = _native.lib
    o = _native.make_opts()
    rc = lib.gsc_summate_f64(None, 1, 1, None, 1, None, 1, None, 1, 1, 3, 10, 8, None, 1,
                             ctypes.byref(o))
    assert rc == _native.GSC_ERR_INVALID
    assert b"NULL" in lib.gsc_last_error()
    rc = lib.gsc_summate_f64(None, 1, 1, None, 1, None, 1, None, 1, 1, -1, 10, 8, None, 1, None)
    assert rc == _native.GSC_ERR_INVALID
    bad = _native.make_opts()
    bad.struct_size = 4
    cov, z1, z2, pos = _args()
    out = np.empty(8)
    rc = lib.gsc_summate_f64(cov.ctypes.data, 10, 1, z1.ctypes.data, 1, z2.ctypes.data, 1,
                             pos.ctypes.data, 8, 1, 3, 10, 8, out.ctypes.data, 1,
                             ctypes.byref(bad))
    assert rc == _native.GSC_ERR_INVALID
    rc = lib.gsc_summate_incompr_f64(cov.ctypes.data, 10, 1, z1.ctypes.data, 1, z2.ctypes.data,
                                     1, pos.ctypes.data, 8, 1, 4, 10, 8, out.ctypes.data, 8, 1,
                                     None)
    assert rc == _native.GSC_ERR_DIM


def test_no_device_fails_loudly(gsc):
    """Without a GPU the compute path raises; it never falls back to the CPU."""
    if gsc.device_count() > 0:
        pytest.skip("a CUDA device is present")
    cov, z1, z2, pos = _args()
    with pytest.raises(gsc.GscError, match="no usable CUDA device"):
        gsc.summate(cov, z1, z2, pos)
    with pytest.raises(gsc.GscError, match="no usable CUDA device"):
        gsc.summate_incompr(cov, z1, z2, pos)


def test_result_pool_without_device(gsc):
    """Without a device the pinned pool cannot allocate: results fall back to
    ordinary numpy arrays, and the pool's bookkeeping calls still answer."""
    import ctypes
    from gstools_core import _native
    if gsc.device_count() > 0:
        pytest.skip("a CUDA device is present")
    a = gsc._result((3, 100_000), order="F")
    assert a.flags.owndata and a.flags.f_contiguous and a.shape == (3, 100_000)
    ptr = ctypes.c_void_p()
    assert _native.lib.gsc_host_alloc(1 << 20, ctypes.byref(ptr)) == _native.GSC_ERR_NO_DEVICE
    assert _native.lib.gsc_host_free(None) == 0
    assert gsc.host_pool_stats() == {"live_bytes": 0, "cached_bytes": 0}
    gsc.host_pool_trim()
