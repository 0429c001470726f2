"""Structured-mesh recognition of the point entry points, without a GPU.

GSTools passes a structured field to `summate` as the flattened
meshgrid(*axes, indexing="ij"); the point entry points recognise that
layout under form AUTO and compute on the axes (the separable forms).  The
recognition (capi.cu: detect_grid) runs on the host alone and is reached
here through gsc_selftest_detect_grid: it must accept exactly the C-order
ij meshes (any element strides), with every point checked, and refuse
everything else, so that no other point set is ever computed as a grid.
"""
import ctypes

import numpy as np
import pytest


def _detect(pos):
    from gstools_core import _native
    pos = np.asarray(pos, dtype=np.float64)
    n = (ctypes.c_int64 * 3)()
    s = pos.strides
    rc = _native.lib.gsc_selftest_detect_grid(pos.ctypes.data, s[0] // 8, s[1] // 8,
                                              pos.shape[0], pos.shape[1], n)
    assert rc == _native.GSC_OK
    return tuple(n)


def _mesh(*axes, indexing="ij"):
    g = np.meshgrid(*axes, indexing=indexing)
    return np.array([a.reshape(-1) for a in g])


@pytest.mark.parametrize("shape", [(64, 80), (2, 2048), (16, 20, 24), (3, 40, 50), (40, 2, 60)])
def test_c_order_meshes_are_recognised(gsc, shape):
    rng = np.random.default_rng(len(shape) + shape[0])
    axes = [np.sort(rng.uniform(-50.0, 50.0, s)) for s in shape]
    pos = _mesh(*axes)
    assert _detect(pos) == tuple(shape) + (0,) * (3 - len(shape))
    # the same points through a Fortran-ordered (transposed) buffer
    pos_f = np.asfortranarray(pos)
    assert pos_f.strides[0] == 8
    assert _detect(pos_f) == _detect(pos)


def test_any_changed_point_is_refused(gsc):
    pos = _mesh(np.arange(32.0), np.arange(40.0), np.arange(8.0))
    P = pos.shape[1]
    assert _detect(pos) == (32, 40, 8)
    for i in (0, 1, P // 2 + 3, P - 1):
        for d in range(3):
            bad = pos.copy()
            bad[d, i] = np.nextafter(bad[d, i], np.inf)
            assert _detect(bad) == (0, 0, 0), (i, d)
    bad = pos.copy()
    bad[1, 777] = np.nan
    assert _detect(bad) == (0, 0, 0)


@pytest.mark.parametrize("case", ["xy", "repeated", "small", "random", "dim1", "dim4", "single"])
def test_other_point_sets_are_refused(gsc, case):
    rng = np.random.default_rng(5)
    if case == "xy":
        pos = _mesh(np.arange(64.0), np.arange(80.0), indexing="xy")
    elif case == "repeated":
        a0 = np.array([0.0, 0.0] + list(range(1, 62)), dtype=np.float64)
        pos = _mesh(a0, np.arange(80.0))
    elif case == "small":
        pos = _mesh(np.arange(60.0), np.arange(60.0))      # 3600 points: below the routing size
    elif case == "random":
        pos = rng.uniform(0.0, 10.0, (3, 10000))
    elif case == "dim1":
        pos = np.arange(10000.0)[None, :]
    elif case == "dim4":
        pos = _mesh(*(np.arange(10.0),) * 4)
    else:
        pos = _mesh(np.array([3.0]), np.arange(5000.0))   # an axis of one point
    assert _detect(pos) == (0, 0, 0)


def test_argument_errors(gsc):
    from gstools_core import _native
    pos = _mesh(np.arange(64.0), np.arange(80.0))
    rc = _native.lib.gsc_selftest_detect_grid(pos.ctypes.data, pos.shape[1], 1, 2, pos.shape[1],
                                              None)
    assert rc == _native.GSC_ERR_INVALID
    n = (ctypes.c_int64 * 3)()
    assert _native.lib.gsc_selftest_detect_grid(None, 1, 1, 2, 100, n) == _native.GSC_ERR_INVALID
    assert _native.lib.gsc_selftest_detect_grid(None, 1, 1, 2, 0, n) == _native.GSC_OK
    assert tuple(n) == (0, 0, 0)
