"""Flattened structured meshes passed to the point API (GPU tests).

GSTools lays out the points of a structured mesh as
meshgrid(*axes, indexing="ij") flattened in C order before it calls
summate / summate_incompr / summate_fourier.  With form "auto" the library
recognises that layout (every point checked) and computes on the axes with
the separable FP64 form, within the same 1e-12 bar as the plain kernel;
anything else -- a perturbed point, repeated axis values, an explicit form --
takes the point kernels.  Checked against the oracle in every case.
"""
import os

import numpy as np
import pytest

import oracle
from conftest import rel_err

pytestmark = pytest.mark.gpu

NT = os.cpu_count() or 1


def _flat(axes):
    return np.ascontiguousarray(np.array(np.meshgrid(*axes, indexing="ij")).reshape(len(axes), -1))


def _kernels(gsc):
    return {name for name, _ in gsc.last_timings()}


def _case(seed, shape, n):
    rng = np.random.default_rng(seed)
    dim = len(shape)
    cov = rng.normal(0.0, 0.3, (dim, n))
    z1, z2 = rng.standard_normal(n), rng.standard_normal(n)
    axes = tuple(np.sort(rng.uniform(-20, 20, s)) for s in shape)
    return cov, z1, z2, axes


@pytest.mark.parametrize("shape", [(20, 30, 40), (100, 90)])
def test_scalar_grid_is_routed(gsc, shape):
    cov, z1, z2, axes = _case(1, shape, 300)
    pos = _flat(axes)
    out = gsc.summate(cov, z1, z2, pos, timing=True)
    assert "sep_f64_dmma" in _kernels(gsc)
    assert rel_err(out, oracle.summator(cov, z1, z2, pos, num_threads=NT)) <= 1e-12


def test_incompr_grid_fortran_output(gsc):
    cov, z1, z2, axes = _case(2, (16, 24, 32), 200)
    pos = _flat(axes)
    out = gsc.summate_incompr(cov, z1, z2, pos, timing=True)
    assert "sep_f64_dmma" in _kernels(gsc)
    assert out.flags.f_contiguous and out.shape == (3, pos.shape[1])
    assert rel_err(out, oracle.summator_incompr(cov, z1, z2, pos, num_threads=NT)) <= 1e-12


def test_fourier_grid_is_routed(gsc):
    rng = np.random.default_rng(3)
    m = np.array(np.meshgrid(*[np.arange(-6, 7)] * 2, indexing="ij")).reshape(2, -1)
    modes = np.ascontiguousarray(m[:, np.any(m != 0, axis=0)] * (2 * np.pi / 50.0))
    n = modes.shape[1]
    sf = rng.uniform(0.1, 1.0, n)
    z1, z2 = rng.standard_normal(n), rng.standard_normal(n)
    pos = _flat((np.arange(80) * 0.625, np.arange(60) * 0.625))
    out = gsc.summate_fourier(sf, modes, z1, z2, pos, timing=True)
    assert "sep_f64_dmma" in _kernels(gsc)
    assert rel_err(out, oracle.summator_fourier(sf, modes, z1, z2, pos, num_threads=NT)) <= 1e-12


def test_strided_grid_view_is_routed(gsc):
    cov, z1, z2, axes = _case(4, (20, 25, 30), 150)
    pos_f = np.asfortranarray(_flat(axes))
    out = gsc.summate(cov, z1, z2, pos_f, timing=True)
    assert "sep_f64_dmma" in _kernels(gsc)
    assert rel_err(out, oracle.summator(cov, z1, z2, pos_f, num_threads=NT)) <= 1e-12


def test_not_a_grid_takes_the_point_kernel(gsc):
    cov, z1, z2, axes = _case(5, (20, 30, 40), 120)
    pos = _flat(axes)
    pos[2, 12345] += 1e-9                                   # one point off the grid
    out = gsc.summate(cov, z1, z2, pos, timing=True)
    assert "sep_f64_dmma" not in _kernels(gsc)
    assert rel_err(out, oracle.summator(cov, z1, z2, pos, num_threads=NT)) <= 1e-12
    # repeated values on an axis: not separable as detected, still correct
    ax = (np.array([0.0, 0.0, 1.0, 2.0] * 10), np.arange(50.0), np.arange(40.0))
    pos = _flat(ax)
    out = gsc.summate(cov, z1, z2, pos)
    assert rel_err(out, oracle.summator(cov, z1, z2, pos, num_threads=NT)) <= 1e-12


def test_explicit_form_is_not_routed(gsc):
    cov, z1, z2, axes = _case(6, (20, 30, 40), 100)
    pos = _flat(axes)
    gsc.summate(cov, z1, z2, pos, form="plain", timing=True)
    assert "sep_f64_dmma" not in _kernels(gsc)


def test_incompr_grid_fortran_output_waves(gsc):
    """A grid of many row tiles at tolerance 1e-6 (sep_f16x5 in waves): the
    rows of each wave are rearranged into the Fortran-ordered result on the
    device and copied while the next wave computes."""
    cov, z1, z2, axes = _case(7, (160, 256, 40), 200)
    pos = _flat(axes)
    out = gsc.summate_incompr(cov, z1, z2, pos, tolerance=1e-6, timing=True)
    k = _kernels(gsc)
    assert "sep_tc_f16x5" in k and "interleave" in k
    # every timed launch has its own record, nested ones included
    assert all(ms >= 0 for _, ms in gsc.last_timings())
    assert out.flags.f_contiguous and out.shape == (3, pos.shape[1])
    idx = np.sort(np.random.default_rng(0).choice(pos.shape[1], 4096, replace=False))
    ref = oracle.summator_incompr(cov, z1, z2, np.ascontiguousarray(pos[:, idx]), num_threads=NT)
    assert rel_err(out[:, idx], ref) <= 1e-6
    # the same field through the structured entry point, C-ordered
    ref_s = gsc.summate_incompr_structured(cov, z1, z2, axes, tolerance=1e-6)
    assert np.array_equal(out, ref_s.reshape(3, -1))


@pytest.mark.parametrize("grid", [True, False])
def test_incompr_any_output_strides(gsc, grid):
    """The C ABI takes any element strides for the result: a padded
    (n_points, 4) buffer neither C- nor Fortran-ordered, on a grid and off
    it."""
    import ctypes
    from gstools_core import _native
    cov, z1, z2, axes = _case(8, (12, 20, 30), 150)
    pos = _flat(axes)
    if not grid:
        pos[0, 7] += 1e-9
    P = pos.shape[1]
    buf = np.full((P, 4), np.nan)
    rc = _native.lib.gsc_summate_incompr_f64(
        cov.ctypes.data, cov.shape[1], 1, z1.ctypes.data, 1, z2.ctypes.data, 1,
        pos.ctypes.data, P, 1, 3, cov.shape[1], P, buf.ctypes.data, 1, 4, None)
    assert rc == 0, _native.lib.gsc_last_error()
    assert np.isnan(buf[:, 3]).all()
    ref = oracle.summator_incompr(cov, z1, z2, pos, num_threads=NT)
    assert rel_err(buf[:, :3].T, ref) <= 1e-12


def _device_slices(n0, dim, nout=1):
    """x-slices the device checks: the first n0 (0.687 - 0.313 nout / dim)
    (at least one, not all)."""
    return max(1, min(n0 - 1, n0 * (687 - 313 * nout // dim) // 1000))


@pytest.mark.parametrize("where", ["clean", "device_half", "host_half", "nan_device_half",
                                   "device_last", "host_first"])
def test_large_mesh_check_shared_with_the_device(gsc, where):
    """Meshes of 32 MiB and more, where the GPU reads host memory in place:
    the GPU checks the first x-slices over the host link (a share that
    balances the link against the host cores) while the host cores check
    the rest.  A clean mesh takes the separable form;
    one coordinate moved by an ulp (or a NaN) in either half sends the call
    to the point kernels.  Against the oracle on a subset that holds the
    changed point."""
    shape = (64, 128, 256)                                  # 2.1 M points, 50 MB
    cov, z1, z2, axes = _case(7, shape, 64)
    pos = _flat(axes)
    L0 = shape[1] * shape[2]
    na = _device_slices(shape[0], 3)
    p = {"device_last": na * L0 - 1, "host_first": na * L0}.get(
        where, 1234 + (5 if where != "host_half" else shape[0] - 3) * L0)
    if where == "nan_device_half":
        pos[2, p] = np.nan
    elif where != "clean":
        pos[1, p] = np.nextafter(pos[1, p], np.inf)
    out = gsc.summate(cov, z1, z2, pos, timing=True)
    ks = _kernels(gsc)
    if where == "clean":
        assert "sep_f64_dmma" in ks
    else:
        assert "sep_f64_dmma" not in ks and any(k.startswith("plain") for k in ks), ks
    idx = np.unique(np.concatenate([np.random.default_rng(8).choice(pos.shape[1], 2048, replace=False), [p]]))
    ref = oracle.summator(cov, z1, z2, np.ascontiguousarray(pos[:, idx]), num_threads=NT)
    got = out[idx]
    bad = np.isnan(ref)
    assert np.array_equal(np.isnan(got), bad)
    assert rel_err(got[~bad], ref[~bad]) <= 1e-12


@pytest.mark.parametrize("where", ["clean", "device_row", "host_row"])
def test_large_2d_mesh_check(gsc, where):
    """A 2-D flattened mesh of 64 MiB: the device checks whole x-slices as
    rows.  One coordinate moved by an ulp in a device or a host slice sends
    the call to the point kernels."""
    shape = (2048, 2048)
    cov, z1, z2, axes = _case(9, shape, 48)
    pos = _flat(axes)
    na = _device_slices(shape[0], 2)
    p = {"device_row": (na - 1) * shape[1] + 77, "host_row": na * shape[1] + 5}.get(where, 0)
    if where != "clean":
        pos[1, p] = np.nextafter(pos[1, p], -np.inf)
    out = gsc.summate(cov, z1, z2, pos, timing=True)
    ks = _kernels(gsc)
    if where == "clean":
        assert "sep_f64_dmma" in ks
    else:
        assert "sep_f64_dmma" not in ks, ks
    idx = np.unique(np.concatenate([np.random.default_rng(10).choice(pos.shape[1], 2048, replace=False), [p]]))
    ref = oracle.summator(cov, z1, z2, np.ascontiguousarray(pos[:, idx]), num_threads=NT)
    assert rel_err(out[idx], ref) <= 1e-12
