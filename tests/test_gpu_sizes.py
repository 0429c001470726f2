"""Exhaustive small sizes at every tile edge, against the oracle (GPU tests).

Point and mode counts run over 0, 1 and one below / at / above each tile
boundary of the kernels they reach:
  plain FP64      8 modes per staged tile, 128 threads x 4 points per block
  mixed           32 modes per FP32 tile, 128 threads x 4 points per block
  batch           the same tiles inside the persistent kernels
  sep_f64 / x5    128 grid rows per tile (slices x rows for d = 3), 192 or
                  256 columns per tile, 16 modes per k-block, 256 modes per
                  cross drain, split tails from 16 k-blocks up
Each output equals the reference's summator, summator_incompr or
summator_fourier (src/field.rs:37-65, :97-182, :219-249) on the same inputs,
with the form's bar on max |err| over max(field RMS, sqrt(sum z^2 / 2)), the
expected field RMS of the modes, so that a field that is small at its few
points by chance does not turn rounding into a failure.  Where the reference
gives exact zeros (no modes), the output is exact zeros.
"""
import os
import zlib

import numpy as np
import pytest

import oracle
from conftest import rms

pytestmark = pytest.mark.gpu

NT = os.cpu_count() or 1
BOUND = {"plain": 1e-12, "plain_libm": 1e-12, "mixed": 1e-6, "sep_f64": 1e-12,
         "sep_f16x5": 1e-6}
MODES = (0, 1, 7, 8, 9, 31, 32, 33)
POINTS = (0, 1, 31, 32, 33, 127, 128, 129, 511, 512, 513)


def _modes(rng, dim, n, kind):
    if kind == "fourier":
        return rng.integers(-12, 13, (dim, n)) * (2.0 * np.pi / 40.0)
    return rng.normal(0.0, 0.4, (dim, n))


def _scaled_err(got, ref, z1, z2):
    got, ref = np.asarray(got), np.asarray(ref)
    assert got.shape == ref.shape
    if ref.size == 0:
        return 0.0
    if not np.any(ref):
        return 0.0 if np.array_equal(got, ref) else np.inf
    scale = max(rms(ref), np.sqrt(0.5 * (np.sum(z1 * z1) + np.sum(z2 * z2))))
    return float(np.max(np.abs(got - ref)) / scale)


def _oracle(kind, sf, cov, z1, z2, pos):
    if kind == "incompr":
        return oracle.summator_incompr(cov, z1, z2, pos, num_threads=NT)
    if kind == "fourier":
        return oracle.summator_fourier(sf, cov, z1, z2, pos, num_threads=NT)
    return oracle.summator(cov, z1, z2, pos, num_threads=NT)


def _gpu(gsc, kind, sf, cov, z1, z2, pos, form):
    if kind == "incompr":
        return gsc.summate_incompr(cov, z1, z2, pos, form=form)
    if kind == "fourier":
        return gsc.summate_fourier(sf, cov, z1, z2, pos, form=form)
    return gsc.summate(cov, z1, z2, pos, form=form)


@pytest.mark.parametrize("form", ["plain", "plain_libm", "mixed"])
@pytest.mark.parametrize("kind,dim", [("scalar", 1), ("scalar", 3), ("incompr", 2),
                                      ("incompr", 3), ("fourier", 2)])
def test_point_and_mode_edges(gsc, form, kind, dim):
    rng = np.random.default_rng(zlib.crc32(f"{form} {kind} {dim}".encode()))
    bad = []
    for n in MODES:
        for p in POINTS:
            cov = _modes(rng, dim, n, kind)
            z1, z2 = rng.standard_normal(n), rng.standard_normal(n)
            sf = rng.uniform(0.1, 1.0, n)
            pos = rng.uniform(-30.0, 30.0, (dim, p))
            ref = _oracle(kind, sf, cov, z1, z2, pos)
            got = _gpu(gsc, kind, sf, cov, z1, z2, pos, form)
            err = _scaled_err(got, ref, z1 * (sf if kind == "fourier" else 1.0),
                              z2 * (sf if kind == "fourier" else 1.0))
            if not err <= BOUND[form]:
                bad.append((n, p, err))
    assert not bad, f"{form} {kind} d={dim}: (modes, points, err) {bad[:8]}"


@pytest.mark.parametrize("form", ["plain", "mixed"])
def test_mode_tile_multiples(gsc, form):
    """Mode counts around the chunk and record boundaries (255 to 257, 1023
    to 1025) on point counts around one block."""
    rng = np.random.default_rng(11)
    for n in (255, 256, 257, 1023, 1024, 1025):
        for p in (511, 512, 513):
            cov = rng.normal(0.0, 0.4, (3, n))
            z1, z2 = rng.standard_normal(n), rng.standard_normal(n)
            pos = rng.uniform(-30.0, 30.0, (3, p))
            ref = oracle.summator(cov, z1, z2, pos, num_threads=NT)
            err = _scaled_err(gsc.summate(cov, z1, z2, pos, form=form), ref, z1, z2)
            assert err <= BOUND[form], (n, p, err)


def _flat(axes):
    return np.ascontiguousarray(np.array(np.meshgrid(*axes, indexing="ij")).reshape(len(axes), -1))


# (shape, what it reaches): rows = slices x rows for d = 3, columns = the
# last axis (times the component count for the incompressible field)
GRIDS = [((1, 1), "one point"), ((127, 191), "one row tile, one 192 tile"),
         ((128, 192), "exact tiles"), ((129, 193), "ragged rows and columns"),
         ((1, 256), "one 256 tile"), ((5, 257), "257 columns"),
         ((2, 64, 33), "128 rows over two slices"), ((3, 43, 65), "129 rows over slices"),
         ((40, 96), "components of 96 columns"), ((3, 50, 64), "components of 64 columns"),
         ((0, 9), "no points")]


@pytest.mark.parametrize("form", ["sep_f64", "sep_f16x5"])
@pytest.mark.parametrize("n", [1, 15, 16, 17, 255, 257])
def test_structured_tile_edges(gsc, form, n):
    rng = np.random.default_rng(n)
    bad = []
    for shape, what in GRIDS:
        dim = len(shape)
        cov = rng.normal(0.0, 0.3, (dim, n))
        z1, z2 = rng.standard_normal(n), rng.standard_normal(n)
        axes = tuple(0.7 * np.arange(s, dtype=np.float64) - 3.0 for s in shape)
        ref = oracle.summator(cov, z1, z2, _flat(axes), num_threads=NT)
        got = gsc.summate_structured(cov, z1, z2, axes, form=form)
        err = _scaled_err(np.asarray(got).reshape(-1), ref, z1, z2)
        if not err <= BOUND[form]:
            bad.append((what, err))
        if dim >= 2 and shape[0] > 0:
            refi = oracle.summator_incompr(cov, z1, z2, _flat(axes), num_threads=NT)
            goti = gsc.summate_incompr_structured(cov, z1, z2, axes, form=form)
            erri = _scaled_err(np.asarray(goti).reshape(dim, -1), refi, z1, z2)
            if not erri <= BOUND[form]:
                bad.append(("incompr " + what, erri))
    assert not bad, f"{form} x {n} modes: {bad}"


@pytest.mark.parametrize("form", ["plain", "mixed"])
def test_batch_tile_edges(gsc, form):
    """One batch over items at every edge size: the persistent kernels'
    units cut the same boundaries as the single-call kernels."""
    rng = np.random.default_rng(5)
    items = []
    for i, (n, p) in enumerate((n, p) for n in (0, 1, 8, 9, 31, 33, 257) for p in (0, 1, 127, 129, 513)):
        kind = ("scalar", "incompr", "fourier")[i % 3]
        dim = 2 + i % 2
        it = {"kind": kind, "cov": np.ascontiguousarray(_modes(rng, dim, n, kind)),
              "z1": rng.standard_normal(n), "z2": rng.standard_normal(n),
              "pos": rng.uniform(-30.0, 30.0, (dim, p))}
        if kind == "fourier":
            it["spectrum_factor"] = rng.uniform(0.1, 1.0, n)
        items.append(it)
    outs = gsc.summate_batch([dict(it) for it in items], form=form,
                             tolerance=1e-6 if form == "mixed" else None)
    bad = []
    for it, got in zip(items, outs):
        sf = it.get("spectrum_factor")
        ref = _oracle(it["kind"], sf, it["cov"], it["z1"], it["z2"], it["pos"])
        w = sf if sf is not None else 1.0
        err = _scaled_err(got, ref, it["z1"] * w, it["z2"] * w)
        if not err <= BOUND[form]:
            bad.append((it["kind"], it["z1"].size, it["pos"].shape[1], err))
    assert not bad, bad
