"""The field-benchmark input files of GSTools-Core, read and written here.

The reference's criterion benchmarks (``benches/main.rs:51-133``) read their
inputs from text files in ``benches/input`` that its generator script writes
with ``numpy.savetxt`` (``benches/gen_benchmark_inputs.py:10-34``): one value
per line for 1-D arrays, one whitespace-separated row per line for 2-D ones
(``benches/main.rs:20-49``).  The generator needs GSTools; where it is absent,
``synthesize_field_inputs`` writes stand-ins with the same names, shapes and
kinds of values, so the same file path can be replayed by ``bench.py
--workload field``.
"""
from __future__ import annotations

import os

import numpy as np

FILES_1D = ("field_x.txt", "field_y.txt", "field_z.txt", "field_z_1.txt", "field_z_2.txt",
            "field_fourier_z_1.txt", "field_fourier_z_2.txt", "field_fourier_factor_2d.txt")
FILES_2D = ("field_cov_samples_2d.txt", "field_cov_samples_3d.txt", "field_fourier_modes_2d.txt")


def read_1d(path) -> np.ndarray:
    """One float per line (benches/main.rs:20-28)."""
    with open(path) as fh:
        return np.array([float(line) for line in fh if line.strip()], dtype=np.float64)


def read_2d(path) -> np.ndarray:
    """Whitespace-separated rows, shape (lines, values / lines) (benches/main.rs:30-49)."""
    vals, lines = [], 0
    with open(path) as fh:
        for line in fh:
            if not line.strip():
                continue
            vals.extend(float(v) for v in line.split())
            lines += 1
    if lines == 0:
        return np.zeros((0, 0))
    return np.array(vals, dtype=np.float64).reshape(lines, len(vals) // lines)


def write_1d(path, a) -> None:
    np.savetxt(path, np.asarray(a, dtype=np.float64))


def write_2d(path, a) -> None:
    np.savetxt(path, np.asarray(a, dtype=np.float64))


def field_inputs(directory) -> dict:
    """The arrays benches/main.rs:51-74 builds from the files in `directory`."""
    r1 = {f: read_1d(os.path.join(directory, f)) for f in FILES_1D}
    r2 = {f: read_2d(os.path.join(directory, f)) for f in FILES_2D}
    x, y, z = r1["field_x.txt"], r1["field_y.txt"], r1["field_z.txt"]
    return {
        "pos_2d": np.stack([x, y]),
        "pos_3d": np.stack([x, y, z]),
        "cov_samples_2d": r2["field_cov_samples_2d.txt"],
        "cov_samples_3d": r2["field_cov_samples_3d.txt"],
        "z_1": r1["field_z_1.txt"],
        "z_2": r1["field_z_2.txt"],
        "z_1_fourier": r1["field_fourier_z_1.txt"],
        "z_2_fourier": r1["field_fourier_z_2.txt"],
        "spectrum_factor_2d": r1["field_fourier_factor_2d.txt"],
        "modes_2d": r2["field_fourier_modes_2d.txt"],
    }


def synthesize_field_inputs(directory, seed=19031977, pos_no=10_000, mode_no=1_000,
                            fourier_cut=16) -> None:
    """Writes stand-ins for the generator's files: the same point lines
    (linspace over [0, 10], [-5, 5], [-6, 8]), mode_no wave vectors from a
    Gaussian spectrum of unit length scale, standard-normal z1, z2, and a
    Fourier grid of period 10 in both directions (|m| <= fourier_cut per
    axis, origin excluded) with Gaussian spectrum factors.  Seeded numpy
    default_rng; GSTools' own sampling is not reproduced."""
    os.makedirs(directory, exist_ok=True)
    rng = np.random.default_rng(seed)
    j = lambda f: os.path.join(directory, f)
    write_1d(j("field_x.txt"), np.linspace(0.0, 10.0, pos_no))
    write_1d(j("field_y.txt"), np.linspace(-5.0, 5.0, pos_no))
    write_1d(j("field_z.txt"), np.linspace(-6.0, 8.0, pos_no))
    write_2d(j("field_cov_samples_2d.txt"), rng.normal(0.0, np.sqrt(np.pi / 2.0), (2, mode_no)))
    write_2d(j("field_cov_samples_3d.txt"), rng.normal(0.0, np.sqrt(np.pi / 2.0), (3, mode_no)))
    write_1d(j("field_z_1.txt"), rng.standard_normal(mode_no))
    write_1d(j("field_z_2.txt"), rng.standard_normal(mode_no))
    ticks = np.arange(-fourier_cut, fourier_cut + 1) * (2.0 * np.pi / 10.0)
    grid = np.array(np.meshgrid(ticks, ticks, indexing="ij")).reshape(2, -1)
    modes = grid[:, np.any(grid != 0.0, axis=0)]
    n = modes.shape[1]
    dk = (2.0 * np.pi / 10.0) ** 2
    spectrum = np.exp(-np.sum(modes ** 2, axis=0) / np.pi) / (2.0 * np.pi)
    write_2d(j("field_fourier_modes_2d.txt"), modes)
    write_1d(j("field_fourier_factor_2d.txt"), np.sqrt(2.0 * spectrum * dk))
    write_1d(j("field_fourier_z_1.txt"), rng.standard_normal(n))
    write_1d(j("field_fourier_z_2.txt"), rng.standard_normal(n))
