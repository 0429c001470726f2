"""Structured-grid forms against the oracle on the expanded meshgrid (GPU tests).

The oracle evaluates the reference's summator (src/field.rs:37-65,
src/field.rs:97-182) on pos = meshgrid(*axes, indexing="ij") flattened, the
points GSTools passes for a structured mesh.  Bars (max |err| / field RMS):
  plain FP64 on the expanded grid              1e-12
  sep_f16x5 (tcgen05, exact leading product)   1e-6   (the bar of the reduced-precision forms)
  sep_f16x3 (tcgen05, f16 hi/lo)               1e-5
  sep_bf16x3 (tcgen05, bf16 hi/lo)             1e-4
"""
import os

import numpy as np
import pytest

import oracle
from conftest import rel_err, rms

pytestmark = pytest.mark.gpu

NT = os.cpu_count() or 1
BOUND = {"plain": 1e-12, "sep_f64": 1e-12, "sep_f16x5": 1e-6, "sep_f16x3": 1e-5,
         "sep_bf16x3": 1e-4}


def _grid_case(seed, shape, n, kscale=0.3, heavy=False, spacing=1.0, origin=0.0):
    rng = np.random.default_rng(seed)
    dim = len(shape)
    if heavy:
        cov = rng.standard_normal((dim, n)) / np.sqrt(rng.chisquare(1, n)) * kscale
    else:
        cov = rng.normal(0.0, kscale, (dim, n))
    z1, z2 = rng.standard_normal(n), rng.standard_normal(n)
    axes = tuple(origin + spacing * np.arange(s, dtype=np.float64) for s in shape)
    return cov, z1, z2, axes


def _flat(axes):
    return np.ascontiguousarray(np.array(np.meshgrid(*axes, indexing="ij")).reshape(len(axes), -1))


def _report(name, err):
    print(f"{name}: max|err|/rms = {err:.3e}")


@pytest.mark.parametrize("form", ["plain", "sep_f64", "sep_f16x5", "sep_f16x3", "sep_bf16x3"])
@pytest.mark.parametrize("shape,n", [
    ((37, 300), 100),          # 2-D: 1 row tile, 2 column tiles
    ((20, 150, 40), 77),       # 3-D: ragged rows, one k-chunk
    ((9, 130, 260), 300),      # 3-D: 2 row tiles, 2 column tiles, 3 k-chunks
    ((3, 5, 7), 1),            # one mode
])
def test_structured_scalar(gsc, form, shape, n):
    cov, z1, z2, axes = _grid_case(sum(shape) + n, shape, n)
    ref = oracle.summator(cov, z1, z2, _flat(axes), num_threads=NT)
    out = gsc.summate_structured(cov, z1, z2, axes, form=form)
    assert out.shape == ref.shape
    err = rel_err(out, ref)
    _report(f"{form} {shape} x {n}", err)
    assert err <= BOUND[form]


@pytest.mark.parametrize("form", ["plain", "sep_f64", "sep_f16x5", "sep_f16x3"])
@pytest.mark.parametrize("shape,n", [((30, 70), 150), ((12, 40, 30), 200), ((5, 129, 100), 64)])
def test_structured_incompr(gsc, form, shape, n):
    cov, z1, z2, axes = _grid_case(3 * sum(shape) + n, shape, n)
    ref = oracle.summator_incompr(cov, z1, z2, _flat(axes), num_threads=NT)
    out = gsc.summate_incompr_structured(cov, z1, z2, axes, form=form)
    assert out.shape == ref.shape == (len(shape), int(np.prod(shape)))
    err = rel_err(out, ref)
    _report(f"incompr {form} {shape} x {n}", err)
    assert err <= BOUND[form]


def test_heavy_tailed_c2_like(gsc):
    """The exponential-covariance (Student-t) spectrum of the benchmark on a
    64^3 grid with 2000 modes: the tensor-core form stays within its bound."""
    cov, z1, z2, axes = _grid_case(2, (64, 64, 64), 2000, kscale=1 / 20, heavy=True)
    ref = oracle.summator(cov, z1, z2, _flat(axes), num_threads=NT)
    for form in ("sep_f64", "sep_f16x5", "sep_f16x3"):
        out = gsc.summate_structured(cov, z1, z2, axes, form=form)
        err = rel_err(out, ref)
        e_rms = float(np.sqrt(np.mean((out - ref) ** 2)) / rms(ref))
        _report(f"{form} c2-like 64^3 x 2000 (rms err {e_rms:.2e})", err)
        assert err <= BOUND[form]


def test_auto_respects_tolerance(gsc):
    cov, z1, z2, axes = _grid_case(4, (8, 16, 24), 50)
    ref = oracle.summator(cov, z1, z2, _flat(axes))
    tight = gsc.summate_structured(cov, z1, z2, axes, timing=True)
    assert rel_err(tight, ref) <= 1e-12            # default tolerance: FP64 forms only
    assert "sep_f64_dmma" in [k for k, _ in gsc.last_timings()]
    mid = gsc.summate_structured(cov, z1, z2, axes, tolerance=1e-6, timing=True)
    assert "sep_tc_f16x5" in [k for k, _ in gsc.last_timings()]
    assert rel_err(mid, ref) <= BOUND["sep_f16x5"]
    loose = gsc.summate_structured(cov, z1, z2, axes, tolerance=1e-5, timing=True)
    assert "sep_tc_f16x3" in [k for k, _ in gsc.last_timings()]
    assert rel_err(loose, ref) <= BOUND["sep_f16x3"]


def test_one_dimensional_structured(gsc):
    cov, z1, z2, axes = _grid_case(5, (1000,), 64)
    ref = oracle.summator(cov, z1, z2, _flat(axes))
    out = gsc.summate_structured(cov, z1, z2, axes, form="sep_f16x3")   # 1-D runs plain
    assert rel_err(out, ref) <= 1e-12


def test_offset_nonuniform_axes(gsc):
    """Axes need not be equidistant nor start at 0."""
    rng = np.random.default_rng(6)
    cov = rng.normal(0, 0.4, (3, 120))
    z1, z2 = rng.standard_normal(120), rng.standard_normal(120)
    axes = (np.sort(rng.uniform(-50, 50, 17)), np.sort(rng.uniform(100, 300, 33)),
            np.sort(rng.uniform(-9, 9, 11)))
    ref = oracle.summator(cov, z1, z2, _flat(axes), num_threads=NT)
    for form in ("sep_f16x5", "sep_f16x3"):
        out = gsc.summate_structured(cov, z1, z2, axes, form=form)
        assert rel_err(out, ref) <= BOUND[form]


def test_many_modes_x5(gsc):
    """N = 5000 modes takes the narrower leading grid (8-bit); still below 1e-6."""
    cov, z1, z2, axes = _grid_case(9, (6, 70, 90), 5000, kscale=0.5)
    ref = oracle.summator(cov, z1, z2, _flat(axes), num_threads=NT)
    out = gsc.summate_structured(cov, z1, z2, axes, form="sep_f16x5")
    err = rel_err(out, ref)
    _report("sep_f16x5 6x70x90 x 5000", err)
    assert err <= BOUND["sep_f16x5"]


def test_structured_device_api(gsc):
    torch = pytest.importorskip("torch")
    cov, z1, z2, axes = _grid_case(7, (16, 140, 33), 90)
    ref = oracle.summator(cov, z1, z2, _flat(axes), num_threads=NT)
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    out = torch.empty(int(np.prod([len(a) for a in axes])), dtype=torch.float64, device="cuda")
    st = torch.cuda.current_stream()
    gsc.summate_structured_device(d(cov), d(z1), d(z2), tuple(d(a) for a in axes), out,
                                  form="sep_f16x5", stream=st.cuda_stream)
    st.synchronize()
    gsc.device_status()
    assert rel_err(out.cpu().numpy(), ref) <= BOUND["sep_f16x5"]


def test_separable_rejected_for_unstructured(gsc):
    cov, z1, z2, axes = _grid_case(8, (4, 4), 10)
    with pytest.raises(ValueError, match="structured grid"):
        gsc.summate(cov, z1, z2, _flat(axes), form="sep_f16x3")


def _spectral_divergence(u, L):
    """max_k |k . u_hat(k)| / max_k |k| |u_hat(k)| of a periodic vector field
    u (d, n, n[, n]) on [0, L)^d."""
    d = u.shape[0]
    n = u.shape[1:]
    uh = [np.fft.fftn(u[i]) for i in range(d)]
    ks = np.meshgrid(*[2.0 * np.pi * np.fft.fftfreq(m, d=L / m) for m in n], indexing="ij")
    div = sum(ks[i] * uh[i] for i in range(d))
    kmag = np.sqrt(sum(k ** 2 for k in ks))
    umag = np.sqrt(sum(np.abs(x) ** 2 for x in uh))
    return float(np.max(np.abs(div)) / np.max(kmag * umag))


@pytest.mark.parametrize("form,bound", [("plain", 1e-12), ("sep_f64", 1e-12), ("sep_f16x5", 1e-6)])
@pytest.mark.parametrize("shape", [(32, 32, 32), (64, 48)])
def test_incompr_divergence_free_in_spectral_space(gsc, form, bound, shape):
    """Modes on the FFT grid of a periodic box: the field's Fourier
    coefficients satisfy k . u_hat(k) = 0 (the projector of src/field.rs:138-152
    removes the longitudinal part), to round-off of the form."""
    dim = len(shape)
    L = 8.0 * np.pi
    rng = np.random.default_rng(11 + dim)
    m = rng.integers(-min(shape) // 2 + 1, min(shape) // 2, (dim, 300))
    m = m[:, np.any(m != 0, axis=0)]
    cov = m * (2.0 * np.pi / L)
    n = cov.shape[1]
    z1, z2 = rng.standard_normal(n), rng.standard_normal(n)
    axes = tuple(np.arange(s) * (L / s) for s in shape)
    u = gsc.summate_incompr_structured(cov, z1, z2, axes, form=form)
    div = _spectral_divergence(u.reshape((dim,) + shape), L)
    print(f"divergence {form} {shape}: {div:.3e}")
    assert div <= bound
