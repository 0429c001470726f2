"""Plain FP64 GPU summators against the oracle (GPU tests).

Bar: max |gpu - oracle| <= 1e-12 * RMS(oracle field) for both FP64 forms
(table-driven sincos and CUDA's sincos), on the reference's own known answers
(src/field.rs:359-430), seeded random cases for d = 1, 2, 3, heavy-tailed
spectra, and the edge cases the reference handles (no modes, one mode, empty
and odd point counts, strided / Fortran-ordered views, NaN inputs, any
dimension for the scalar field).
"""
import os

import numpy as np
import pytest

import oracle
from conftest import rel_err, ulps_eq

pytestmark = pytest.mark.gpu

TOL_PLAIN = 1e-12
FORMS = ["plain", "plain_libm"]
NT = os.cpu_count() or 1


def _case(seed, dim, n, p, kscale=0.5, xspan=50.0, heavy=False):
    rng = np.random.default_rng(seed)
    if heavy:   # multivariate Student-t, nu = 1 (exponential covariance spectrum)
        cov = rng.standard_normal((dim, n)) / np.sqrt(rng.chisquare(1, n)) * kscale
    else:
        cov = rng.normal(0.0, kscale, (dim, n))
    z1, z2 = rng.standard_normal(n), rng.standard_normal(n)
    pos = rng.uniform(-xspan, xspan, (dim, p))
    return cov, z1, z2, pos


@pytest.mark.parametrize("form", FORMS)
def test_golden_summate(gsc, goldens, form):
    g = goldens
    out = gsc.summate(g["setup.cov_samples"], g["setup.z_1"], g["setup.z_2"], g["setup.pos"],
                      form=form)
    exp = g["expected.summate"]
    assert rel_err(out, exp) <= 1e-14
    assert all(ulps_eq(a, b, max_ulps=64) for a, b in zip(out, exp))


@pytest.mark.parametrize("form", FORMS)
def test_golden_incompr(gsc, goldens, form):
    g = goldens
    out = gsc.summate_incompr(g["setup.cov_samples"], g["setup.z_1"], g["setup.z_2"],
                              g["setup.pos"], form=form)
    exp = g["expected.summate_incompr"]
    assert out.shape == (3, 8) and out.flags.f_contiguous
    assert rel_err(out, exp) <= 1e-14


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("dim,n,p", [
    (1, 1, 1), (1, 37, 1000), (2, 7, 33), (2, 1000, 5000), (3, 9, 513), (3, 100, 1000),
    (3, 64, 1 << 17), (2, 8, 512), (3, 1, 10007),
])
def test_summate_random(gsc, form, dim, n, p):
    cov, z1, z2, pos = _case(100 * dim + n, dim, n, p)
    ref = oracle.summator(cov, z1, z2, pos, num_threads=NT)
    out = gsc.summate(cov, z1, z2, pos, form=form)
    assert rel_err(out, ref) <= TOL_PLAIN


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("dim,n,p", [(2, 10, 8), (2, 500, 3001), (3, 7, 129), (3, 300, 2000),
                                     (3, 32, 1 << 16)])
def test_incompr_random(gsc, form, dim, n, p):
    cov, z1, z2, pos = _case(7 * dim + n, dim, n, p)
    ref = oracle.summator_incompr(cov, z1, z2, pos, num_threads=NT)
    out = gsc.summate_incompr(cov, z1, z2, pos, form=form)
    assert out.shape == (dim, p) and out.flags.f_contiguous
    assert rel_err(out, ref) <= TOL_PLAIN


@pytest.mark.parametrize("form", FORMS)
def test_heavy_tailed_large_phases(gsc, form):
    """Student-t spectrum on [0, 1000]^3: |k.x| reaches 1e4..1e6."""
    cov, z1, z2, pos = _case(5, 3, 512, 4096, kscale=0.2, xspan=1000.0, heavy=True)
    assert np.max(np.abs(cov.T @ pos)) > 1e4
    ref = oracle.summator(cov, z1, z2, pos, num_threads=NT)
    assert rel_err(gsc.summate(cov, z1, z2, pos, form=form), ref) <= TOL_PLAIN
    refi = oracle.summator_incompr(cov, z1, z2, pos, num_threads=NT)
    assert rel_err(gsc.summate_incompr(cov, z1, z2, pos, form=form), refi) <= TOL_PLAIN


def test_extreme_phases_take_the_exact_path(gsc):
    """|k.x| > 1e13 is outside the table reduction's range; results must still
    match glibc's cos/sin of the same FP64 phase."""
    cov, z1, z2, pos = _case(6, 2, 40, 300)
    cov[:, :5] *= 1e12
    pos *= 100.0
    ref = oracle.summator(cov, z1, z2, pos, num_threads=NT)
    assert rel_err(gsc.summate(cov, z1, z2, pos), ref) <= TOL_PLAIN


def test_many_modes_chunked(gsc):
    """More modes than one table chunk (16384) with few points (mode split)."""
    cov, z1, z2, pos = _case(8, 3, 16384 + 777, 300)
    ref = oracle.summator(cov, z1, z2, pos, num_threads=NT)
    assert rel_err(gsc.summate(cov, z1, z2, pos), ref) <= TOL_PLAIN
    refi = oracle.summator_incompr(cov, z1, z2, pos, num_threads=NT)
    assert rel_err(gsc.summate_incompr(cov, z1, z2, pos), refi) <= TOL_PLAIN


def test_no_modes_gives_zeros(gsc):
    z = np.zeros(0)
    assert np.array_equal(gsc.summate(np.zeros((3, 0)), z, z, np.ones((3, 5))), np.zeros(5))
    assert np.array_equal(gsc.summate_incompr(np.zeros((2, 0)), z, z, np.ones((2, 5))),
                          np.zeros((2, 5)))


@pytest.mark.parametrize("dim", [0, 4, 6])
def test_other_dimensions_scalar(gsc, dim):
    cov, z1, z2, pos = _case(9, max(dim, 1), 50, 200)
    cov, pos = cov[:dim], pos[:dim]
    ref = oracle.summator(cov, z1, z2, pos)
    assert rel_err(gsc.summate(cov, z1, z2, pos), ref) <= TOL_PLAIN


def test_strided_and_fortran_views(gsc):
    cov, z1, z2, pos = _case(11, 3, 200, 3000)
    ref = oracle.summator(cov, z1, z2, pos, num_threads=NT)
    out1 = gsc.summate(np.asfortranarray(cov), z1, z2, np.asfortranarray(pos))
    big = np.zeros((3, 6000))
    big[:, 1::2] = pos
    zz = np.zeros(400)
    zz[::2] = z2
    out2 = gsc.summate(cov, z1, zz[::2], big[:, 1::2])
    assert rel_err(out1, ref) <= TOL_PLAIN and rel_err(out2, ref) <= TOL_PLAIN
    refi = oracle.summator_incompr(cov, z1, z2, pos, num_threads=NT)
    outi = gsc.summate_incompr(cov[:, ::-1][:, ::-1], z1, z2, np.asfortranarray(pos))
    assert rel_err(outi, refi) <= TOL_PLAIN


def test_nan_stays_local(gsc):
    cov, z1, z2, pos = _case(12, 2, 30, 1000)
    pos[0, 17] = np.nan
    out = gsc.summate(cov, z1, z2, pos)
    assert np.isnan(out[17]) and np.isfinite(np.delete(out, 17)).all()
    ref = oracle.summator(cov, z1, z2, pos)
    mask = np.isfinite(ref)
    assert rel_err(out[mask], ref[mask]) <= TOL_PLAIN


def test_device_api_and_timings(gsc):
    torch = pytest.importorskip("torch")
    cov, z1, z2, pos = _case(13, 3, 256, 20000)
    ref = oracle.summator(cov, z1, z2, pos, num_threads=NT)
    dev = [torch.from_numpy(a).cuda() for a in (cov, z1, z2, pos)]
    out = torch.empty(pos.shape[1], dtype=torch.float64, device="cuda")
    st = torch.cuda.current_stream()
    gsc.summate_device(*dev, out, stream=st.cuda_stream, timing=True)
    st.synchronize()
    assert rel_err(out.cpu().numpy(), ref) <= TOL_PLAIN
    names = [n for n, ms in gsc.last_timings()]
    assert "plain_f64_scalar" in names and all(ms >= 0 for _, ms in gsc.last_timings())
    outi = torch.empty((3, pos.shape[1]), dtype=torch.float64, device="cuda")
    gsc.summate_incompr_device(*dev, outi, stream=st.cuda_stream)
    st.synchronize()
    refi = oracle.summator_incompr(cov, z1, z2, pos, num_threads=NT)
    assert rel_err(outi.cpu().numpy(), refi) <= TOL_PLAIN


def test_device_api_rejects_host_memory(gsc):
    torch = pytest.importorskip("torch")
    cov, z1, z2, pos = _case(14, 2, 16, 64)
    dev = [torch.from_numpy(a).cuda() for a in (cov, z1, z2)]
    out = torch.empty(64, dtype=torch.float64, device="cuda")

    class HostView:   # a host pointer dressed up as a CUDA array
        def __init__(self, a):
            self.a = a
            self.__cuda_array_interface__ = {"shape": a.shape, "typestr": "<f8",
                                             "data": (a.ctypes.data, False), "version": 2}
    with pytest.raises(ValueError, match="not device-accessible|not a CUDA pointer"):
        gsc.summate_device(*dev, HostView(pos), out)


def test_repeated_calls_and_buffer_growth(gsc):
    """Host-path buffers grow across calls of increasing size; results stay exact."""
    for p in (10, 100000, 50):
        cov, z1, z2, pos = _case(15 + p, 3, 64, p)
        ref = oracle.summator(cov, z1, z2, pos, num_threads=NT)
        assert rel_err(gsc.summate(cov, z1, z2, pos), ref) <= TOL_PLAIN
