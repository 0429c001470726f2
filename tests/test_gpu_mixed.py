"""Mixed-precision forms on explicit points against the oracle (GPU tests).

`mixed`: phase as a 32-bit fixed-point integer (units of 2^-32 turn), FP32
table and polynomial sincos, FP32 pair and tile sums with a compensated
total.  `mixed_f64phase`: phase and reduction in FP64.  Bar for both: max |err| <= 1e-6 x RMS of the oracle field
(reference src/field.rs:37-65, :97-182), including the heavy-tailed spectrum
of the unstructured 3-D benchmark where |k.x| reaches 1e5.
"""
import os

import numpy as np
import pytest

import oracle
from conftest import rel_err, rms

pytestmark = pytest.mark.gpu
NT = os.cpu_count() or 1
TOL = 1e-6


def _case(seed, dim, n, p, kscale=0.5, span=50.0, heavy=False):
    rng = np.random.default_rng(seed)
    if heavy:
        cov = rng.standard_normal((dim, n)) / np.sqrt(rng.chisquare(1, n)) * kscale
    else:
        cov = rng.normal(0, kscale, (dim, n))
    z1, z2 = rng.standard_normal(n), rng.standard_normal(n)
    pos = rng.uniform(0, span, (dim, p))
    return cov, z1, z2, pos


@pytest.mark.parametrize("form", ["mixed", "mixed_f64phase"])
@pytest.mark.parametrize("dim,n,p", [(1, 300, 5000), (2, 1000, 20000), (3, 64, 1 << 16),
                                     (3, 1, 100), (2, 7, 33), (3, 2000, 4000)])
def test_mixed_scalar(gsc, form, dim, n, p):
    cov, z1, z2, pos = _case(dim * 100 + n, dim, n, p)
    ref = oracle.summator(cov, z1, z2, pos, num_threads=NT)
    out = gsc.summate(cov, z1, z2, pos, form=form)
    err = rel_err(out, ref)
    print(f"{form} d={dim} N={n} P={p}: {err:.3e}")
    assert err <= TOL


@pytest.mark.parametrize("form", ["mixed", "mixed_f64phase"])
@pytest.mark.parametrize("dim", [2, 3])
def test_mixed_incompr(gsc, form, dim):
    cov, z1, z2, pos = _case(7 + dim, dim, 500, 8000)
    ref = oracle.summator_incompr(cov, z1, z2, pos, num_threads=NT)
    out = gsc.summate_incompr(cov, z1, z2, pos, form=form)
    assert out.shape == ref.shape and out.flags.f_contiguous
    err = rel_err(out, ref)
    print(f"incompr {form} d={dim}: {err:.3e}")
    assert err <= TOL


def test_mixed_heavy_tailed_unstructured(gsc):
    """The unstructured 3-D benchmark's spectrum (Student-t, l = 5) on
    [0, 1000]^3 with 4096 modes: |k.x| reaches 1e5."""
    cov, z1, z2, pos = _case(3, 3, 4096, 1 << 15, kscale=0.2, span=1000.0, heavy=True)
    assert np.max(np.abs(cov.T @ pos[:, :256])) > 1e4
    ref = oracle.summator(cov, z1, z2, pos, num_threads=NT)
    for form in ("mixed", "mixed_f64phase"):
        out = gsc.summate(cov, z1, z2, pos, form=form)
        err = rel_err(out, ref)
        e_rms = float(np.sqrt(np.mean((out - ref) ** 2)) / rms(ref))
        print(f"{form} heavy 3-D 4096 modes: max {err:.3e} rms {e_rms:.3e}")
        assert err <= TOL


def _max_bi(cov, pos):
    """Largest |BI| of the call, the integer part of kappa 2^(61 - s) with
    2^s the positions' fixed-point scale (max |x| in [2^(e-1), 2^e): s = 60 - e)."""
    e = np.frexp(np.abs(pos).max(axis=1))[1]
    return float(np.max(np.abs(cov) / (2.0 * np.pi) * np.ldexp(1.0, e + 1)[:, None]))


@pytest.mark.parametrize("incompr", [False, True])
def test_mixed_both_product_forms(gsc, incompr):
    """While every |BI| < 2^20 (about 2^19 turns across the domain), the
    kernel forms BI Xl 2^-29 with an FP32 product; a wider call takes integer
    high products.  One heavy-tailed call of each, against the oracle."""
    for span, small in ((1000.0, True), (2.0e6, False)):
        cov, z1, z2, pos = _case(21, 3, 512, 4096, kscale=0.2, span=span, heavy=True)
        assert (_max_bi(cov, pos) < 2.0 ** 20) == small
        if incompr:
            ref = oracle.summator_incompr(cov, z1, z2, pos, num_threads=NT)
            out = gsc.summate_incompr(cov, z1, z2, pos, form="mixed")
        else:
            ref = oracle.summator(cov, z1, z2, pos, num_threads=NT)
            out = gsc.summate(cov, z1, z2, pos, form="mixed")
        err = rel_err(out, ref)
        print(f"span {span:g} (max |BI| {_max_bi(cov, pos):.3g}): {err:.3e}")
        assert err <= TOL


def test_mixed_many_modes_chunks_and_splits(gsc):
    cov, z1, z2, pos = _case(4, 2, 9000, 700)     # few points: modes split across CTAs
    ref = oracle.summator(cov, z1, z2, pos, num_threads=NT)
    assert rel_err(gsc.summate(cov, z1, z2, pos, form="mixed"), ref) <= TOL


def test_auto_picks_mixed_within_tolerance(gsc):
    cov, z1, z2, pos = _case(5, 3, 100, 3000)
    ref = oracle.summator(cov, z1, z2, pos, num_threads=NT)
    out = gsc.summate(cov, z1, z2, pos, tolerance=1e-6, timing=True)
    assert "mixed_scalar" in [k for k, _ in gsc.last_timings()]
    assert rel_err(out, ref) <= TOL
    out = gsc.summate(cov, z1, z2, pos, timing=True)             # default: FP64
    assert "plain_f64_scalar" in [k for k, _ in gsc.last_timings()]
    assert rel_err(out, ref) <= 1e-12


def test_mixed_on_structured_grid(gsc):
    rng = np.random.default_rng(6)
    cov = rng.normal(0, 0.3, (3, 300))
    z1, z2 = rng.standard_normal(300), rng.standard_normal(300)
    axes = tuple(np.arange(s, dtype=np.float64) for s in (10, 20, 30))
    pos = np.array(np.meshgrid(*axes, indexing="ij")).reshape(3, -1)
    ref = oracle.summator(cov, z1, z2, pos, num_threads=NT)
    assert rel_err(gsc.summate_structured(cov, z1, z2, axes, form="mixed"), ref) <= TOL


@pytest.mark.parametrize("kind", ["scalar", "incompr"])
def test_mixed_phase_range_falls_back(gsc, kind):
    """A wave number whose phase across the domain passes 2^30 turns does
    not fit the integer phase.  AUTO at tolerance 1e-6 (the mixed form)
    recomputes such a call on the plain FP64 kernel, so the FP64 bar holds;
    an explicit mixed form reports the error, and the next call computes.
    Scalar (C-ordered result) and incompressible (Fortran-ordered result)."""
    rng = np.random.default_rng(8)
    n, p = 50, 3000
    cov = rng.normal(0.0, 0.5, (3, n))
    cov[0, 7] = 40.0                          # 40 x 2e8 / 2 pi = 1.3e9 turns > 2^30
    z1, z2 = rng.standard_normal(n), rng.standard_normal(n)
    pos = rng.uniform(0.0, 2.0e8, (3, p))
    fn = gsc.summate_incompr if kind == "incompr" else gsc.summate
    ofn = oracle.summator_incompr if kind == "incompr" else oracle.summator
    ref = ofn(cov, z1, z2, pos, num_threads=NT)
    out = fn(cov, z1, z2, pos, tolerance=1e-6)
    err = rel_err(out, ref)
    print(f"range fallback ({kind}): {err:.3e}")
    assert err <= 1e-12
    with pytest.raises(gsc.GscError, match="2\\^30 turns"):
        fn(cov, z1, z2, pos, form="mixed")
    ok = rel_err(fn(cov[:, :7], z1[:7], z2[:7], pos, form="mixed"),
                 ofn(cov[:, :7], z1[:7], z2[:7], pos, num_threads=NT))
    assert ok <= TOL


@pytest.mark.parametrize("kind", ["scalar", "incompr"])
def test_device_auto_falls_back_on_the_device(gsc, kind):
    """Device arrays under AUTO at tolerance 1e-6: the mixed form, with the
    plain FP64 kernels queued behind it and predicated on its range word.
    In range, the predicated launches leave the mixed result as it is (bit
    for bit the explicit mixed form's); past the range (2^30 turns), they
    recompute it at the FP64 bar and no status is left; an explicit mixed
    form past the range leaves the sticky status."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(12)
    n, p = 64, 5000
    cov = rng.normal(0.0, 0.5, (3, n))
    z1, z2 = rng.standard_normal(n), rng.standard_normal(n)
    pos = rng.uniform(0.0, 100.0, (3, p))
    fn = gsc.summate_incompr_device if kind == "incompr" else gsc.summate_device
    ofn = oracle.summator_incompr if kind == "incompr" else oracle.summator
    shape = (3, p) if kind == "incompr" else (p,)

    def run(c, ps, **kw):
        dev = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (c, z1, z2, ps)]
        out = torch.full(shape, float("nan"), dtype=torch.float64, device="cuda")
        fn(*dev, out, **kw)
        torch.cuda.synchronize()
        return out.cpu().numpy()

    auto = run(cov, pos, tolerance=1e-6)
    mixed = run(cov, pos, form="mixed")
    assert np.array_equal(auto, mixed)
    assert rel_err(auto, ofn(cov, z1, z2, pos, num_threads=NT)) <= TOL
    gsc.device_status()                                  # nothing reported
    far = pos * 2.0e6                                    # [0, 2e8]
    big = cov.copy()
    big[0, 3] = 40.0                                     # 40 x 2e8 / 2 pi > 2^30 turns
    got = run(big, far, tolerance=1e-6)
    gsc.device_status()                                  # handled on the device
    assert rel_err(got, ofn(big, z1, z2, far, num_threads=NT)) <= 1e-12
    run(big, far, form="mixed")
    with pytest.raises(gsc.GscError):
        gsc.device_status()


def test_issue_rate_probe_is_ordered_and_repeatable(gsc):
    """gsc_selftest_pipe_rates measures the issue rates the mixed form's
    roofline weighs its instructions with: FP32 FMAs issue faster than low
    32-bit integer multiply-adds, and those faster than high ones; two
    measurements agree within 10 %."""
    import ctypes
    from gstools_core import _native
    runs = []
    for _ in range(2):
        r = (ctypes.c_double * 3)()
        _native.check(_native.lib.gsc_selftest_pipe_rates(-1, r))
        runs.append(np.array(r[:]))
    for hi, lo, ffma in runs:
        assert 0 < hi < lo < ffma
        assert 1.2 < ffma / lo < 3.0 and 2.0 < ffma / hi < 6.0
    assert np.all(np.abs(runs[0] / runs[1] - 1.0) < 0.10)


@pytest.mark.parametrize("in_range", [True, False])
def test_mixed_padded_output_and_range(gsc, in_range):
    """A result buffer neither C- nor Fortran-ordered (a padded (P, 4) array
    through the C ABI) at tolerance 1e-6: in range the mixed form's result,
    past the phase range the plain FP64 recomputation; the padding stays
    untouched."""
    import ctypes
    from gstools_core import _native
    rng = np.random.default_rng(12)
    n, p = 40, 5000
    cov = rng.normal(0.0, 0.5, (3, n))
    if not in_range:
        cov[1, 5] = 40.0                      # 40 x 2e8 / 2 pi > 2^30 turns
    z1, z2 = rng.standard_normal(n), rng.standard_normal(n)
    pos = rng.uniform(0.0, 2.0e8, (3, p))
    buf = np.full((p, 4), np.nan)
    o = gsc._opts("auto", 1e-6, False, -1)
    rc = _native.lib.gsc_summate_incompr_f64(
        cov.ctypes.data, n, 1, z1.ctypes.data, 1, z2.ctypes.data, 1,
        pos.ctypes.data, p, 1, 3, n, p, buf.ctypes.data, 1, 4, ctypes.byref(o))
    assert rc == 0, _native.lib.gsc_last_error()
    assert np.isnan(buf[:, 3]).all()
    ref = oracle.summator_incompr(cov, z1, z2, pos, num_threads=NT)
    assert rel_err(buf[:, :3].T, ref) <= (TOL if in_range else 1e-12)


@pytest.mark.parametrize("case", ["subnormal", "zero", "tiny", "huge"])
def test_mixed_extreme_coordinate_magnitudes(gsc, case):
    """The fixed-point scale comes from the exponent of the largest |x|: a
    subnormal largest coordinate (frexp), all coordinates zero (no finite
    nonzero value), and magnitudes near the ends of the FP64 range with wave
    numbers scaled the other way (phases of order one, the scaling outside
    the range of a normal power of two).  Against the oracle at 1e-6."""
    rng = np.random.default_rng(21)
    n, p = 64, 4000
    cov = rng.normal(0.0, 1.0, (3, n))
    z1, z2 = rng.standard_normal(n), rng.standard_normal(n)
    pos = rng.uniform(-1.0, 1.0, (3, p))
    if case == "subnormal":
        pos *= 1e-310
    elif case == "zero":
        pos[:] = 0.0
    elif case == "tiny":
        pos *= 1e-300
        cov *= 1e300
    else:
        pos *= 1e300
        cov *= 1e-300
    ref = oracle.summator(cov, z1, z2, pos, num_threads=NT)
    got = gsc.summate(cov, z1, z2, pos, form="mixed")
    assert rel_err(got, ref) <= TOL
    if case != "huge":             # |k|^2 underflows there: the reference's projector is NaN
        gi = gsc.summate_incompr(cov, z1, z2, pos, form="mixed")
        assert rel_err(gi, oracle.summator_incompr(cov, z1, z2, pos, num_threads=NT)) <= TOL


@pytest.mark.parametrize("kind", ["scalar", "incompr"])
def test_range_fallback_into_a_pinned_result(gsc, kind):
    """A result of 64 KiB and more comes from the pinned pool, and the
    kernels write it in place; past the phase range AUTO recomputes it on
    the plain FP64 kernel over the mixed form's invalid values.  C-ordered
    (scalar) and Fortran-ordered (incompressible) results."""
    rng = np.random.default_rng(31)
    n, p = 40, 20_000                                  # 160 KB per component
    cov = rng.normal(0.0, 0.5, (3, n))
    cov[2, 9] = 40.0                                   # 40 x 2e8 / 2 pi > 2^30 turns
    z1, z2 = rng.standard_normal(n), rng.standard_normal(n)
    pos = rng.uniform(0.0, 2.0e8, (3, p))
    fn = gsc.summate_incompr if kind == "incompr" else gsc.summate
    ofn = oracle.summator_incompr if kind == "incompr" else oracle.summator
    out = fn(cov, z1, z2, pos, tolerance=1e-6)
    assert rel_err(out, ofn(cov, z1, z2, pos, num_threads=NT)) <= 1e-12
    ok = fn(cov[:, :9], z1[:9], z2[:9], pos, tolerance=1e-6)
    assert rel_err(ok, ofn(cov[:, :9], z1[:9], z2[:9], pos, num_threads=NT)) <= TOL
