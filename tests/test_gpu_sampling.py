"""On-device spectral sampling of cov_samples, z1, z2 (GPU tests).

The generator is Philox4x32-10 (Salmon et al., SC'11) on counters (mode,
realization, draw) with Box-Muller normals.  Checked here:
  * the values against a numpy restatement of the same generator and
    transform (Philox words bit for bit; normals to libm rounding, 1e-13);
  * the distributions: Gaussian spectrum k ~ N(0, 2/l^2), exponential
    spectrum k*l ~ Cauchy per component, z1, z2 ~ N(0, 1), by moments and
    Kolmogorov-Smirnov statistics;
  * determinism: values depend only on (seed, realization, mode), so batch
    and single calls, and different mode counts, agree on shared modes.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from philox_ref import normals_host


@pytest.mark.parametrize("spectrum", ["gaussian", "exponential"])
def test_values_match_the_host_restatement(gsc, spectrum):
    seed, realization, n, ell, dim = 0x0123456789ABCDEF, 7, 4099, 3.5, 3
    cov, z1, z2 = gsc.sample_modes(spectrum, dim, n, ell, seed, realization)
    nrm = normals_host(seed, realization, n)
    scale = np.sqrt(2.0) / ell if spectrum == "gaussian" else 1.0 / (np.abs(nrm[3]) * ell)
    exp_cov = np.array([nrm[d] * scale for d in range(dim)])
    assert np.allclose(cov, exp_cov, rtol=1e-13, atol=1e-13 * np.max(np.abs(exp_cov)))
    assert np.allclose(z1, nrm[4], rtol=1e-13, atol=1e-14)
    assert np.allclose(z2, nrm[5], rtol=1e-13, atol=1e-14)


def test_distributions(gsc):
    stats = pytest.importorskip("scipy.stats")
    n, ell = 200_000, 4.0
    cov, z1, z2 = gsc.sample_modes("gaussian", 3, n, ell, 2024, 0)
    sd = np.sqrt(2.0) / ell
    for d in range(3):
        assert abs(cov[d].mean()) < 5 * sd / np.sqrt(n)
        assert abs(cov[d].std() / sd - 1.0) < 0.01
        assert stats.kstest(cov[d] / sd, "norm").pvalue > 1e-3
    for z in (z1, z2):
        assert stats.kstest(z, "norm").pvalue > 1e-3
    assert abs(np.corrcoef(z1, z2)[0, 1]) < 5 / np.sqrt(n)
    cov, _, _ = gsc.sample_modes("exponential", 2, n, ell, 2024, 1)
    for d in range(2):
        assert stats.kstest(cov[d] * ell, "cauchy").pvalue > 1e-3
    # components of one mode share the Student-t divisor: |k| is heavier
    # tailed than any single component, and their signs are independent
    assert abs(np.mean(np.sign(cov[0]) * np.sign(cov[1]))) < 5 / np.sqrt(n)


def test_values_depend_only_on_seed_realization_mode(gsc):
    torch = pytest.importorskip("torch")
    a = gsc.sample_modes("exponential", 3, 1000, 2.0, 99, 5)
    b = gsc.sample_modes("exponential", 3, 1500, 2.0, 99, 5)
    assert np.array_equal(a[0], b[0][:, :1000]) and np.array_equal(a[1], b[1][:1000])
    c = gsc.sample_modes("exponential", 3, 1000, 2.0, 99, 6)
    assert not np.array_equal(a[1], c[1])
    d = gsc.sample_modes("exponential", 3, 1000, 2.0, 100, 5)
    assert not np.array_equal(a[1], d[1])
    # one batched launch over realizations 5 and 6 gives the same values
    items = []
    for r, (dim, n, spec) in zip((5, 6), ((3, 1000, "exponential"), (2, 777, "gaussian"))):
        items.append({"spectrum": spec, "len_scale": 2.0, "realization": r,
                      "cov": torch.empty((dim, n), dtype=torch.float64, device="cuda"),
                      "z1": torch.empty(n, dtype=torch.float64, device="cuda"),
                      "z2": torch.empty(n, dtype=torch.float64, device="cuda")})
    gsc.sample_modes_batch_device(items, 99)
    torch.cuda.synchronize()
    assert np.array_equal(items[0]["cov"].cpu().numpy(), a[0])
    assert np.array_equal(items[0]["z2"].cpu().numpy(), a[2])
    single = gsc.sample_modes("gaussian", 2, 777, 2.0, 99, 6)
    assert np.array_equal(items[1]["z1"].cpu().numpy(), single[1])


def test_sampled_ensemble_feeds_the_batch(gsc):
    """Sampled on the device and summed by a batch plan without leaving the
    GPU: the result equals the host path on the same draws (plain FP64)."""
    torch = pytest.importorskip("torch")
    import oracle
    rng = np.random.default_rng(3)
    items = []
    for r in range(4):
        dim, n, p = 2 + r % 2, 200 + 50 * r, 3000
        items.append({"spectrum": "gaussian" if r % 2 == 0 else "exponential",
                      "len_scale": 5.0, "realization": r,
                      "cov": torch.empty((dim, n), dtype=torch.float64, device="cuda"),
                      "z1": torch.empty(n, dtype=torch.float64, device="cuda"),
                      "z2": torch.empty(n, dtype=torch.float64, device="cuda"),
                      "pos": torch.from_numpy(rng.uniform(0, 100, (dim, p))).cuda(),
                      "out": torch.empty(p, dtype=torch.float64, device="cuda")})
    gsc.sample_modes_batch_device(items, 7)
    with gsc.Batch([{k: it[k] for k in ("cov", "z1", "z2", "pos", "out")} for it in items],
                   form="plain") as b:
        b.run()
    torch.cuda.synchronize()
    for it in items:
        ref = oracle.summator(it["cov"].cpu().numpy(), it["z1"].cpu().numpy(),
                              it["z2"].cpu().numpy(), it["pos"].cpu().numpy())
        got = it["out"].cpu().numpy()
        assert np.max(np.abs(got - ref)) <= 1e-12 * np.sqrt(np.mean(ref ** 2))


def test_rejects_bad_arguments(gsc):
    with pytest.raises(ValueError):
        gsc.sample_modes("matern", 2, 10, 1.0, 0)
    with pytest.raises(ValueError):
        gsc.sample_modes("gaussian", 4, 10, 1.0, 0)
    with pytest.raises(ValueError):
        gsc.sample_modes("gaussian", 2, 10, 0.0, 0)
