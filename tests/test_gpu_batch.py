"""Batched ensembles: one persistent launch over many realizations (GPU tests).

Each item of a batch computes what one call of the reference's summator,
summator_incompr or summator_fourier computes for it (src/field.rs:37-65,
:97-182, :219-249), so every output is checked against the oracle on the
same inputs, at the bar of its form (max |err| / field RMS): 1e-12 for the
FP64 form, 1e-6 for the mixed form.  Cases: items of every kind and
dimension with uneven point and mode counts (including no points and no
modes), split modes, the CUDA-graph replay after the inputs change in place,
deterministic repeats, the autotuner's report, fixed configurations, and
the host-array entry point.
"""
import os

import numpy as np
import pytest

import oracle
from conftest import rel_err

pytestmark = pytest.mark.gpu

NT = os.cpu_count() or 1
BOUND = {"plain": 1e-12, "mixed": 1e-6}


def _items(seed, specs):
    """specs: (kind, dim, n_modes, n_points) -> host item dicts."""
    rng = np.random.default_rng(seed)
    items = []
    for kind, dim, n, p in specs:
        ell = rng.uniform(2.0, 50.0)
        if kind == "fourier":
            cov = rng.integers(-20, 21, (dim, n)) * (2.0 * np.pi / 500.0)
        elif rng.random() < 0.5:
            cov = rng.normal(0.0, np.sqrt(2.0) / ell, (dim, n))
        else:
            cov = rng.standard_normal((dim, n)) / np.sqrt(rng.chisquare(1, n)) / ell
        it = {"kind": kind, "cov": np.ascontiguousarray(cov), "z1": rng.standard_normal(n),
              "z2": rng.standard_normal(n), "pos": rng.uniform(0.0, 500.0, (dim, p))}
        if kind == "fourier":
            it["spectrum_factor"] = rng.uniform(0.1, 1.0, n)
        items.append(it)
    return items


def _oracle(it):
    if it["kind"] == "incompr":
        return oracle.summator_incompr(it["cov"], it["z1"], it["z2"], it["pos"], num_threads=NT)
    if it["kind"] == "fourier":
        return oracle.summator_fourier(it["spectrum_factor"], it["cov"], it["z1"], it["z2"],
                                       it["pos"], num_threads=NT)
    return oracle.summator(it["cov"], it["z1"], it["z2"], it["pos"], num_threads=NT)


SPECS = [("scalar", 2, 300, 70000), ("scalar", 3, 2000, 5000), ("incompr", 3, 257, 12345),
         ("incompr", 2, 64, 1), ("fourier", 2, 500, 3000), ("scalar", 1, 37, 999),
         ("scalar", 3, 0, 100), ("scalar", 2, 10, 0), ("fourier", 3, 129, 4096),
         ("scalar", 3, 4096, 600), ("incompr", 3, 1500, 40000)]


def _device(torch, items):
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    dev = []
    for it in items:
        p = it["pos"].shape[1]
        dim = it["pos"].shape[0]
        x = {k: d(v) for k, v in it.items() if k != "kind"}
        x["kind"] = it["kind"]
        shape = (dim, p) if it["kind"] == "incompr" else (p,)
        x["out"] = torch.full(shape, float("nan"), dtype=torch.float64, device="cuda")
        dev.append(x)
    return dev


def _check(items, outs, form):
    for i, (it, out) in enumerate(zip(items, outs)):
        ref = _oracle(it)
        assert out.shape == ref.shape, i
        if ref.size == 0:
            continue
        if not np.any(ref):
            assert np.array_equal(out, ref), i
            continue
        err = rel_err(out, ref)
        assert err <= BOUND[form], f"item {i} {it['kind']} {it['pos'].shape} x {it['z1'].size}: {err:.3e}"


@pytest.mark.parametrize("form", ["plain", "mixed"])
def test_batch_matches_oracle_run_and_graph(gsc, form):
    torch = pytest.importorskip("torch")
    items = _items(1, SPECS)
    dev = _device(torch, items)
    with gsc.Batch(dev, form=form) as b:
        cfg = b.config
        assert cfg["form"] == form and cfg["units"] > 0 and cfg["blocks"] > 0
        b.run()
        torch.cuda.synchronize()
        first = [x["out"].cpu().numpy().copy() for x in dev]
        _check(items, first, form)
        # graph replay: same results, bit for bit (deterministic split order)
        for x in dev:
            x["out"].fill_(float("nan"))
        b.run_graph()
        b.run_graph()
        torch.cuda.synchronize()
        for a, x in zip(first, dev):
            assert np.array_equal(a, x["out"].cpu().numpy())
        # new data in the same arrays: the replayed graph sees it
        items2 = _items(2, SPECS)
        for x, it in zip(dev, items2):
            for k in ("cov", "z1", "z2", "pos", "spectrum_factor"):
                if k in it:
                    x[k].copy_(torch.from_numpy(np.ascontiguousarray(it[k])))
        b.run_graph()
        torch.cuda.synchronize()
        _check(items2, [x["out"].cpu().numpy() for x in dev], form)


def test_batch_split_modes(gsc):
    """Few points and many modes with a fine unit target: modes are split
    over units and reduced in split order."""
    torch = pytest.importorskip("torch")
    items = _items(3, [("scalar", 3, 6000, 700), ("incompr", 2, 3000, 300), ("scalar", 2, 50, 50)])
    dev = _device(torch, items)
    with gsc.Batch(dev, form="plain", points_per_thread=4, tile_modes=8,
                   units_per_block=64) as b:
        assert b.config["max_splits"] > 1 and not b.config["tuned"]
        b.run()
        torch.cuda.synchronize()
        _check(items, [x["out"].cpu().numpy() for x in dev], "plain")


@pytest.mark.parametrize("R,tile", [(2, 8), (4, 16), (8, 8)])
def test_batch_fixed_configs(gsc, R, tile):
    torch = pytest.importorskip("torch")
    items = _items(4, SPECS[:5])
    dev = _device(torch, items)
    with gsc.Batch(dev, form="plain", points_per_thread=R, tile_modes=tile,
                   units_per_block=4) as b:
        c = b.config
        assert (c["points_per_thread"], c["tile_modes"]) == (R, tile)
        b.run()
        torch.cuda.synchronize()
        _check(items, [x["out"].cpu().numpy() for x in dev], "plain")


def test_batch_rejects_bad_input(gsc):
    torch = pytest.importorskip("torch")
    items = _items(5, [("scalar", 2, 10, 10)])
    dev = _device(torch, items)
    with pytest.raises(ValueError):
        gsc.Batch(dev, form="plain", points_per_thread=3, tile_modes=8, units_per_block=4)
    with pytest.raises(ValueError):
        gsc.Batch(dev, form="sep_f16x5")
    bad = _device(torch, _items(6, [("incompr", 2, 10, 10)]))
    bad[0]["kind"] = "nope"
    with pytest.raises(ValueError):
        gsc.Batch(bad)


def test_summate_batch_host_api(gsc):
    items = _items(7, SPECS)
    host = [{k: v for k, v in it.items()} for it in items]
    outs = gsc.summate_batch(host, form="mixed", tolerance=1e-6)
    _check(items, outs, "mixed")
    cfg = gsc.last_batch_config()
    assert cfg["form"] == "mixed"
    # the same shapes again reuse the plan; plain FP64 bar on a second ensemble
    outs = gsc.summate_batch(_items(8, SPECS), form="plain")
    _check(_items(8, SPECS), outs, "plain")


def test_batch_mixed_both_product_forms(gsc):
    """Items whose wave numbers times extent keep every |BI| < 2^20 (FP32
    product of BI Xl 2^-29) beside items beyond it (integer high products),
    in one persistent launch."""
    rng = np.random.default_rng(31)
    items = []
    for span in (500.0, 3.0e6, 800.0, 2.0e6):
        n, p = int(rng.integers(200, 700)), int(rng.integers(500, 3000))
        cov = rng.standard_normal((3, n)) / np.sqrt(rng.chisquare(1, n)) * 0.2
        items.append({"kind": "scalar", "cov": cov, "z1": rng.standard_normal(n),
                      "z2": rng.standard_normal(n), "pos": rng.uniform(0.0, span, (3, p))})
    outs = gsc.summate_batch(items, form="mixed")
    _check(items, outs, "mixed")


def test_summate_batch_host_api_groups(gsc):
    """An ensemble of at least 4e9 point*modes and 8 items runs as four
    groups whose copies overlap the computing of their neighbours.  Every
    item against the oracle on a seeded subset of its points, on two calls
    (the second reuses the plans with new values), and the reported totals
    cover all groups."""
    rng = np.random.default_rng(41)
    items = []
    for i in range(16):
        dim = 2 + i % 2
        n, p = int(rng.integers(2000, 3000)), int(rng.integers(150_000, 250_000))
        cov = rng.standard_normal((dim, n)) / np.sqrt(rng.chisquare(1, n)) / 10.0
        items.append({"kind": "scalar", "cov": cov, "z1": rng.standard_normal(n),
                      "z2": rng.standard_normal(n), "pos": rng.uniform(0.0, 500.0, (dim, p))})
    work = sum(it["pos"].shape[1] * it["z1"].size for it in items)
    assert work >= 4e9
    for call in range(2):
        if call:
            for it in items:
                it["z1"][:] = rng.standard_normal(it["z1"].size)
        outs = gsc.summate_batch(items, form="mixed", timing=call == 1)
        for i, (it, out) in enumerate(zip(items, outs)):
            idx = np.sort(rng.choice(it["pos"].shape[1], 512, replace=False))
            ref = oracle.summator(it["cov"], it["z1"], it["z2"],
                                  np.ascontiguousarray(it["pos"][:, idx]), num_threads=NT)
            err = rel_err(out[idx], ref)
            assert err <= BOUND["mixed"], f"call {call} item {i}: {err:.3e}"
    # the timed call's records on one clock: four groups, each copied in,
    # computed and copied out in that order
    tl = gsc.last_timeline()
    assert [(k, ms) for k, _, ms in tl] == gsc.last_timings()
    assert tl[0][1] == 0.0 and all(s >= 0 and ms >= 0 for _, s, ms in tl)
    h2d = [s for k, s, _ in tl if k == "copy_h2d"]
    sums = [(s, s + ms) for k, s, ms in tl if k == "batch_mixed"]
    d2h = [s + ms for k, s, ms in tl if k == "copy_d2h"]
    assert len(h2d) == len(sums) == len(d2h) == 4
    assert all(a <= b for a, (b, _) in zip(h2d, sums))
    assert all(e <= f + 1e-3 for (_, e), f in zip(sums, d2h))
    cfg = gsc.last_batch_config()
    assert cfg["form"] == "mixed" and cfg["work"] == work


def test_summate_batch_phase_range(gsc):
    """An item whose wave number times extent passes 2^30 turns does not fit
    the mixed form's integer phase.  The host-array call under AUTO at
    tolerance 1e-6 recomputes the ensemble on the plain FP64 form (the FP64
    bar holds for every item); an explicit mixed form reports it; neither
    leaves a device status behind."""
    rng = np.random.default_rng(44)
    items = []
    for k in range(3):
        n, p = 40, 2000
        cov = rng.normal(0.0, 0.5, (3, n))
        span = 100.0
        if k == 1:
            cov[0, 5] = 40.0
            span = 2.0e8                     # 40 x 2e8 / 2 pi > 2^30 turns
        items.append({"kind": "scalar", "cov": cov, "z1": rng.standard_normal(n),
                      "z2": rng.standard_normal(n), "pos": rng.uniform(0.0, span, (3, p))})
    cfg = dict(points_per_thread=4, tile_modes=8, units_per_block=16)
    outs = gsc.summate_batch(items, tolerance=1e-6, **cfg)
    _check(items, outs, "plain")
    with pytest.raises(gsc.GscError, match="2\\^30 turns"):
        gsc.summate_batch(items, form="mixed", **cfg)
    gsc.device_status()


def test_summate_batch_eight_groups_with_empty_items(gsc):
    """From 4e10 point*modes and 16 items the host-array call runs in eight
    groups (the first and the last 1/32 of the work each).  Items without points or without
    modes among them; every item against the oracle on a seeded subset."""
    rng = np.random.default_rng(45)
    items = []
    for i in range(20):
        dim = 2 + i % 2
        n, p = 4000 + 7 * i, 600_000 + 1000 * i
        if i == 3:
            p = 0
        if i == 11:
            n = 0
        cov = rng.standard_normal((dim, n)) / np.sqrt(rng.chisquare(1, n)) / 10.0
        items.append({"kind": "scalar", "cov": cov, "z1": rng.standard_normal(n),
                      "z2": rng.standard_normal(n), "pos": rng.uniform(0.0, 500.0, (dim, p))})
    work = sum(it["pos"].shape[1] * it["z1"].size for it in items)
    assert work >= 4e10
    outs = gsc.summate_batch(items, form="mixed")
    for i, (it, out) in enumerate(zip(items, outs)):
        p = it["pos"].shape[1]
        assert out.shape == (p,)
        if p == 0:
            continue
        if it["z1"].size == 0:
            assert np.all(out == 0.0)
            continue
        idx = np.sort(rng.choice(p, 256, replace=False))
        ref = oracle.summator(it["cov"], it["z1"], it["z2"],
                              np.ascontiguousarray(it["pos"][:, idx]), num_threads=NT)
        err = rel_err(out[idx], ref)
        assert err <= BOUND["mixed"], f"item {i}: {err:.3e}"
