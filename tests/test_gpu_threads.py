"""Concurrent host-array calls from several Python threads (GPU test).

The C ABI is documented thread safe: host-pointer calls on one device are
serialised on the device context, and the Python layer releases the GIL
inside every foreign call (ctypes).  Four threads run mixed forms (plain,
mixed, structured tensor-core, batch) on their own inputs at once; every
result must equal what the same call gives alone, bit for bit.
"""
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _inputs(seed):
    rng = np.random.default_rng(seed)
    cov = rng.normal(0.0, 0.3, (3, 200))
    z1, z2 = rng.standard_normal(200), rng.standard_normal(200)
    pos = rng.uniform(-20.0, 20.0, (3, 40000))
    axes = tuple(np.arange(s, dtype=np.float64) for s in (8, 64, 96))
    return cov, z1, z2, pos, axes


def _work(gsc, seed):
    cov, z1, z2, pos, axes = _inputs(seed)
    kind = seed % 4
    if kind == 0:
        return gsc.summate(cov, z1, z2, pos, form="plain")
    if kind == 1:
        return gsc.summate_incompr(cov, z1, z2, pos, form="mixed")
    if kind == 2:
        return gsc.summate_structured(cov, z1, z2, axes, form="sep_f16x5")
    item = {"cov": cov, "z1": z1, "z2": z2, "pos": pos}
    return gsc.summate_batch([item, dict(item)], form="plain")[1]


def test_concurrent_calls_match_serial(gsc):
    seeds = list(range(12))
    serial = {s: np.array(_work(gsc, s), copy=True) for s in seeds}
    results, errors = {}, []

    def run(my_seeds):
        try:
            for _ in range(3):
                for s in my_seeds:
                    results.setdefault(s, []).append(np.array(_work(gsc, s), copy=True))
        except Exception as e:                      # reported below
            errors.append(e)

    threads = [threading.Thread(target=run, args=(seeds[i::4],)) for i in range(4)]
    for t in threads:
        t.start()
    for t in threads:
        t.join(timeout=300)
    assert not any(t.is_alive() for t in threads)
    assert not errors, errors
    for s in seeds:
        assert len(results[s]) == 3
        for got in results[s]:
            assert np.array_equal(got, serial[s]), s
