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


_FIRST_CALLS = r'''
import sys, threading
import numpy as np
sys.path[:0] = [sys.argv[1], sys.argv[2]]
import gstools_core as gsc
import oracle

rng = np.random.default_rng(3)
cov = rng.normal(0.0, 0.3, (3, 300))
z1, z2 = rng.standard_normal(300), rng.standard_normal(300)
pos = rng.uniform(-20.0, 20.0, (3, 30000))
axes = tuple(np.arange(s, dtype=np.float64) for s in (6, 40, 64))
axes_inc = tuple(np.arange(s, dtype=np.float64) for s in (6, 40, 192))

def flat(ax):
    return np.ascontiguousarray(np.array(np.meshgrid(*ax, indexing="ij")).reshape(len(ax), -1))

# every call below is the first of its kernel instantiation in this process
jobs = [
    ("plain 3-D", lambda: gsc.summate(cov, z1, z2, pos, form="plain"),
     lambda: oracle.summator(cov, z1, z2, pos, num_threads=4), 1e-12),
    ("plain 2-D", lambda: gsc.summate(cov[:2], z1, z2, pos[:2], form="plain"),
     lambda: oracle.summator(cov[:2], z1, z2, pos[:2], num_threads=4), 1e-12),
    ("plain incompr", lambda: gsc.summate_incompr(cov, z1, z2, pos, form="plain"),
     lambda: oracle.summator_incompr(cov, z1, z2, pos, num_threads=4), 1e-12),
    ("x5 256-wide", lambda: gsc.summate_structured(cov, z1, z2, axes, form="sep_f16x5"),
     lambda: oracle.summator(cov, z1, z2, flat(axes), num_threads=4), 1e-6),
    ("x5 192-wide incompr",
     lambda: gsc.summate_incompr_structured(cov, z1, z2, axes_inc, form="sep_f16x5"),
     lambda: oracle.summator_incompr(cov, z1, z2, flat(axes_inc), num_threads=4), 1e-6),
    ("f16x3", lambda: gsc.summate_structured(cov, z1, z2, axes, form="sep_f16x3"),
     lambda: oracle.summator(cov, z1, z2, flat(axes), num_threads=4), 1e-5),
    ("batch", lambda: gsc.summate_batch([{"cov": cov, "z1": z1, "z2": z2, "pos": pos}],
                                        form="plain")[0],
     lambda: oracle.summator(cov, z1, z2, pos, num_threads=4), 1e-12),
]
out, errs = {}, []
barrier = threading.Barrier(len(jobs))

def run(name, fn):
    try:
        barrier.wait()
        out[name] = np.array(fn(), copy=True)
    except Exception as e:
        errs.append(f"{name}: {e!r}")

th = [threading.Thread(target=run, args=(n, f)) for n, f, _, _ in jobs]
for t in th: t.start()
for t in th: t.join(300)
assert not errs, errs
for name, _, ref_fn, tol in jobs:
    ref = np.asarray(ref_fn())
    e = float(np.max(np.abs(out[name] - ref)) / np.sqrt(np.mean(ref ** 2)))
    assert e <= tol, (name, e)
print("ok", len(jobs))
'''


def test_first_calls_of_fresh_kernels_race_safely():
    """A fresh process whose threads make the first call of seven kernel
    instantiations at once (each needs its one-time launch set-up on the
    device, among them the >48 KB shared-memory plain and x5 kernels): every
    result must match the oracle at its form's bar."""
    import subprocess
    import sys
    from conftest import PKG_DIR, ROOT
    r = subprocess.run([sys.executable, "-c", _FIRST_CALLS, PKG_DIR, ROOT],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "ok 7" in r.stdout
