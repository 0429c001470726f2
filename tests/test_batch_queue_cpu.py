"""The batch planner's work queue, checked on the host (no GPU needed).

gsc_selftest_batch_queue builds the cost-sorted queue that a batch plan
would upload (point blocks of 128 threads x points-per-thread, modes split
into tile-multiple ranges) from item descriptors alone and runs the same
validator every plan runs before its upload.  Checked here: the planner's
queues are valid over seeded random ensembles, configurations and block
counts (edge sizes included: no points, no modes, one point, one mode), and
each injected corruption (a dropped, duplicated or misaddressed unit, a
shifted mode range, a misaligned point block, a split out of range) is
refused with GSC_ERR_INVALID and a message naming the fault.
"""
import ctypes

import numpy as np
import pytest

FORMS = {"plain": 1, "mixed": 6}   # GSC_FORM_PLAIN_F64, GSC_FORM_MIXED
CONFIGS = {"plain": [(2, 8, 4), (4, 8, 16), (4, 16, 4), (8, 8, 16)],
           "mixed": [(2, 32, 4), (4, 32, 16), (8, 32, 4)]}


def _items(native, specs):
    arr = (native.GscBatchItem * max(1, len(specs)))()
    for i, (kind, dim, n, p) in enumerate(specs):
        arr[i].dim = dim
        arr[i].kind = kind
        arr[i].n_modes = n
        arr[i].n_points = p
    return arr


def _config(native, R, tile, upb):
    c = native.GscBatchConfig()
    c.struct_size = ctypes.sizeof(native.GscBatchConfig)
    c.points_per_thread = R
    c.tile_modes = tile
    c.units_per_block = upb
    return c


def _run(native, specs, form, cfg, blocks, corruption):
    items = _items(native, specs)
    return native.lib.gsc_selftest_batch_queue(items, len(specs), FORMS[form],
                                               ctypes.byref(_config(native, *cfg)), blocks,
                                               corruption)


def _random_specs(rng, count):
    specs = []
    for _ in range(count):
        kind = int(rng.integers(0, 3))
        dim = int(rng.integers(2, 4)) if kind == 1 else int(rng.integers(1, 4))
        n = int(rng.choice([0, 1, 7, 8, 9, 31, 32, 33, 255, 256, 257, 1000, 5000]))
        p = int(rng.choice([0, 1, 127, 128, 129, 511, 512, 513, 4096, 70000]))
        specs.append((kind, dim, n, p))
    return specs


@pytest.fixture(scope="module")
def native():
    from gstools_core import _native
    return _native


@pytest.mark.parametrize("form", ["plain", "mixed"])
def test_planner_queues_are_valid(native, form):
    rng = np.random.default_rng(17 if form == "plain" else 18)
    for trial in range(40):
        specs = _random_specs(rng, int(rng.integers(1, 12)))
        for cfg in CONFIGS[form]:
            for blocks in (1, 152, 608, 4864):
                rc = _run(native, specs, form, cfg, blocks, 0)
                assert rc == 0, (trial, specs, cfg, blocks, native.lib.gsc_last_error())


def test_splits_are_exercised(native):
    """Few points over many modes with many blocks: the planner splits the
    modes, and the split queue still validates."""
    specs = [(0, 3, 6000, 700), (1, 2, 3000, 300), (2, 2, 4096, 129)]
    assert _run(native, specs, "plain", (4, 8, 64), 4864, 0) == 0
    # one corrupted split range is caught
    assert _run(native, specs, "plain", (4, 8, 64), 4864, 4) == native.GSC_ERR_INVALID


@pytest.mark.parametrize("corruption,words", [
    (1, b"units for"), (2, b"repeats"), (3, b"names item"), (4, b"does not start where"),
    (5, b"starts at point"), (6, b"names split")])
@pytest.mark.parametrize("form", ["plain", "mixed"])
def test_corrupt_queues_are_refused(native, form, corruption, words):
    specs = [(0, 3, 300, 70000), (1, 3, 257, 12345), (2, 2, 500, 3000), (0, 1, 0, 100)]
    rc = _run(native, specs, form, CONFIGS[form][1], 152, corruption)
    assert rc == native.GSC_ERR_INVALID
    msg = native.lib.gsc_last_error()
    assert b"corrupt batch work queue" in msg and words in msg, msg


def test_item_and_argument_checks_without_device(native):
    ok = (4, 8, 4)
    assert _run(native, [(0, 2, -1, 10)], "plain", ok, 152, 0) == native.GSC_ERR_INVALID
    assert _run(native, [(7, 2, 10, 10)], "plain", ok, 152, 0) == native.GSC_ERR_INVALID
    assert _run(native, [(1, 1, 10, 10)], "plain", ok, 152, 0) == native.GSC_ERR_DIM
    assert _run(native, [(0, 2, 10, 10)], "plain", (3, 8, 4), 152, 0) == native.GSC_ERR_INVALID
    assert _run(native, [(0, 2, 10, 10)], "plain", ok, 0, 0) == native.GSC_ERR_INVALID
    assert _run(native, [(0, 2, 10, 10)], "plain", ok, 152, 9) == native.GSC_ERR_INVALID
    assert _run(native, [(0, 2, 10, 0)], "plain", ok, 152, 1) == native.GSC_ERR_INVALID
    assert b"no units" in native.lib.gsc_last_error()


def test_allocation_injection_arguments(native):
    lib = native.lib
    assert lib.gsc_selftest_fail_alloc(-2) == native.GSC_ERR_INVALID
    assert lib.gsc_selftest_fail_alloc(3) == 0
    assert lib.gsc_selftest_fail_alloc(-1) == 0
