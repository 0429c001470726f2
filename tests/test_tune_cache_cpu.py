"""The autotuner's cache file, on the CPU (no device is touched).

Tuned launch configurations are kept per (device name, kernel family, shape
buckets) and, with a cache file, persisted as text with a header, one entry
per line and an FNV-1a 64 checksum of everything above the checksum line.
Checked here: entries written through the C ABI land in the file and load
back in a fresh process; a file with a changed byte, a wrong header, a
malformed entry or no checksum is refused (GSC_ERR_INVALID) and is then
neither read nor overwritten; a missing file is created on the first entry.
Each case runs in a fresh process, since the cache is process-wide.
"""
import os
import subprocess
import sys

import pytest

from conftest import PKG_DIR, ROOT

_PRELUDE = r'''
import ctypes, sys
sys.path[:0] = [sys.argv[1], sys.argv[2]]
from gstools_core import _native
lib = _native.lib
def put(key, *v):
    arr = (ctypes.c_int32 * 4)(*v)
    assert lib.gsc_tune_cache_put(key.encode(), arr) == 0
def get(key):
    arr = (ctypes.c_int32 * 4)()
    rc = lib.gsc_tune_cache_get(key.encode(), arr)
    return list(arr) if rc == 0 else None
def size():
    n = ctypes.c_int64(-1)
    assert lib.gsc_tune_cache_size(ctypes.byref(n)) == 0
    return n.value
path = sys.argv[3].encode()
'''


def _run(body, path):
    r = subprocess.run([sys.executable, "-c", _PRELUDE + body, PKG_DIR, ROOT, str(path)],
                       capture_output=True, text=True, timeout=120,
                       env=dict(os.environ, GSC_TUNE_CACHE=""))
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


def _fnv1a(data: bytes) -> int:
    h = 1469598103934665603
    for b in data:
        h = ((h ^ b) * 1099511628211) & 0xFFFFFFFFFFFFFFFF
    return h


def test_entries_persist_across_processes(native_lib, tmp_path):
    path = tmp_path / "tune.txt"
    _run("""
assert lib.gsc_tune_cache_open(path) == 0
assert size() == 0
put("GPU X|mixed|d3s|p25|n13", 8, 16, 0, 0)
put("GPU X|batch|f6|c512|w38|p27", 4, 32, 16, 0)
""", path)
    text = path.read_bytes()
    assert text.startswith(b"# gstools-core-gb300 autotuner cache v1\n")
    body, tail = text.rsplit(b"#checksum ", 1)
    assert int(tail.strip(), 16) == _fnv1a(body)
    assert b"GPU X|mixed|d3s|p25|n13\t8 16 0 0\n" in body
    out = _run("""
assert lib.gsc_tune_cache_open(path) == 0
print(size(), get("GPU X|mixed|d3s|p25|n13"), get("GPU X|batch|f6|c512|w38|p27"), get("nope"))
""", path)
    assert out.strip() == "2 [8, 16, 0, 0] [4, 32, 16, 0] None"


@pytest.mark.parametrize("damage", ["byte", "header", "entry", "checksum"])
def test_damaged_file_is_refused_and_left_alone(native_lib, tmp_path, damage):
    path = tmp_path / "tune.txt"
    _run("""
assert lib.gsc_tune_cache_open(path) == 0
put("GPU X|mixed|d2s|p20|n10", 2, 4, 0, 0)
""", path)
    text = path.read_bytes()
    if damage == "byte":
        i = text.index(b"\t2 4") + 1
        bad = text[:i] + b"8" + text[i + 1:]
    elif damage == "header":
        bad = b"# some other file\n" + text.split(b"\n", 1)[1]
    elif damage == "entry":
        body, _ = text.rsplit(b"#checksum ", 1)
        body = body + b"no tab here\n"
        bad = body + b"#checksum %016x\n" % _fnv1a(body)
    else:
        bad = text.rsplit(b"#checksum ", 1)[0]
    path.write_bytes(bad)
    out = _run("""
rc = lib.gsc_tune_cache_open(path)
print(rc, lib.gsc_last_error().decode())
print(size())
put("GPU X|mixed|d3s|p21|n11", 4, 8, 0, 0)      # kept in memory only
""", path)
    rc, msg = out.splitlines()[0].split(" ", 1)
    assert int(rc) == 1 and "refused" in msg
    assert out.splitlines()[1] == "0"
    assert path.read_bytes() == bad                 # not overwritten


def test_missing_file_is_created(native_lib, tmp_path):
    path = tmp_path / "sub_tune.txt"
    _run("""
assert lib.gsc_tune_cache_open(path) == 0
put("k", 1, 2, 3, 4)
assert lib.gsc_tune_set_mode(3) == 1 and lib.gsc_tune_set_mode(1) == 0
""", path)
    assert b"k\t1 2 3 4\n" in path.read_bytes()
