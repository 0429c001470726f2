import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG_DIR = os.path.join(ROOT, "gstools-core_gb300")
for p in (ROOT, PKG_DIR):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN_DIR = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def goldens():
    """Known answers of the reference crate's src/field.rs tests."""
    with open(os.path.join(GOLDEN_DIR, "field_rs_goldens.json")) as fh:
        raw = json.load(fh)["arrays"]
    return {k: np.array(v["value"], dtype=np.float64) for k, v in raw.items()}


def ulps_eq(a: float, b: float, max_ulps: int = 6, epsilon: float = np.finfo(np.float64).eps):
    """approx 0.5 `ulps_eq` for f64: abs diff <= epsilon, else same sign and
    at most ``max_ulps`` units in the last place apart."""
    if abs(a - b) <= epsilon:
        return True
    if (a < 0) != (b < 0):
        return False
    ia = np.array(a, dtype=np.float64).view(np.int64)
    ib = np.array(b, dtype=np.float64).view(np.int64)
    return abs(int(ia) - int(ib)) <= max_ulps


def _build_native():
    """Builds the CUDA library (cross-compiles without a GPU) once per session."""
    import shutil
    from gsc_build import build, LIB_PATH, _up_to_date
    if not _up_to_date():
        if not (shutil.which("nvcc") or os.path.exists("/usr/local/cuda/bin/nvcc")):
            pytest.skip("nvcc not available to build the native library")
        build()
    return LIB_PATH


@pytest.fixture(scope="session")
def native_lib():
    return _build_native()


@pytest.fixture(scope="session")
def gsc(native_lib):
    import gstools_core
    return gstools_core


def rms(a):
    a = np.asarray(a, dtype=np.float64)
    return float(np.sqrt(np.mean(a * a))) if a.size else 0.0


def rel_err(got, ref):
    """max |got - ref| / RMS(ref) (the error measure of every parity bar)."""
    got = np.asarray(got, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    if ref.size == 0:
        return 0.0
    r = rms(ref)
    return float(np.max(np.abs(got - ref)) / (r if r > 0 else 1.0))
