"""Shared fixtures.  Tests marked ``gpu`` need a CUDA device and the built library; everything
else runs on the CPU (oracle against golden vectors, host logic, the C ABI surface)."""
from __future__ import annotations

import importlib
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

PACKAGE = "sphere-stereo_gb300"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built sm_103a library")


@pytest.fixture(autouse=True)
def _restore_tuning_knobs(request):
    """The library's launch-shape knobs are process-wide: a GPU test that tunes or sets them must
    not change the launches of the tests after it."""
    if "gpu" not in request.keywords:
        yield
        return
    tune = importlib.import_module(PACKAGE + ".autotune")
    try:
        saved = {k: tune.get(k) for k in tune.KNOBS}
    except Exception:  # library not loadable: the test itself reports that
        saved = {}
    yield
    for k, v in saved.items():
        tune.set_knob(k, v)


@pytest.fixture(scope="session")
def ss():
    return importlib.import_module(PACKAGE)


@pytest.fixture(scope="session")
def synthetic():
    return importlib.import_module(PACKAGE + ".synthetic")


@pytest.fixture(scope="session")
def native(ss):
    """The loaded C ABI library (built first if needed and nvcc is available)."""
    builder = importlib.import_module(PACKAGE + "._build")
    if not os.path.exists(builder.LIBRARY):
        try:
            builder.build()
        except RuntimeError as e:
            pytest.skip(f"library not built and cannot be built here: {e}")
    return ss._native.library()


@pytest.fixture(scope="session")
def oracle_mod():
    import sphere_oracle

    sphere_oracle.build()
    return sphere_oracle


def load_golden(name: str):
    z = np.load(os.path.join(GOLDEN, name))
    out = {k: z[k] for k in z.files}
    if "config" in out:
        out["config"] = json.loads(str(out["config"]))
        out["calibration"] = json.loads(str(out["calibration"]))
    return out


@pytest.fixture(scope="session")
def golden_small():
    return load_golden("pipeline_small.npz")


@pytest.fixture(scope="session")
def golden_c1():
    return load_golden("pipeline_c1.npz")


@pytest.fixture(scope="session")
def golden_c2():
    g = load_golden("pipeline_c2.npz")
    g["inputs"] = json.loads(str(g["inputs"]))
    return g


def sample_lattice(cols: int, rows: int, stride: int) -> np.ndarray:
    """The pixel sample of the c2 fixture: flat indices of (x, y) with (x + 3 y) mod stride == 0."""
    y, x = np.divmod(np.arange(cols * rows, dtype=np.int64), cols)
    return np.nonzero((x + 3 * y) % stride == 0)[0]


@pytest.fixture(scope="session")
def golden_isb():
    return load_golden("isb_cases.npz")


def psnr(a, b) -> float:
    mse = float(np.mean((np.asarray(a, np.float64) - np.asarray(b, np.float64)) ** 2))
    return float("inf") if mse == 0 else 10 * np.log10(255.0 ** 2 / mse)


def inverse_distance_mae(d_test, d_ref) -> float:
    return float(np.mean(np.abs(1.0 / np.asarray(d_test, np.float64) - 1.0 / np.asarray(d_ref, np.float64))))
