"""Shared pytest setup: markers, golden-fixture loading and the repository path."""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = ROOT / "tests" / "golden"
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built library")
    config.addinivalue_line("markers", "slow: long-running case")


def load_golden(name):
    """Return a golden fixture as a dict, decoding the physics JSON strings."""
    with np.load(GOLDEN / f"{name}.npz") as data:
        out = {key: data[key] for key in data.files}
    for key, value in list(out.items()):
        if key.endswith("physics"):
            out[key] = json.loads(str(value))
    return out


@pytest.fixture
def golden():
    return load_golden


def rel_l2(actual, expected):
    actual = np.asarray(actual)
    expected = np.asarray(expected)
    return float(np.linalg.norm((actual - expected).ravel())
                 / max(np.linalg.norm(expected.ravel()), 1e-300))


@pytest.fixture(scope="session")
def cuda_lib():
    """The built CUDA library; GPU tests fail loudly when it or the device is missing."""
    from polarism_gb300 import _lib

    lib = _lib.load()
    if lib.pg_device_count() < 1:
        raise RuntimeError("no CUDA device visible to the polarism_gb300 library")
    return lib
