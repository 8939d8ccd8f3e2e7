"""The full-size precision check (1024^2, 1000 steps, rk4-fdm and split-step-fft, FP32 and
FP64, against the FP64 oracle on psi, n_R and the norm trajectory).  The oracle leg takes about
a quarter of an hour of CPU per case, so the test runs only when PG_PRECISION_CHECK=1; the
recorded errors are in ``profiles/precision_check_1024x1000.md``."""
from __future__ import annotations

import os

import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.skipif(os.environ.get("PG_PRECISION_CHECK") != "1",
                    reason="full-size precision check: set PG_PRECISION_CHECK=1 (CPU-heavy oracle)")
def test_precision_check_full_size(cuda_lib, tmp_path):
    from tests import precision_check as pc

    pc.gpu_leg(tmp_path)
    results = pc.oracle_leg(tmp_path, tmp_path / "results.json")
    failed = {k: v for k, v in results.items() if not v["pass"]}
    assert not failed, failed
