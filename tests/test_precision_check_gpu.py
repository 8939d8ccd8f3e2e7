"""The full-size precision check on the GPU: 1024^2 periodic, lx = ly = 400 um, dt = 5e-4 ps,
1000 steps with Wigner noise on (Philox key 42), rk4-fdm and split-step-fft (CPU ordering), in
complex64 and complex128, against the FP64 oracle.

The oracle's side (a quarter of an hour of CPU per case) is committed as
``tests/golden/precision_<case>.npz`` by ``tests/golden/make_precision_golden.py``: the
1000-entry norm trajectory and the final psi and n_R on every 8th row and column.  The device
leg runs here in full and is compared on those: relative L2 of the norm trajectory, of psi and
of n_R on the sampled sites, and the largest relative error of any single norm.

Bars: 1e-10 in FP64, 1e-4 in FP32 (the precision the path is held to); the FP32 runs are
also held to 5e-5, half that bar, so that a systematic drift shows before it reaches it.
"""
from __future__ import annotations

import numpy as np
import pytest

from tests.conftest import load_golden, rel_l2

pytestmark = pytest.mark.gpu

BARS = {"double": (1e-10, 1e-10), "single": (1e-4, 5e-5)}


@pytest.mark.parametrize("method,precision", [("rk4", "single"), ("rk4", "double"),
                                              ("split", "single"), ("split", "double")])
def test_precision_check_1024_1000_steps(cuda_lib, method, precision):
    from tests import precision_check as pc

    ref = load_golden(f"precision_{pc.case_name(method, precision)}")
    stride = int(ref["stride"])
    g = pc.gpu_case(method, precision, int(ref["steps"]), int(ref["n"]))
    assert g["inputs"] == str(ref["inputs"]), "the device run started from another initial field"
    errors = {
        "norm_trajectory": rel_l2(g["norms"], ref["norms"]),
        "norm_max": float(np.max(np.abs(g["norms"] - ref["norms"]) / np.abs(ref["norms"]))),
        "psi": rel_l2(g["psi"][0, 0, ::stride, ::stride].astype(np.complex128), ref["psi"]),
        "n_R": rel_l2(g["res"][0, 0, ::stride, ::stride].astype(np.float64), ref["res"]),
    }
    bar, margin = BARS[precision]
    print(f"{pc.case_name(method, precision)}: " +
          "  ".join(f"{k} {v:.3e}" for k, v in errors.items()) + f"  (bar {bar:g})")
    assert all(v < bar for v in errors.values()), errors
    assert all(v < margin for v in errors.values()), (f"inside the {bar:g} bar but above "
                                                      f"{margin:g}", errors)
