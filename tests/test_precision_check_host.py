"""Host logic of the full-size precision check, on a small grid without a GPU: the oracle leg
reads a device leg's files and reports relative L2 errors (zero for an oracle-made file)."""
from __future__ import annotations

import numpy as np


def test_oracle_leg_reports_errors_of_a_device_file(tmp_path):
    from tests import precision_check as pc

    n, steps = 16, 3
    for method, precision in pc.CASES:
        psi, res, norms, fp = pc.oracle_case(method, precision, steps, n)
        env = pc.inputs(n)[3]
        np.savez(tmp_path / f"{pc.case_name(method, precision)}.npz", psi=psi, res=res,
                 norms=norms, wall=0.0, inputs=fp, env=env, steps=steps, n=n)
    results = pc.oracle_leg(tmp_path, tmp_path / "r.json", jobs=1)
    assert set(results) == {pc.case_name(m, p) for m, p in pc.CASES}
    for r in results.values():
        assert r["psi_rel_l2"] == 0.0 and r["n_R_rel_l2"] == 0.0 and r["pass"]
    # A perturbed device state is reported, not hidden.
    g = dict(np.load(tmp_path / "rk4_fp32.npz"))
    g["psi"] = g["psi"] * (1 + 1e-3)
    np.savez(tmp_path / "rk4_fp32.npz", **g)
    r = pc.oracle_leg(tmp_path, tmp_path / "r.json", jobs=1)["rk4_fp32"]
    assert abs(r["psi_rel_l2"] - 1e-3) < 1e-9 and not r["pass"]


def test_committed_oracle_fixtures_start_from_the_workload_and_match_the_oracle():
    """The full-size fixtures (tests/golden/precision_*.npz, written by
    make_precision_golden.py) belong to this workload: same initial field (fingerprint),
    1000 norms, 128^2 sampled sites, and the oracle's first two steps reproduce their first
    two norms."""
    from tests import precision_check as pc
    from tests.conftest import load_golden

    fp = pc.fingerprint(pc.inputs(pc.N)[4])
    for method, precision in pc.CASES:
        g = load_golden(f"precision_{pc.case_name(method, precision)}")
        assert str(g["inputs"]) == fp
        assert g["norms"].shape == (pc.STEPS,) and int(g["steps"]) == pc.STEPS
        assert g["psi"].shape == (128, 128) and g["res"].shape == (128, 128)
        assert np.all(g["res"] >= 0) and np.all(np.isfinite(g["psi"]))
        _, _, norms, _ = pc.oracle_case(method, precision, 2, pc.N)
        np.testing.assert_allclose(norms, g["norms"][:2], rtol=1e-13)
