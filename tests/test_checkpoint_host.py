"""Checkpoint format 2 files (``polarism/simulation_controller.py:736-923``) without a GPU: the
entry names of ``save_checkpoint`` and a lossless round trip through the archive."""
from __future__ import annotations

import numpy as np
import pytest

from polarism_gb300 import checkpoint


def _ckpt():
    rng = np.random.default_rng(0)
    b, ny, nx = 3, 4, 8
    return {
        "attrs": {"checkpoint_version": 2, "polarism_version": "polarism_gb300", "step": 40,
                  "t": 0.4, "t0": 0.0, "dt": 0.01, "ndim": 2, "shape": np.asarray([ny, nx]),
                  "components": 1, "batched": True, "reservoir_type": "double",
                  "config_json": '{"solver": {"dt": 0.01}}', "steady_last_step": 40,
                  "stop_time": np.asarray([0.3, np.nan, 0.4]), "steady_norm": rng.random(b)},
        "data": {"field": rng.standard_normal((b, 1, ny, nx)) + 1j,
                 "steady_density": rng.random((b, ny, nx)).astype(np.float32)},
        "reservoir": {"nA": rng.random((b, 1, ny, nx)), "nI": rng.random((b, 1, ny, nx))},
        "accumulators": {"g2": {"t_first": 0.0, "t_last": None, "samples": 5,
                                "sum_density": rng.random((b, ny, nx)),
                                "sum_density_squared": rng.random((b, ny, nx))}},
        "step_controller": {"h_next": 0.02, "err_prev": 0.5, "accepted": 7, "rejected": 1},
    }


def test_npz_round_trip_keeps_every_entry(tmp_path):
    ck = _ckpt()
    path = checkpoint.save(tmp_path / "run.npz", ck)
    back = checkpoint.load(path)
    assert list(back["reservoir"]) == ["nA", "nI"]  # state_names order
    for group in ("data", "reservoir"):
        for key, value in ck[group].items():
            assert np.array_equal(back[group][key], value) and back[group][key].dtype == value.dtype
    for key, value in ck["attrs"].items():
        np.testing.assert_array_equal(back["attrs"][key], value)
    acc = back["accumulators"]["g2"]
    assert acc["samples"] == 5 and acc["t_first"] == 0.0 and acc["t_last"] is None
    assert np.array_equal(acc["sum_density"], ck["accumulators"]["g2"]["sum_density"])
    assert back["step_controller"]["accepted"] == 7
    assert isinstance(back["attrs"]["config_json"], str)


def test_h5_layout_matches_save_checkpoint(tmp_path):
    h5py = pytest.importorskip("h5py")
    path = checkpoint.save(tmp_path / "run.h5", _ckpt())
    with h5py.File(path, "r") as h5:
        assert h5.attrs["checkpoint_version"] == 2
        assert set(h5["reservoir"]) == {"nA", "nI"}
        assert h5["accumulators"]["g2"].attrs["samples"] == 5
        assert "steady_density" in h5 and "field" in h5
    back = checkpoint.load(path)
    assert np.array_equal(back["data"]["field"], _ckpt()["data"]["field"])


def test_accumulator_names_follow_the_reference():
    assert set(checkpoint.ACCUMULATORS) == {"g2", "momentum-distribution"}
    assert [k for _, k in checkpoint.ACCUMULATORS["g2"]] == ["sum_density", "sum_density_squared"]


class _RecordingEngine:
    """Stands in for an engine: records what restore() hands it."""

    members, ny, nx = 3, 4, 8
    complex, real = np.complex128, np.float64

    def set_state(self, psi, res):
        self.psi, self.res = psi, res

    def steady_import(self, density, norms, stops):
        self.stops = stops

    def accumulator_load(self, kind, sums, samples):
        pass


def test_restore_orders_quadratic_double_fields_by_state_names():
    """A quadratic-double reservoir's state_names are ('nR', 'nI'); an HDF5 group lists them
    alphabetically ('nI', 'nR'), so restore must take the order from the reservoir type."""
    ck = _ckpt()
    ck["attrs"]["reservoir_type"] = "quadratic-double"
    n_r, n_i = ck["reservoir"]["nA"], ck["reservoir"]["nI"]
    ck["reservoir"] = {"nI": n_i, "nR": n_r}  # the order h5py iterates a group in
    eng = _RecordingEngine()
    assert checkpoint.restore(eng, ck) == 40
    assert np.array_equal(eng.res[0], n_r) and np.array_equal(eng.res[1], n_i)
    ck["attrs"]["reservoir_type"] = "double"
    ck["reservoir"] = {"nI": n_i, "nA": n_r}
    checkpoint.restore(eng, ck)
    assert np.array_equal(eng.res[0], n_r) and np.array_equal(eng.res[1], n_i)


def test_restore_rejects_reservoir_names_of_another_type():
    ck = _ckpt()
    ck["attrs"]["reservoir_type"] = "quadratic-double"  # stored names are nA / nI
    with pytest.raises(ValueError, match="reservoir names mismatch"):
        checkpoint.restore(_RecordingEngine(), ck)
