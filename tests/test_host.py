"""CPU-side checks: the C ABI exports, the host mirror and the solver-registry boundary."""
from __future__ import annotations

import ctypes
import sys

import numpy as np
import pytest

from tests.conftest import ROOT


@pytest.fixture(scope="module")
def built_library():
    from polarism_gb300 import build

    return build.build()


def test_library_exports_every_declared_symbol(built_library):
    from polarism_gb300 import _lib

    lib = ctypes.CDLL(str(built_library))
    declared = _lib.header_symbols()
    assert declared, "no pg_* declarations found in include/polarism_gb300.h"
    missing = [name for name in declared if not hasattr(lib, name)]
    assert not missing, f"declared but not exported: {missing}"
    assert set(declared) == set(_lib.SIGNATURES), "ctypes signatures out of sync with the header"


def test_library_loads_without_gpu(built_library):
    from polarism_gb300 import _lib

    lib = _lib.load(built_library)
    assert lib.pg_version() >= 1
    assert lib.pg_device_count() >= 0
    if lib.pg_device_count() == 0:
        # Without a device, creation fails loudly instead of falling back to the CPU.
        cfg = _lib.PgConfig(nx=8, ny=8, members=1, precision=0, reservoir=1, potential=0,
                            pump_per_member=0, potential_per_member=0, dx=1.0, dy=1.0, dt=1e-3)
        phys = (_lib.PgPhysics * 1)(_lib.PgPhysics(hbar=0.658, m_eff=0.284))
        handle = ctypes.c_void_p()
        status = lib.pg_create(ctypes.byref(cfg), phys, ctypes.byref(handle))
        assert status != _lib.PG_OK
        with pytest.raises(RuntimeError):
            _lib.check(status, "pg_create")


def test_invalid_arguments_rejected_before_device_use(built_library):
    from polarism_gb300 import _lib

    lib = _lib.load(built_library)
    cfg = _lib.PgConfig(nx=2, ny=8, members=1, precision=0, reservoir=1, potential=0,
                        pump_per_member=0, potential_per_member=0, dx=1.0, dy=1.0, dt=1e-3)
    phys = (_lib.PgPhysics * 1)(_lib.PgPhysics(hbar=0.658, m_eff=0.284))
    handle = ctypes.c_void_p()
    assert lib.pg_create(ctypes.byref(cfg), phys, ctypes.byref(handle)) == _lib.PG_ERR_INVALID
    assert b"4x4" in lib.pg_last_error()


def test_host_grid_matches_reference_construction():
    from polarism_gb300.host import GridParameters, PeriodicGrid

    grid = PeriodicGrid(GridParameters(nx=8, ny=6, lx=4.0, ly=3.0))
    assert grid.shape == (6, 8) and grid.dx == 0.5 and grid.dy == 0.5
    assert np.isclose(grid.X[0, 0], -1.75) and np.isclose(grid.Y[0, 0], -1.25)
    assert np.allclose(grid.k_squared[0, 1], (2 * np.pi / 4.0) ** 2)


def test_initial_field_is_zero_mean_rms_normalised():
    from polarism_gb300.host import make_initial_psi

    psi = make_initial_psi((32, 16), 1e-3, 0)
    assert abs(np.mean(psi)) < 1e-15
    assert np.isclose(np.sqrt(np.mean(np.abs(psi) ** 2)), 1e-3)
    assert np.array_equal(psi, make_initial_psi((32, 16), 1e-3, 0))


def test_stage_scales_follow_stage_times():
    from polarism_gb300.host import Config, build_simulation
    from polarism_gb300.solvers import RK4CudaSolver

    cfg = Config()
    cfg.solver.dt = 0.1
    solver = RK4CudaSolver.__new__(RK4CudaSolver)
    solver._dt = 0.1
    scales = solver.stage_scales(lambda t: t, 0.0, 3, 2, 1)
    assert np.allclose(scales[:, :, 0], [[0.3, 0.35, 0.4], [0.4, 0.45, 0.5]])
    member = solver.stage_scales(lambda t: np.asarray([t, 2 * t]), 0.0, 0, 1, 2)
    assert np.allclose(member[0], [[0.0, 0.0], [0.05, 0.1], [0.1, 0.2]])
    two = solver.stage_scales([lambda t: t, lambda t: np.asarray([1.0, 2.0])], 0.0, 1, 1, 2)
    assert two.shape == (1, 3, 2, 2)  # [step][stage][laser][member]
    assert np.allclose(two[0, :, 0], [[0.1, 0.1], [0.15, 0.15], [0.2, 0.2]])
    assert np.allclose(two[0, :, 1], [[1.0, 2.0]] * 3)
    half = solver.half_scales([lambda t: t, lambda t: 3.0], 0.0, 0, 2, 1)
    assert half.shape == (2, 2, 2, 1) and np.allclose(half[1, :, 0, 0], [0.125, 0.175])
    grid, model, state = build_simulation(cfg)
    assert state.field.shape == (1, 1, cfg.grid.ny, cfg.grid.nx)


def test_member_physics_reads_batch_values():
    from polarism_gb300.engine import MemberPhysics
    from polarism_gb300.host import BatchPhysicsLite, Config

    members = [Config(), Config()]
    members[1].physics.R = 0.05
    bp = BatchPhysicsLite(members[0].physics, members)
    assert MemberPhysics.from_object(bp, 0).R == 0.02
    assert MemberPhysics.from_object(bp, 1).R == 0.05
    assert MemberPhysics.from_object(bp, 1).gamma_C == 0.083


def _reference_importable():
    sys.path.insert(0, str(ROOT / "tests" / "golden"))
    try:
        import make_golden  # noqa: F401
        from pathlib import Path

        found = make_golden.reference_root()
        root = Path(found) if found else None
        if root is None or not (root / "polarism" / "__init__.py").exists():
            return None
        make_golden._import_reference(str(root))
        return root
    except Exception:
        return None


def test_registers_as_drop_in_for_reference_solver_names():
    root = _reference_importable()
    if root is None:
        pytest.skip("Polarism source tree not available on this host")
    import warnings

    import polarism_gb300
    from polarism.solver.solver_compatibility import solver_capabilities
    from polarism.solver.solver_registry import available_solvers

    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        registered = polarism_gb300.register()
    assert available_solvers.lookup("rk4-cuda") is registered["rk4-cuda"]
    caps = solver_capabilities("rk4-cuda")
    assert "wigner" in caps.noise and 1 in caps.components


def test_pulse_gaussian_coefficient_matches_reference_fixture():
    """The host mirror's pulsed-laser time envelope reproduces the coefficients the reference
    computed for the two-laser fixtures (``polarism/laser/pulse_gaussian.py:101-135``)."""
    import json

    from polarism_gb300.host import GridParameters, LaserParameters, PeriodicGrid, make_lasers
    from tests.conftest import load_golden

    for case in ("rk4_fdm_two_lasers", "split_cpu_two_lasers"):
        g = load_golden(case)
        pulse = json.loads(str(g["pulse"]))
        cw = LaserParameters(laser_type="continuous-gaussian", P0=0.05, sigma_space=8.0)
        pl = LaserParameters(laser_type="pulse-gaussian", **pulse)
        grid = PeriodicGrid(GridParameters(nx=32, ny=16, lx=40.0, ly=20.0))
        lasers = make_lasers(LaserParameters(mode="multiple", lasers=[cw, pl]), grid.X, grid.Y)
        assert np.allclose(lasers[1]._spatial_envelope, g["envelopes"][1], rtol=1e-15, atol=0)
        dt = float(g["dt"])
        got = np.asarray([[[laser.power_coefficient(k * dt + c * dt) for laser in lasers]
                           for c in g["nodes"]] for k in range(int(g["steps"]))])
        np.testing.assert_allclose(got, g["coefficients"], rtol=1e-13, atol=1e-15)
