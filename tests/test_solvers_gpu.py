"""The reference-facing solver classes (the drop-in boundary) on the GPU.

Drives ``RK4CudaSolver``, ``SplitStepFFTSolver`` and ``SplitStepFFTCudaSolver`` through
the ``AbstractSolver`` contract (``advance(model, state, n)``, ``step``) with the host
mirror of Polarism's objects, and checks them against the FP64 oracle: 1e-10 in FP64
and 1e-4 in FP32 (relative L2), plus the state bookkeeping of
``polarism/solver/rk4_cuda_solver.py:3641-3642``.
"""
from __future__ import annotations

import copy

import numpy as np
import pytest

from oracle import gpe
from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu


def _config(precision="double", nx=32, ny=16, wigner=True):
    from polarism_gb300.host import Config

    cfg = Config()
    cfg.grid.nx, cfg.grid.ny, cfg.grid.lx, cfg.grid.ly = nx, ny, 40.0, 20.0
    cfg.solver.dt = 2e-3
    cfg.solver.precision = precision
    cfg.laser.P0, cfg.laser.sigma_space = 0.05, 6.0
    cfg.noise.seed = 42
    cfg.noise.initial_amplitude = 0.05
    if wigner:
        cfg.noise.stochastic = "wigner"
    return cfg


def _members(cfg, n):
    out = []
    for m in range(n):
        c = copy.deepcopy(cfg)
        c.noise.seed = 42 + m
        c.laser.P0 = 0.03 + 0.01 * m
        c.laser.sigma_space = 5.0 + m
        c.physics.R = 0.02 + 0.002 * m
        out.append(c)
    return out


def _physics(cfg):
    return {k: getattr(cfg.physics, k) for k in ("hbar", "m_eff", "g_C", "g_R", "g_I", "R",
                                                  "gamma_C", "gamma_R")}


def _oracle_member(cfg, grid, psi0, n0, env, steps, method, normals):
    p = _physics(cfg)
    dt = cfg.solver.dt
    noise = gpe.Noise([cfg.noise.seed], [p["gamma_C"]], [p["R"]], [1.0], dt, grid.dx * grid.dy,
                      "double", normals_precision=normals)
    pump = env * cfg.laser.P0
    if method == "rk4":
        return gpe.rk4_advance(psi0, (n0,), lambda t: pump, 0.0, p, grid.dx, grid.dy, dt, 0, steps,
                               noise=noise)
    return gpe.split_advance(method, psi0, (n0,), lambda t: pump, 0.0, p, grid.k_squared,
                             grid.dx, grid.dy, dt, 0, steps, noise=noise)


@pytest.mark.parametrize("precision,tol", [("double", 1e-10), ("single", 1e-4)])
@pytest.mark.parametrize("solver_name", ["RK4CudaSolver", "SplitStepFFTSolver",
                                         "SplitStepFFTCudaSolver"])
def test_solver_contract_batched_members(cuda_lib, precision, tol, solver_name):
    from polarism_gb300 import solvers
    from polarism_gb300.host import build_simulation

    cfg = _config(precision)
    members = _members(cfg, 3)
    grid, model, state = build_simulation(cfg, members)
    psi0 = state.field.astype(np.complex128).copy()
    n0 = model.reservoir.get_state()[0].astype(np.float64).copy()
    solver = getattr(solvers, solver_name)(cfg, grid, model)
    steps = 9
    solver.advance(model, state, 5)
    solver.step(model, state, cfg.solver.dt)
    solver.advance(model, state, steps - 6)
    assert state.step == steps and state.t == state.t0 + steps * cfg.solver.dt
    if solver_name == "SplitStepFFTCudaSolver":
        assert state.field_k is not None and state._field is None
        psi = np.fft.ifft2(state.field_k.astype(np.complex128), axes=(-2, -1))
    else:
        psi = state.field
    res = model.reservoir.get_state()[0]
    method = {"RK4CudaSolver": "rk4", "SplitStepFFTSolver": "cpu",
              "SplitStepFFTCudaSolver": "kouter"}[solver_name]
    envs = model.pump.separable_terms()[0][0]
    for m, mc in enumerate(members):
        env = np.asarray(envs[m, 0] if np.ndim(envs) == 4 else envs, dtype=np.float64)
        if solver_name == "SplitStepFFTCudaSolver":
            # The GPU ordering continues from a spectrum across calls: run the oracle the same way.
            p_o, f_o = psi0[m:m + 1], (n0[m:m + 1],)
            for start, count in ((0, 5), (5, 1), (6, steps - 6)):
                p = _physics(mc)
                noise = gpe.Noise([mc.noise.seed], [p["gamma_C"]], [p["R"]], [1.0], mc.solver.dt,
                                  grid.dx * grid.dy, "double", normals_precision=precision)
                p_o, f_o = gpe.split_advance("kouter", p_o, f_o, lambda t: env * mc.laser.P0, 0.0,
                                             p, grid.k_squared, grid.dx, grid.dy, mc.solver.dt,
                                             start, count, noise=noise)
        else:
            p_o, f_o = _oracle_member(mc, grid, psi0[m:m + 1].copy(), n0[m:m + 1].copy(), env,
                                      steps, method, precision)
        assert rel_l2(psi[m], p_o[0]) < tol, m
        assert rel_l2(res[m], f_o[0][0]) < tol, m


def test_device_resident_state(cuda_lib):
    """CUDA tensors in the state stay on the device (pointer path of the C ABI)."""
    import torch

    from polarism_gb300.host import build_simulation
    from polarism_gb300.solvers import RK4CudaSolver

    cfg = _config("single")
    grid, model, state = build_simulation(cfg)
    host_psi = state.field.copy()
    host_n = model.reservoir.get_state()[0].copy()
    ref_solver = RK4CudaSolver(cfg, grid, model)
    ref_solver.advance(model, state, 4)
    expect_psi, expect_n = state.field.copy(), model.reservoir.get_state()[0].copy()

    grid2, model2, state2 = build_simulation(cfg)
    state2.field = torch.as_tensor(host_psi, device="cuda")
    model2.reservoir.nR = torch.as_tensor(host_n, device="cuda")

    class DeviceReservoir:
        def __init__(self, n):
            self.nR = n

        def get_state(self):
            return (self.nR,)

        def set_state(self, s):
            self.nR = s[0].clamp_min(0)

    model2.reservoir = DeviceReservoir(model2.reservoir.nR)
    solver = RK4CudaSolver(cfg, grid2, model2)
    solver.advance(model2, state2, 4)
    assert state2.field.is_cuda
    assert np.array_equal(state2.field.cpu().numpy(), expect_psi)
    assert np.array_equal(model2.reservoir.nR.cpu().numpy(), expect_n)


@pytest.mark.parametrize("solver_name", ["RK4CudaSolver", "SplitStepFFTSolver"])
def test_in_place_host_results_match_default_path(cuda_lib, solver_name):
    """``inplace_host``: results land in the caller's own psi and n_R arrays (no new arrays, no
    second host clamp of n_R) and equal the default path's bit for bit across several calls."""
    from polarism_gb300 import solvers
    from polarism_gb300.host import build_simulation

    cfg = _config("single")
    members = _members(cfg, 2)
    outs = []
    for inplace in (False, True):
        grid, model, state = build_simulation(cfg, members)
        solver = getattr(solvers, solver_name)(cfg, grid, model)
        solver.inplace_host = inplace
        psi_buf, n_buf = state.field, model.reservoir.get_state()[0]
        for _ in range(3):
            solver.advance(model, state, 4)
        if inplace:
            assert state.field is psi_buf and model.reservoir.get_state()[0] is n_buf
        assert np.all(model.reservoir.get_state()[0] >= 0)
        outs.append((state.field.copy(), model.reservoir.get_state()[0].copy()))
    assert np.array_equal(outs[0][0], outs[1][0])
    assert np.array_equal(outs[0][1], outs[1][1])
