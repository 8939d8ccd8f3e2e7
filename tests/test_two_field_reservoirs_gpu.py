"""Two-field reservoirs on the GPU: double (n_A, n_I) and quadratic-double (n_R, n_I) in the fused
RK4 step (tiled kernel), the split-step column pass (both orderings) and the Lawson IFRK passes.

FP64 against the reference's own rk4-fdm and split-step-fft trajectories
(``polarism/reservoir/double_reservoir.py:106-130``, ``quadratic_double_reservoir.py:13-14``;
fixtures ``rk4_fdm_double``, ``rk4_fdm_quadratic_double``, ``split_cpu_p2_double``,
``split_cpu_p2_quadratic_double``, Wigner noise on) within 1e-10; FP32 within 1e-4 of the FP64
oracle on the same noise realisation; the drop-in ``rk4-cuda`` class on a host-mirror config.
"""
from __future__ import annotations

import numpy as np
import pytest

from oracle import gpe
from tests.conftest import load_golden, rel_l2

pytestmark = pytest.mark.gpu

CASES = [("rk4_fdm_double", "double"), ("rk4_fdm_quadratic_double", "quadratic-double")]


def _engine(g, precision, kind):
    from polarism_gb300.engine import MemberPhysics, RK4Engine

    p = g["physics"]
    ny, nx = g["psi0"].shape[-2:]
    eng = RK4Engine(nx, ny, 1, float(g["dx"]), float(g["dy"]), float(g["dt"]),
                    MemberPhysics.from_object(p), precision, reservoir=kind)
    eng.set_pump(g["envelope"].astype(eng.real))
    dv = float(g["dx"]) * float(g["dy"])
    eng.set_noise([int(g["seed"])], p["gamma_C"], p["R"], 1.0, float(g["dt"]) / (4 * dv))
    eng.set_state(g["psi0"].astype(eng.complex), np.ascontiguousarray(g["res0"], dtype=eng.real))
    return eng


@pytest.mark.parametrize("case,kind", CASES)
def test_fp64_matches_reference_rk4_fdm(cuda_lib, case, kind):
    g = load_golden(case)
    eng = _engine(g, "double", kind)
    norms = []
    for k in range(int(g["steps"])):
        eng.advance(k, 1, np.full((1, 3, 1), float(g["p0"])), use_graphs=False)
        psi, res = eng.get_state()
        norms.append(gpe.norm(psi, float(g["dx"]), float(g["dy"]))[0])
    assert rel_l2(psi, g["psi"]) < 1e-10
    for q in range(2):
        assert rel_l2(res[q], g["res"][q]) < 1e-10, q
    assert rel_l2(np.asarray(norms), g["norms"]) < 1e-10
    eng.close()


@pytest.mark.parametrize("case,kind", CASES)
def test_fp32_within_1e4_of_fp64_oracle(cuda_lib, case, kind):
    g = load_golden(case)
    steps = int(g["steps"])
    eng = _engine(g, "single", kind)
    eng.advance(0, steps, np.full((steps, 3, 1), float(g["p0"])))
    psi, res = eng.get_state()
    p = g["physics"]
    dx, dy, dt = float(g["dx"]), float(g["dy"]), float(g["dt"])
    noise = gpe.Noise([int(g["seed"])], [p["gamma_C"]], [p["R"]], [1.0], dt, dx * dy, "double",
                      normals_precision="single")
    pump = g["envelope"] * float(g["p0"])
    psi_o, f_o = gpe.rk4_advance(g["psi0"].copy(), tuple(g["res0"]), lambda t: pump, 0.0, p, dx, dy, dt, 0,
                                 steps, kind=kind, noise=noise)
    assert rel_l2(psi, psi_o) < 1e-4
    for q in range(2):
        assert rel_l2(res[q], f_o[q]) < 1e-4, q
    eng.close()


@pytest.mark.parametrize("kind", ["double", "quadratic-double"])
def test_split_cpu_ordering_matches_reference_output(cuda_lib, kind):
    """The reference's own split-step-fft trajectory (FP64, Wigner on, 32x16)."""
    from polarism_gb300.engine import MemberPhysics, RK4Engine

    g = load_golden("split_cpu_p2_" + kind.replace("-", "_"))
    p = g["physics"]
    ny, nx = g["psi0"].shape[-2:]
    dx, dy, dt = float(g["dx"]), float(g["dy"]), float(g["dt"])
    eng = RK4Engine(nx, ny, 1, dx, dy, dt, MemberPhysics.from_object(p), "double", reservoir=kind)
    eng.set_pump(g["envelope"])
    eng.set_noise([int(g["seed"])], p["gamma_C"], p["R"], 1.0, dt / (4 * dx * dy))
    eng.set_state(g["psi0"], np.ascontiguousarray(g["res0"]))
    norms = []
    for k in range(int(g["steps"])):
        eng.split_advance(0, k, 1, np.full((1, 2, 1), float(g["p0"])), use_graphs=False)
        psi, res = eng.get_state()
        norms.append(gpe.norm(psi, dx, dy)[0])
    assert rel_l2(psi, g["psi"]) < 1e-10
    for q in range(2):
        assert rel_l2(res[q], g["res"][q]) < 1e-10, q
    assert rel_l2(np.asarray(norms), g["norms"]) < 1e-10
    eng.close()


@pytest.mark.parametrize("kind", ["double", "quadratic-double"])
@pytest.mark.parametrize("ordering", ["cpu", "kouter"])
@pytest.mark.parametrize("precision,tol", [("double", 1e-10), ("single", 1e-4)])
def test_split_orderings_match_oracle(cuda_lib, kind, ordering, precision, tol):
    """Both orderings with graphs, a pulsed pump and noise against the FP64 oracle."""
    from polarism_gb300.engine import MemberPhysics, RK4Engine

    g = load_golden("split_cpu_p2_" + kind.replace("-", "_"))
    p = g["physics"]
    ny, nx = g["psi0"].shape[-2:]
    dx, dy, dt = float(g["dx"]), float(g["dy"]), float(g["dt"])
    steps = 10

    def coeff(t):
        return float(g["p0"]) * (1.0 + 0.5 * np.sin(40.0 * t))

    eng = RK4Engine(nx, ny, 1, dx, dy, dt, MemberPhysics.from_object(p), precision, reservoir=kind)
    eng.set_pump(g["envelope"].astype(eng.real))
    eng.set_noise([int(g["seed"])], p["gamma_C"], p["R"], 1.0, dt / (4 * dx * dy))
    eng.set_state(g["psi0"].astype(eng.complex), np.ascontiguousarray(g["res0"], dtype=eng.real))
    scales = np.asarray([[[coeff(k * dt + dt / 4)], [coeff(k * dt + 3 * dt / 4)]] for k in range(steps)])
    eng.split_advance(0 if ordering == "cpu" else 1, 0, steps, scales)
    psi, res = eng.get_state()
    if ordering == "kouter":
        psi = np.fft.ifft2(psi.astype(np.complex128), axes=(-2, -1))
    noise = gpe.Noise([int(g["seed"])], [p["gamma_C"]], [p["R"]], [1.0], dt, dx * dy, "double",
                      normals_precision=precision)
    psi_o, f_o = gpe.split_advance(ordering, g["psi0"].copy(), tuple(g["res0"]),
                                   lambda t: g["envelope"] * coeff(t), 0.0, p, g["k_squared"], dx, dy,
                                   dt, 0, steps, kind=kind, noise=noise)
    assert rel_l2(psi, psi_o) < tol
    for q in range(2):
        assert rel_l2(res[q], f_o[q]) < tol, q
    eng.close()


@pytest.mark.parametrize("kind", ["double", "quadratic-double"])
def test_ifrk_two_field_reservoirs_match_oracle(cuda_lib, kind):
    """The Lawson DP5 passes with the two-field reservoirs (power-of-two grid, the fixtures'
    physics), three fixed steps against the FP64 oracle."""
    from polarism_gb300.engine import MemberPhysics, RK4Engine

    p = load_golden("rk4_fdm_" + kind.replace("-", "_"))["physics"]
    ny, nx, dx, dy, dt = 16, 32, 1.0, 1.25, 0.01
    rng = np.random.default_rng(8)
    psi0 = 0.2 * (rng.standard_normal((1, 1, ny, nx)) + 1j * rng.standard_normal((1, 1, ny, nx)))
    res0 = np.abs(rng.standard_normal((2, 1, 1, ny, nx))) * 0.5
    x = (np.arange(nx) - nx / 2) * dx
    y = (np.arange(ny) - ny / 2) * dy
    env = np.exp(-0.5 * (x[None, :] ** 2 + y[:, None] ** 2) / 25.0)
    kx = 2 * np.pi * np.fft.fftfreq(nx, d=dx)
    ky = 2 * np.pi * np.fft.fftfreq(ny, d=dy)
    k2 = kx[None, :] ** 2 + ky[:, None] ** 2
    eng = RK4Engine(nx, ny, 1, dx, dy, dt, MemberPhysics.from_object(p), "double", reservoir=kind)
    eng.set_pump(env)
    eng.set_state(psi0, res0)
    eng.ifrk_advance("dp5", 0, 3, np.full((3, 7, 1), 2.0))
    psi, res = eng.get_state()
    state = gpe.IFRKState(psi=psi0.copy(), fields=tuple(res0))
    for _ in range(3):
        gpe.ifrk_step(state, dt, gpe.DP5_TABLEAU, lambda t: env * 2.0, 0.0, p, k2, dx, dy, kind=kind)
    assert rel_l2(psi, state.real_space()) < 1e-10
    for q in range(2):
        assert rel_l2(res[q], state.fields[q]) < 1e-10, q
    eng.close()


@pytest.mark.parametrize("method", ["rk4-cuda", "split-step-fft-cuda"])
@pytest.mark.parametrize("kind", ["double", "quadratic-double"])
def test_drop_in_solvers_two_field_reservoirs(cuda_lib, method, kind):
    """The reference-facing classes on a host-mirror config: state in, ten steps, both reservoir
    fields written back in the reservoir's own (active, inactive) order."""
    from polarism_gb300 import host
    from polarism_gb300.solvers import RK4CudaSolver, SplitStepFFTCudaSolver

    cfg = host.Config()
    cfg.grid.nx, cfg.grid.ny, cfg.grid.lx, cfg.grid.ly = 64, 32, 64.0, 32.0
    cfg.solver.precision, cfg.solver.dt = "double", 2e-3
    cfg.reservoir.reservoir_type = kind
    cfg.laser.P0, cfg.laser.sigma_space = 0.3, 8.0
    cfg.noise.seed = 5
    grid, model, state = host.build_simulation(cfg)
    psi0 = state.field.copy()
    cls = RK4CudaSolver if method == "rk4-cuda" else SplitStepFFTCudaSolver
    solver = cls(cfg, grid, model)
    solver.advance(model, state, 10)
    n_a, n_i = model.reservoir.get_state()
    p = {k: getattr(cfg.physics, k) for k in ("hbar", "m_eff", "g_C", "g_R", "g_I", "R", "gamma_C",
                                              "gamma_R", "gamma_I", "gamma_A", "R_IA", "R_AI",
                                              "kappa")}
    pump = model.pump.lasers[0]._spatial_envelope * cfg.laser.P0
    zeros = (np.zeros_like(n_a), np.zeros_like(n_i))
    if method == "rk4-cuda":
        psi_o, f_o = gpe.rk4_advance(psi0, zeros, lambda t: pump, 0.0, p, grid.dx, grid.dy,
                                     cfg.solver.dt, 0, 10, kind=kind)
    else:
        kx = 2 * np.pi * np.fft.fftfreq(grid.nx, d=grid.dx)
        ky = 2 * np.pi * np.fft.fftfreq(grid.ny, d=grid.dy)
        psi_o, f_o = gpe.split_advance("kouter", psi0, zeros, lambda t: pump, 0.0, p,
                                       kx[None, :] ** 2 + ky[:, None] ** 2, grid.dx, grid.dy,
                                       cfg.solver.dt, 0, 10, kind=kind)
    assert state.step == 10
    assert rel_l2(state.field, psi_o) < 1e-10
    assert rel_l2(n_a, f_o[0]) < 1e-10 and rel_l2(n_i, f_o[1]) < 1e-10
