"""Several separable lasers on the GPU: P(x, t) = sum_l c_l(t) E_l(x) summed per site inside the
RK4, split-step and IFRK kernels (``polarism/laser/pump_field.py:81-89`` with the combiner of
``polarism/solver/cuda_pump.py:7-19``: products and partial sums rounded separately).

FP64 against the reference's own trajectories with a continuous Gaussian plus a pulsed Gaussian
(fixtures ``rk4_fdm_two_lasers`` and ``split_cpu_two_lasers``, Wigner noise on, 1e-10); FP32 and
the other orderings against the FP64 oracle (1e-4 / 1e-10); per-member envelopes.
"""
from __future__ import annotations

import numpy as np
import pytest

from oracle import gpe
from tests.conftest import load_golden, rel_l2
from tests.test_oracle_golden import two_laser_pump

pytestmark = pytest.mark.gpu


def _engine(g, precision, members=1, **kw):
    from polarism_gb300.engine import MemberPhysics, RK4Engine

    p = g["physics"]
    ny, nx = g["psi0"].shape[-2:]
    eng = RK4Engine(nx, ny, members, float(g["dx"]), float(g["dy"]), float(g["dt"]),
                    MemberPhysics.from_object(p), precision, pump_terms=2, **kw)
    eng.set_pump(np.ascontiguousarray(g["envelopes"], dtype=eng.real))
    dv = float(g["dx"]) * float(g["dy"])
    eng.set_noise([int(g["seed"])] * members, p["gamma_C"], p["R"], 1.0, float(g["dt"]) / (4 * dv))
    eng.set_state(np.repeat(g["psi0"], members, 0).astype(eng.complex),
                  np.repeat(g["res0"][0], members, 0).astype(eng.real))
    return eng


@pytest.mark.parametrize("case", ["rk4_fdm_two_lasers", "split_cpu_two_lasers"])
def test_fp64_matches_reference_trajectory(cuda_lib, case):
    g = load_golden(case)
    eng = _engine(g, "double")
    norms = []
    for k in range(int(g["steps"])):
        coeffs = g["coefficients"][k:k + 1, :, :, None]  # (1, samples, L, members)
        if case.startswith("rk4"):
            eng.advance(k, 1, coeffs, use_graphs=False)
        else:
            eng.split_advance(0, k, 1, coeffs, use_graphs=False)
        psi, res = eng.get_state()
        norms.append(gpe.norm(psi, float(g["dx"]), float(g["dy"]))[0])
    assert rel_l2(psi, g["psi"]) < 1e-10
    assert rel_l2(res, g["res"][0]) < 1e-10
    assert rel_l2(np.asarray(norms), g["norms"]) < 1e-10
    eng.close()


def test_fp32_rk4_within_1e4_of_fp64_oracle(cuda_lib):
    g = load_golden("rk4_fdm_two_lasers")
    steps = int(g["steps"])
    eng = _engine(g, "single")
    eng.advance(0, steps, g["coefficients"][:, :, :, None])
    psi, res = eng.get_state()
    p = g["physics"]
    dx, dy, dt = float(g["dx"]), float(g["dy"]), float(g["dt"])
    noise = gpe.Noise([int(g["seed"])], [p["gamma_C"]], [p["R"]], [1.0], dt, dx * dy, "double",
                      normals_precision="single")
    psi_o, f_o = gpe.rk4_advance(g["psi0"].copy(), tuple(g["res0"]), two_laser_pump(g), 0.0, p, dx,
                                 dy, dt, 0, steps, noise=noise)
    assert rel_l2(psi, psi_o) < 1e-4 and rel_l2(res, f_o[0]) < 1e-4
    eng.close()


def _synthetic(t):
    return np.array([0.3, 0.2 + 0.1 * np.sin(50.0 * t)])


@pytest.mark.parametrize("precision,tol", [("double", 1e-10), ("single", 1e-4)])
def test_kouter_split_and_members(cuda_lib, precision, tol):
    """GPU ordering with two members whose second envelopes differ (per-member envelopes)."""
    g = load_golden("split_cpu_two_lasers")
    p = g["physics"]
    dx, dy, dt = float(g["dx"]), float(g["dy"]), float(g["dt"])
    env = np.stack([g["envelopes"][0], g["envelopes"][1]])        # (L, ny, nx)
    env_m = np.stack([env, np.stack([env[0], np.roll(env[1], 5, axis=1)])], axis=1)  # (L, B, ny, nx)
    from polarism_gb300.engine import MemberPhysics, RK4Engine

    ny, nx = env.shape[-2:]
    eng = RK4Engine(nx, ny, 2, dx, dy, dt, MemberPhysics.from_object(p), precision, pump_terms=2,
                    pump_per_member=True)
    eng.set_pump(np.ascontiguousarray(env_m, dtype=eng.real))
    eng.set_noise([3, 4], p["gamma_C"], p["R"], 1.0, dt / (4 * dx * dy))
    psi0 = np.repeat(g["psi0"], 2, 0)
    n0 = np.repeat(g["res0"][0], 2, 0)
    eng.set_state(psi0.astype(eng.complex), n0.astype(eng.real))
    steps = 12
    half = np.asarray([[_synthetic(k * dt + dt / 4), _synthetic(k * dt + 3 * dt / 4)] for k in range(steps)])
    eng.split_advance(1, 0, steps, half[..., None])
    psi = np.fft.ifft2(eng.get_state()[0].astype(np.complex128), axes=(-2, -1))
    res = eng.get_state()[1]
    noise = gpe.Noise([3, 4], [p["gamma_C"]] * 2, [p["R"]] * 2, [1.0] * 2, dt, dx * dy, "double",
                      normals_precision=precision)

    def pump_at(t):
        c = _synthetic(t)
        return (env_m[0] * c[0] + env_m[1] * c[1])[:, None]

    psi_o, f_o = gpe.split_advance("kouter", psi0.copy(), (n0.copy(),), pump_at, 0.0, p, g["k_squared"],
                                   dx, dy, dt, 0, steps, noise=noise)
    assert rel_l2(psi, psi_o) < tol and rel_l2(res, f_o[0]) < tol
    eng.close()


def test_ifrk_dp5_with_two_lasers(cuda_lib):
    from polarism_gb300.engine import TABLEAU_NODES, MemberPhysics, RK4Engine

    g = load_golden("split_cpu_two_lasers")
    p = g["physics"]
    dx, dy, dt = float(g["dx"]), float(g["dy"]), 0.01
    ny, nx = g["psi0"].shape[-2:]
    eng = RK4Engine(nx, ny, 1, dx, dy, dt, MemberPhysics.from_object(p), "double", pump_terms=2)
    eng.set_pump(np.ascontiguousarray(g["envelopes"]))
    eng.set_state(g["psi0"], g["res0"][0])
    steps = 4
    nodes = TABLEAU_NODES["dp5"]
    scales = np.asarray([[_synthetic(k * dt + c * dt) for c in nodes] for k in range(steps)])
    eng.ifrk_advance("dp5", 0, steps, scales[..., None])
    psi, res = eng.get_state()
    env = g["envelopes"]
    state = gpe.IFRKState(psi=g["psi0"].copy(), fields=(g["res0"][0].copy(),))
    for _ in range(steps):
        gpe.ifrk_step(state, dt, gpe.DP5_TABLEAU,
                      lambda t: env[0] * _synthetic(t)[0] + env[1] * _synthetic(t)[1], 0.0, p,
                      g["k_squared"], dx, dy)
    assert rel_l2(psi, state.real_space()) < 1e-10 and rel_l2(res, state.fields[0]) < 1e-10
    eng.close()


@pytest.mark.parametrize("method", ["rk4-cuda", "split-step-fft", "ifrk-fft-cuda"])
def test_drop_in_solvers_with_a_pulse_train_and_a_cw_spot(cuda_lib, method):
    """Host-mirror configs in laser mode "multiple" (a CW spot and a pulse train whose timing
    differs per member) through the reference-facing classes, against the FP64 oracle."""
    import copy

    from polarism_gb300 import host
    from polarism_gb300.solvers import IFRKFFTCudaSolver, RK4CudaSolver, SplitStepFFTSolver

    cfg = host.Config()
    cfg.grid.nx, cfg.grid.ny, cfg.grid.lx, cfg.grid.ly = 32, 16, 40.0, 20.0
    cfg.solver.precision, cfg.solver.dt = "double", 2e-3
    cfg.noise.seed = 11
    cw = host.LaserParameters(laser_type="continuous-gaussian", P0=0.05, sigma_space=8.0)
    pulse = host.LaserParameters(laser_type="pulse-gaussian", P0=0.3, Pmax=0.5, x0=5.0, y0=-2.0,
                                 sigma_space=4.0, sigma_time=0.0043, cutoff_sigma=3.0,
                                 pulse_separation=0.0217, n_pulses=3)
    # Pulse edges (cut at 3 sigma) fall between stage times, so the oracle's accumulated time
    # and the solver's step-indexed time sit on the same side of every cut.
    cfg.laser.mode, cfg.laser.lasers = "multiple", [cw, pulse]
    members = []
    for m in range(2):
        c = copy.deepcopy(cfg)
        c.noise.seed = 11 + m
        c.laser.lasers[1].delay = 0.0007 + 0.0031 * m
        members.append(c)
    grid, model, state = host.build_simulation(cfg, members=members)
    psi0 = state.field.copy()
    n0 = model.reservoir.get_state()[0].copy()
    cls = {"rk4-cuda": RK4CudaSolver, "split-step-fft": SplitStepFFTSolver,
           "ifrk-fft-cuda": IFRKFFTCudaSolver}[method]
    solver = cls(members[0], grid, model)
    steps = 25
    solver.advance(model, state, steps)
    terms = model.pump.separable_terms()
    assert len(terms) == 2

    def pump_at(t):
        total = 0
        for env, coeff in terms:
            total = total + np.asarray(env) * np.asarray(coeff(t), dtype=np.float64).reshape(-1, 1, 1, 1)
        return total

    p = {k: getattr(cfg.physics, k) for k in ("hbar", "m_eff", "g_C", "g_R", "g_I", "R", "gamma_C",
                                              "gamma_R")}
    dt = cfg.solver.dt
    if method == "rk4-cuda":
        psi_o, f_o = gpe.rk4_advance(psi0, (n0,), pump_at, 0.0, p, grid.dx, grid.dy, dt, 0, steps)
    elif method == "split-step-fft":
        psi_o, f_o = gpe.split_advance("cpu", psi0, (n0,), pump_at, 0.0, p, grid.k_squared, grid.dx,
                                       grid.dy, dt, 0, steps)
    else:
        st = gpe.IFRKState(psi=psi0, fields=(n0,))
        for _ in range(steps):
            gpe.ifrk_step(st, dt, gpe.TABLEAUS[solver.tableau],
                          pump_at, 0.0, p, grid.k_squared, grid.dx, grid.dy)
        psi_o, f_o = st.real_space(), st.fields
    assert rel_l2(state.field, psi_o) < 1e-10
    assert rel_l2(model.reservoir.get_state()[0], f_o[0]) < 1e-10


@pytest.mark.parametrize("nx,ny,members", [(256, 24, 2), (1024, 12, 2)])
def test_two_lasers_on_the_full_width_kernel(cuda_lib, nx, ny, members):
    """Two lasers streamed as extra ring rows of the full-width kernel (kind 2): against the
    tiled kernel (1e-5) and the FP64 oracle (1e-4), per-member envelopes, time-dependent
    coefficients at every half step, Wigner noise on."""
    from polarism_gb300.engine import MemberPhysics, RK4Engine

    rng = np.random.default_rng(nx + 3 * ny)
    p = dict(hbar=0.6582119514, m_eff=0.284, g_C=0.001, g_R=0.002, g_I=0.0, R=0.02,
             gamma_C=0.083, gamma_R=0.005)
    dx, dy, dt, steps = 0.45, 0.55, 1e-3, 9
    psi0 = 0.05 * (rng.standard_normal((members, 1, ny, nx))
                   + 1j * rng.standard_normal((members, 1, ny, nx)))
    res0 = np.abs(rng.standard_normal((members, 1, ny, nx))) * 0.02
    env = np.abs(rng.standard_normal((2, members, 1, ny, nx)))  # [laser][member]
    seeds = [21 + m for m in range(members)]
    samples = 0.02 + 0.01 * rng.random((2 * steps + 1, 2, members))  # [half step][laser][member]
    scales = np.stack([samples[2 * k:2 * k + 3] for k in range(steps)])  # (steps, 3, 2, members)
    outs = {}
    for kernel in (1, 2):
        eng = RK4Engine(nx, ny, members, dx, dy, dt, MemberPhysics(**p), "single",
                        pump_per_member=True, pump_terms=2)
        eng.set_kernel(kernel)
        assert eng.kernel() == kernel
        eng.set_pump(env.astype(np.float32))
        eng.set_noise(seeds, p["gamma_C"], p["R"], 1.0, dt / (4 * dx * dy))
        eng.set_state(psi0.astype(np.complex64), res0.astype(np.float32))
        eng.advance(0, steps, scales)
        outs[kernel] = eng.get_state()
        eng.close()
    assert rel_l2(outs[2][0], outs[1][0]) < 1e-5 and rel_l2(outs[2][1], outs[1][1]) < 1e-5
    nz = gpe.Noise(seeds, [p["gamma_C"]] * members, [p["R"]] * members, [1.0] * members, dt,
                   dx * dy, "double", normals_precision="single")

    def pump_at(t):  # sum over the lasers at the half-step sample of time t
        c = samples[int(round(2 * t / dt))]  # (2, members)
        return sum(c[l][:, None, None, None] * env[l] for l in range(2))

    psi_o, fields = gpe.rk4_advance(psi0.copy(), (res0.copy(),), pump_at, 0.0, p, dx, dy, dt, 0,
                                    steps, noise=nz)
    assert rel_l2(outs[2][0], psi_o) < 1e-4 and rel_l2(outs[2][1], fields[0]) < 1e-4
