"""Two-component Lawson IFRK on the GPU (spinor with TE-TM, Zeeman and cross-spin terms; double
reservoir per component or one shared reservoir), through the C ABI.

Fixtures come from the reference's own generic Lawson path (``polarism/solver/
ifrk_fft_cuda_solver.py:148-293`` with ``polarism/dispersion.py:34-83``, ``polarism/model.py:
129-173``, ``polarism/reservoir/double_reservoir.py:106-130``), the same cases the oracle is pinned
to.  FP64: the final state within 1e-10 relative L2 of the reference and the adaptive DP5 trial
counts equal; FP32: within 1e-4 of the FP64 oracle replaying the same steps (and the same noise
realisation).
"""
from __future__ import annotations

import numpy as np
import pytest

from oracle import gpe
from tests.conftest import load_golden, rel_l2

pytestmark = pytest.mark.gpu

CASES = ["spinor_dp5", "spinor_dp5_shared", "spinor_rk4_wigner"]


def _engine(g, precision):
    from polarism_gb300.engine import Engine, MemberPhysics

    p = g["physics"]
    ny, nx = g["psi0"].shape[-2:]
    res0 = g["res0"]
    kind = str(g["reservoir"])
    phys = MemberPhysics.from_object(p)
    phys.pump_weight_plus, phys.pump_weight_minus = (float(w) for w in g["weights"][0])
    eng = Engine(nx, ny, 1, float(g["dx"]), float(g["dy"]), float(g["dt"]), phys, precision,
                 reservoir=kind, components=2, reservoir_components=res0.shape[2])
    eng.set_pump(g["envelope"].astype(eng.real))
    if bool(g["wigner"]):
        eng.set_noise([int(g["seed"])], p["gamma_C"], p["R"], 1.0,
                      float(g["dt"]) / (4 * float(g["dx"]) * float(g["dy"])))
    res = res0[0] if kind == "single" else res0
    eng.set_state(g["psi0"].astype(eng.complex), np.ascontiguousarray(res, dtype=eng.real))
    return eng


def _run(eng, g):
    """Advance like the reference did; returns the accepted step sizes."""
    from polarism_gb300.engine import TABLEAU_NODES
    from polarism_gb300.step_control import StepController

    dt, ticks, p0 = float(g["dt"]), int(g["ticks"]), float(g["p0"])
    if not bool(g["adaptive"]):
        eng.ifrk_advance(str(g["tableau"]), 0, ticks, np.full((ticks, 4, 1), p0))
        return [dt] * ticks, None
    ctl = StepController(dt)
    t, target, steps = 0.0, ticks * dt, []
    while t < target:
        h, clamped, proposal = ctl.propose(t, target)
        err, acc = eng.ifrk_trial(h, np.full((len(TABLEAU_NODES["dp5"]), 1), p0), float(g["rtol"]),
                                  float(g["atol"]))
        if acc:
            t = target if clamped else t + h
            steps.append(h)
        ctl.update(h, clamped, proposal, acc, err)
    return steps, ctl


def _res_fields(eng, res):
    return (res,) if eng.res_fields == 1 else tuple(res)


@pytest.mark.parametrize("case", CASES)
def test_fp64_matches_reference(cuda_lib, case):
    g = load_golden(case)
    eng = _engine(g, "double")
    _, ctl = _run(eng, g)
    psi, res = eng.get_state()
    if ctl is not None:
        assert (ctl.accepted, ctl.rejected) == (int(g["accepted"]), int(g["rejected"]))
    assert rel_l2(psi, g["psi"]) < 1e-10
    for q, field in enumerate(_res_fields(eng, res)):
        assert rel_l2(field, g["res"][q]) < 1e-10, q
    eng.close()


@pytest.mark.parametrize("case", CASES)
def test_fp32_within_1e4_of_fp64_oracle(cuda_lib, case):
    g = load_golden(case)
    eng = _engine(g, "single")
    steps, _ = _run(eng, g)
    psi, res = eng.get_state()
    p = g["physics"]
    dx, dy = float(g["dx"]), float(g["dy"])
    pump = g["envelope"] * float(g["p0"])
    spin = {"kx": g["kx"], "ky": g["ky"], "weights": g["weights"]}
    tab = gpe.TABLEAUS[str(g["tableau"])]
    state = gpe.IFRKState(psi=g["psi0"].astype(np.complex128), fields=tuple(g["res0"]))
    noise = None
    if bool(g["wigner"]):
        noise = gpe.Noise([int(g["seed"])], [p["gamma_C"]], [p["R"]], [1.0], float(g["dt"]), dx * dy,
                          "double", normals_precision="single")
    for k, h in enumerate(steps):
        gpe.ifrk_step(state, h, tab, lambda t: pump, 0.0, p, g["k_squared"], dx, dy,
                      kind=str(g["reservoir"]), spinor=spin)
        state.psi, state.psi_k = state.real_space(), None
        if noise is not None:
            noise.apply(state.psi, state.fields[0], k)
    assert psi.dtype == np.complex64
    assert rel_l2(psi, state.psi) < 1e-4
    for q, field in enumerate(_res_fields(eng, res)):
        assert rel_l2(field, state.fields[q]) < 1e-4, q
    eng.close()


def test_spinor_observables_sum_components(cuda_lib):
    """Norms and the steady-state density add the two components; the density moments and
    the momentum distribution stay per component (simulation_controller.py:92-103, 710-734;
    results/accumulators.py:95-172)."""
    g = load_golden("spinor_dp5")
    eng = _engine(g, "double")
    psi, _ = eng.get_state()
    cell = float(g["dx"]) * float(g["dy"])
    rho = np.abs(psi) ** 2
    assert np.allclose(eng.norms(), rho.sum(axis=(1, 2, 3)) * cell, rtol=1e-12)
    eng.accumulate(density=True, momentum=True)
    s_rho, n = eng.accumulator_sums("rho")
    s_k, _ = eng.accumulator_sums("k")
    assert n == 1 and s_rho.shape == psi.shape
    assert rel_l2(s_rho, rho) < 1e-14
    assert rel_l2(s_k, np.abs(np.fft.fft2(psi, axes=(-2, -1))) ** 2) < 1e-12
    rd, rn, norms = eng.steady_check()
    assert np.isinf(rd).all()
    _run(eng, g)
    rd, rn, norms1 = eng.steady_check()
    psi1, _ = eng.get_state()
    d0, d1 = rho.sum(axis=1), (np.abs(psi1) ** 2).sum(axis=1)
    expect = np.sqrt(((d1 - d0) ** 2).sum()) / np.sqrt((d0 ** 2).sum())
    assert abs(rd[0] - expect) <= 1e-9 * expect
    eng.close()


def test_drop_in_solver_spinor_double_reservoir_adaptive(cuda_lib):
    """``ifrk-fft-cuda`` drop-in on a two-component config (ring pump, linear polarisation,
    double reservoir per component, adaptive DP5): same trials and state as the FP64 oracle."""
    from polarism_gb300 import host
    from polarism_gb300.solvers import IFRKFFTCudaSolver

    cfg = host.Config()
    cfg.grid.nx, cfg.grid.ny, cfg.grid.lx, cfg.grid.ly = 32, 16, 48.0, 24.0
    cfg.solver.precision, cfg.solver.dt, cfg.solver.tableau = "double", 0.0625, "dp5"
    cfg.solver.adaptive, cfg.solver.rtol, cfg.solver.atol = True, 1e-6, 1e-8
    cfg.reservoir.reservoir_type = "double"
    cfg.physics.spin, cfg.physics.zeeman, cfg.physics.te_tm = "spinor", 0.05, 0.03
    cfg.physics.alpha_2 = -0.1 * cfg.physics.g_C
    cfg.laser.laser_type, cfg.laser.P0 = "profile", 0.3
    cfg.laser.profile = {"type": "ring", "radius": 8.0, "width": 2.0}
    cfg.noise.seed, cfg.noise.initial_amplitude = 3, 0.2
    grid, model, state = host.build_simulation(cfg)
    assert state.field.shape == (1, 2, 16, 32) and model.reservoir.nA.shape == (1, 2, 16, 32)
    psi0 = state.field.copy()
    solver = IFRKFFTCudaSolver(cfg, grid, model)
    solver.advance(model, state, 6)
    n_a, n_i = model.reservoir.get_state()

    p = {k: getattr(cfg.physics, k) for k in ("hbar", "m_eff", "g_C", "g_R", "g_I", "R", "gamma_C",
                                              "gamma_R", "gamma_I", "gamma_A", "R_IA", "R_AI",
                                              "alpha_2", "zeeman", "te_tm")}
    spin = {"kx": grid.KX, "ky": grid.KY, "weights": model.pump_weights.reshape(-1, 2)}
    pump = model.pump.lasers[0]._spatial_envelope * cfg.laser.P0
    ref = gpe.IFRKState(psi=psi0.copy(), fields=(np.zeros_like(n_a), np.zeros_like(n_i)))
    control = gpe.StepControl(cfg.solver.dt, None, 5, 4)

    def trial(st, h):
        return gpe.ifrk_step(st, h, gpe.DP5_TABLEAU, lambda t: pump, 0.0, p, grid.k_squared,
                             grid.dx, grid.dy, kind="double", adaptive=True, rtol=1e-6, atol=1e-8,
                             spinor=spin)

    gpe.ifrk_adaptive_advance(ref, control, trial, 6 * cfg.solver.dt)
    ctl = solver.step_controller
    assert (ctl.accepted, ctl.rejected) == (control.accepted, control.rejected)
    assert state.step == 6 and abs(state.t - 6 * cfg.solver.dt) < 1e-15
    assert rel_l2(state.field, ref.real_space()) < 1e-10
    assert rel_l2(n_a, ref.fields[0]) < 1e-10 and rel_l2(n_i, ref.fields[1]) < 1e-10
