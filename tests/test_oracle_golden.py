"""Pin the CPU oracle against the reference's own outputs and known-answer vectors.

Reference tests mirrored here: ``tests/unit/test_noise.py:56-85`` (Random123
vectors, counter stream), ``tests/unit/test_ifrk_reference.py:13-21`` (IFRK4
goldens at 1e-12 / 1e-5), ``tests/crosscheck/test_split_step_fft_cuda.py:46-70``
(the GPU ordering's NumPy composition), ``tests/unit/test_adaptive_dt.py:14-83``
(the DP5 analytic uniform decay).
"""
from __future__ import annotations

import numpy as np
import pytest

from oracle import gpe
from oracle.philox import counter_words, normal_pair, philox4x32, wigner_increment
from tests.conftest import rel_l2


def test_philox_random123_vectors(golden):
    g = golden("philox")
    for key, ctr, exp in zip(g["kat_keys"], g["kat_counters"], g["kat_expected"]):
        assert np.array_equal(philox4x32(ctr, int(key)), exp)


def test_philox_batch_words_bit_exact(golden):
    g = golden("philox")
    words = philox4x32(counter_words(np.arange(4096), int(g["batch_step"])), int(g["batch_key"]))
    assert words.dtype == np.uint32
    assert np.array_equal(words, g["batch_words"])


def test_philox_step_and_stream_change_words():
    cells = np.arange(1024)
    first = philox4x32(counter_words(cells, 0), 42)
    assert not np.array_equal(first, philox4x32(counter_words(cells, 1), 42))
    assert not np.array_equal(first, philox4x32(counter_words(cells, 0, 2), 42))


@pytest.mark.parametrize("precision", ["single", "double"])
def test_normals_match_reference(golden, precision):
    g = golden("philox")
    re, im = normal_pair(g["batch_words"], precision)
    ref = g[f"normals_{precision}"]
    assert np.array_equal(re, ref[0]) and np.array_equal(im, ref[1])


@pytest.mark.parametrize("precision", ["single", "double"])
def test_wigner_increment_matches_reference(golden, precision):
    g = golden("wigner")
    field = g[f"{precision}_before"].copy()
    wigner_increment(field, g[f"{precision}_active"], int(g["step"]), g["seeds"], g["gamma"],
                     g["R"], g["strength"], float(g["dt"]), float(g["cell_volume"]), precision)
    tol = 2e-6 if precision == "single" else 2e-14
    np.testing.assert_allclose(field, g[f"{precision}_after"], rtol=tol, atol=tol)


def _trajectory(g, method, normals=None):
    p = g["physics"]
    pump = g["envelope"] * g["p0"]
    dx, dy, dt = float(g["dx"]), float(g["dy"]), float(g["dt"])
    noise = None
    if bool(g["wigner"]):
        noise = gpe.Noise([int(g["seed"])], [p["gamma_C"]], [p["R"]], [1.0], dt, dx * dy,
                          "double", normals)
    psi, fields = g["psi0"].copy(), tuple(g["res0"])
    norms = []
    kind = str(g["reservoir"])
    if method == "rk4":
        psi, fields = gpe.rk4_advance(psi, fields, lambda t: pump, 0.0, p, dx, dy, dt, 0,
                                      int(g["steps"]), noise=noise, norm_trace=norms, kind=kind)
    else:
        psi, fields = gpe.split_advance("cpu", psi, fields, lambda t: pump, 0.0, p, g["k_squared"],
                                        dx, dy, dt, 0, int(g["steps"]), noise=noise,
                                        norm_trace=norms, kind=kind)
    return psi, fields, np.asarray(norms).ravel()


@pytest.mark.parametrize("case,method", [("rk4_fdm", "rk4"), ("rk4_fdm_quiet", "rk4"),
                                         ("split_cpu", "split"), ("rk4_fdm_double", "rk4"),
                                         ("rk4_fdm_quadratic_double", "rk4"),
                                         ("split_cpu_p2_double", "split"),
                                         ("split_cpu_p2_quadratic_double", "split")])
def test_fp64_trajectories_match_reference(golden, case, method):
    g = golden(case)
    psi, fields, norms = _trajectory(g, method)
    assert rel_l2(psi, g["psi"]) < 1e-12
    for q in range(len(fields)):
        assert rel_l2(fields[q], g["res"][q]) < 1e-12, q
    assert rel_l2(norms, g["norms"]) < 1e-12


def test_kouter_ordering_matches_reference_composition(golden):
    g = golden("split_kouter")
    p = g["physics"]
    pumps = g["pumps"]
    psi, fields = g["psi0"].copy(), (g["res0"][0],)
    for k in range(3):
        calls = iter([pumps[2 * k], pumps[2 * k + 1]])
        psi, fields = gpe.split_step_kouter(
            psi, fields, lambda t: next(calls), g["potential"], p, g["k_squared"],
            float(g["dx"]), float(g["dy"]), float(g["dt"]), 0.0, k)
    assert rel_l2(psi, g["psi"]) < 1e-12
    assert rel_l2(fields[0], g["res"][0]) < 1e-12


@pytest.mark.parametrize("precision", ["double", "single"])
@pytest.mark.parametrize("eta", ["0", "0.04"])
def test_ifrk4_matches_reference_golden(golden, precision, eta):
    g = golden("ifrk4")
    key = f"{precision}_single_eta{eta}"
    p = g[key + "_physics"]
    times = list(g[key + "_pump_times"])
    pumps = g[key + "_pumps"]

    def pump_at(t):
        return pumps[int(np.argmin(np.abs(np.asarray(times) - t)))]

    state = gpe.IFRKState(psi=g[key + "_psi0"].astype(np.complex128),
                          fields=tuple(g[key + "_res0"].astype(np.float64)))
    for _ in range(5):
        gpe.ifrk_step(state, 0.007, gpe.RK4_TABLEAU, pump_at,
                      g[key + "_potential"].astype(np.complex128), p, g[key + "_k_squared"],
                      float(g[key + "_dx"]), float(g[key + "_dy"]))
    psi = state.real_space()[0, 0]
    tol = 1e-5 if precision == "single" else 1e-12
    ref = g[key + "_psi"]
    np.testing.assert_allclose(psi, ref, rtol=tol, atol=tol * max(1e-3, np.max(abs(ref))))
    np.testing.assert_allclose(state.fields[0][0, 0], g[key + "_res"], rtol=tol, atol=tol)


def test_dp5_adaptive_matches_reference(golden):
    g = golden("dp5")
    p = g["physics"]
    pump = g["envelope"] * g["p0"]
    dx, dy = float(g["dx"]), float(g["dy"])
    state = gpe.IFRKState(psi=g["psi0"].copy(), fields=tuple(g["res0"]))
    control = gpe.StepControl(float(g["dt"]), None, 5, 4)

    def trial(st, h):
        return gpe.ifrk_step(st, h, gpe.DP5_TABLEAU, lambda t: pump, 0.0, p, g["k_squared"],
                             dx, dy, adaptive=True, rtol=float(g["rtol"]), atol=float(g["atol"]))

    gpe.ifrk_adaptive_advance(state, control, trial, int(g["ticks"]) * float(g["dt"]))
    assert control.accepted == int(g["accepted"])
    assert control.rejected == int(g["rejected"])
    assert rel_l2(state.real_space(), g["psi"]) < 1e-12
    assert rel_l2(state.fields[0], g["res"][0]) < 1e-12


@pytest.mark.parametrize("case", ["spinor_dp5", "spinor_dp5_shared", "spinor_rk4_wigner"])
def test_spinor_ifrk_matches_reference(golden, case):
    """Two-component Lawson steps (matrix exponential, TE-TM, Zeeman, cross-spin term, double or
    shared reservoir, ring pump, pump weights) against the reference's generic path."""
    g = golden(case)
    p = g["physics"]
    pump = g["envelope"] * g["p0"]
    dx, dy, dt = float(g["dx"]), float(g["dy"]), float(g["dt"])
    kind = str(g["reservoir"])
    spin = {"kx": g["kx"], "ky": g["ky"], "weights": g["weights"]}
    state = gpe.IFRKState(psi=g["psi0"].copy(), fields=tuple(g["res0"]))
    if bool(g["adaptive"]):
        control = gpe.StepControl(dt, None, 5, 4)

        def trial(st, h):
            return gpe.ifrk_step(st, h, gpe.DP5_TABLEAU, lambda t: pump, 0.0, p, g["k_squared"], dx,
                                 dy, kind=kind, adaptive=True, rtol=float(g["rtol"]),
                                 atol=float(g["atol"]), spinor=spin)

        gpe.ifrk_adaptive_advance(state, control, trial, int(g["ticks"]) * dt)
        assert control.accepted == int(g["accepted"])
        assert control.rejected == int(g["rejected"])
    else:
        noise = gpe.Noise([int(g["seed"])], [p["gamma_C"]], [p["R"]], [1.0], dt, dx * dy, "double")
        for step in range(int(g["ticks"])):
            gpe.ifrk_step(state, dt, gpe.TABLEAUS[str(g["tableau"])], lambda t: pump, 0.0, p,
                          g["k_squared"], dx, dy, kind=kind, spinor=spin)
            state.psi, state.psi_k = state.real_space(), None
            if bool(g["wigner"]):
                noise.apply(state.psi, state.fields[0], step)
    assert rel_l2(state.real_space(), g["psi"]) < 1e-12
    for q in range(len(g["res"])):
        assert rel_l2(state.fields[q], g["res"][q]) < 1e-12


def test_dp5_uniform_decay_known_answer():
    """Uniform nonlinear decay psi(t) = exp(-gamma t/2 + i phi(t)) (analytic)."""
    p = dict(hbar=0.6582119514, m_eff=0.284, g_C=2.0, gamma_C=0.7)
    n = 4
    k2 = np.zeros((n, n))
    for rtol in (1e-6, 1e-9):
        state = gpe.IFRKState(psi=np.ones((1, 1, n, n), dtype=complex), fields=())
        control = gpe.StepControl(1.0, None, 5, 4)

        def trial(st, h):
            return gpe.ifrk_step(st, h, gpe.DP5_TABLEAU, lambda t: 0.0, 0.0, p, k2, 1.0, 1.0,
                                 kind="none", adaptive=True, rtol=rtol, atol=rtol * 0.01)

        gpe.ifrk_adaptive_advance(state, control, trial, 2.0)
        t, gamma = 2.0, p["gamma_C"]
        phase = -p["g_C"] / (p["hbar"] * gamma) * (1 - np.exp(-gamma * t))
        exact = np.exp(-gamma * t / 2 + 1j * phase)
        assert np.max(np.abs(state.real_space() - exact)) <= 50 * rtol


def test_config1_smoke_values():
    """Reference config 1 at 0.2 ps (200 steps of rk4-fdm, 128^2, seed 0)."""
    from polarism_gb300.host import Config, build_simulation

    cfg = Config()
    cfg.grid.nx = cfg.grid.ny = 128
    cfg.grid.lx = cfg.grid.ly = 100.0
    cfg.laser.P0, cfg.laser.sigma_space = 0.02, 12.0
    cfg.solver.dt, cfg.noise.seed = 1e-3, 0
    grid, model, state = build_simulation(cfg)
    env = model.pump.separable_term()[0] * cfg.laser.P0
    p = {k: getattr(cfg.physics, k) for k in ("hbar", "m_eff", "g_C", "g_R", "g_I", "R",
                                               "gamma_C", "gamma_R")}
    psi, fields = gpe.rk4_advance(state.field, (model.reservoir.get_state()[0],), lambda t: env,
                                  0.0, p, grid.dx, grid.dy, cfg.solver.dt, 0, 200)
    norm = float(gpe.norm(psi, grid.dx, grid.dy)[0])
    assert abs(norm - 0.009835377212841102) < 1e-12
    assert abs(float(fields[0].max()) - 0.003993766474840784) < 1e-12


def two_laser_pump(g):
    """P(t) = E_0 c_0(t) + E_1 c_1(t) from the fixture's recorded stage coefficients, keyed by
    quarter steps (the RK4 and split-step stage times are multiples of dt / 4)."""
    dt = float(g["dt"])
    table = {}
    for k in range(int(g["steps"])):
        for s, node in enumerate(g["nodes"]):
            table[int(round(4 * (k + node)))] = g["coefficients"][k, s]
    env = g["envelopes"]

    def pump_at(t):
        c = table[int(round(4 * t / dt))]
        return env[0] * c[0] + env[1] * c[1]
    return pump_at


@pytest.mark.parametrize("case", ["rk4_fdm_two_lasers", "split_cpu_two_lasers"])
def test_two_laser_trajectories_match_reference(golden, case):
    g = golden(case)
    p = g["physics"]
    dx, dy, dt = float(g["dx"]), float(g["dy"]), float(g["dt"])
    noise = gpe.Noise([int(g["seed"])], [p["gamma_C"]], [p["R"]], [1.0], dt, dx * dy, "double")
    norms = []
    if case.startswith("rk4"):
        psi, fields = gpe.rk4_advance(g["psi0"].copy(), tuple(g["res0"]), two_laser_pump(g), 0.0, p,
                                      dx, dy, dt, 0, int(g["steps"]), noise=noise, norm_trace=norms)
    else:
        psi, fields = gpe.split_advance("cpu", g["psi0"].copy(), tuple(g["res0"]), two_laser_pump(g),
                                        0.0, p, g["k_squared"], dx, dy, dt, 0, int(g["steps"]),
                                        noise=noise, norm_trace=norms)
    assert rel_l2(psi, g["psi"]) < 1e-12
    assert rel_l2(fields[0], g["res"][0]) < 1e-12
    assert rel_l2(np.asarray(norms).ravel(), g["norms"]) < 1e-12
