"""GPU parity of the Lawson IFRK passes (fixed step and adaptive Dormand-Prince).

Mirrors ``tests/unit/test_ifrk_reference.py:13-21`` (the reference's IFRK4 trajectories),
``tests/unit/test_ifrk_gpu.py:54-97`` (fused equals generic), and
``tests/unit/test_adaptive_dt.py:14-98`` (uniform-decay known answer within 50 rtol,
rejections and tick landing).  Tolerances: FP64 1e-10 and FP32 1e-4 relative L2 against
the FP64 oracle; adaptive runs reproduce the reference's accepted/rejected trial counts.
"""
from __future__ import annotations

import numpy as np
import pytest

from oracle import gpe
from tests.conftest import load_golden, rel_l2

pytestmark = pytest.mark.gpu

P = dict(hbar=0.6582119514, m_eff=0.284, g_C=0.001, g_R=0.002, g_I=0.0, R=0.02, gamma_C=0.083,
         gamma_R=0.005)


def _k2(nx, ny, dx, dy):
    KX, KY = np.meshgrid(2 * np.pi * np.fft.fftfreq(nx, d=dx), 2 * np.pi * np.fft.fftfreq(ny, d=dy),
                         indexing="xy")
    return KX ** 2 + KY ** 2


@pytest.mark.parametrize("precision,tol", [("double", 1e-10), ("single", 1e-4)])
def test_ifrk4_matches_reference_trajectory(cuda_lib, precision, tol):
    """The reference's IFRK4 golden case (16x16, pulsed pump, complex potential, eta = 0)."""
    from polarism_gb300 import _lib
    from polarism_gb300.engine import Engine, MemberPhysics

    g = load_golden("ifrk4")
    key = "double_single_eta0"
    p = g[key + "_physics"]
    times = np.asarray(g[key + "_pump_times"])
    pumps = g[key + "_pumps"]
    env = pumps[int(np.argmax(pumps.max(axis=(1, 2))))]
    env = env / env.max()
    coeffs = pumps.max(axis=(1, 2)) / env.max()
    ny, nx = env.shape
    dt = 0.007
    eng = Engine(nx, ny, 1, float(g[key + "_dx"]), float(g[key + "_dy"]), dt,
                 MemberPhysics.from_object(p), precision, potential=_lib.PG_POT_COMPLEX)
    eng.set_pump(env.astype(eng.real))
    eng.set_potential(g[key + "_potential"].astype(eng.complex))
    eng.set_state(g[key + "_psi0"].astype(eng.complex), g[key + "_res0"].astype(eng.real))

    def coeff(t):
        return coeffs[int(np.argmin(np.abs(times - t)))]

    scales = np.asarray([[[coeff(k * dt + c * dt)] for c in (0.0, 0.5, 0.5, 1.0)] for k in range(5)])
    eng.ifrk_advance("rk4", 0, 5, scales)
    psi, res = eng.get_state()
    if precision == "double":
        assert rel_l2(psi[0, 0], g[key + "_psi"]) < tol
        assert rel_l2(res[0, 0], g[key + "_res"]) < tol
    else:
        state = gpe.IFRKState(psi=g[key + "_psi0"].astype(np.complex128),
                              fields=(g[key + "_res0"].astype(np.float64),))
        for k in range(5):
            gpe.ifrk_step(state, dt, gpe.RK4_TABLEAU, lambda t: env * coeff(t),
                          g[key + "_potential"].astype(np.complex128), p, g[key + "_k_squared"],
                          float(g[key + "_dx"]), float(g[key + "_dy"]))
        assert rel_l2(psi, state.real_space()) < tol
        assert rel_l2(res, state.fields[0]) < tol


@pytest.mark.parametrize("tableau", ["rk4", "dp5"])
@pytest.mark.parametrize("precision,tol", [("double", 1e-10), ("single", 1e-4)])
@pytest.mark.parametrize("ny,nx", [(16, 32), (32, 1024), (1024, 32)])
def test_fixed_step_with_noise_and_members(cuda_lib, tableau, precision, tol, ny, nx):
    """Fixed-step IFRK with the Wigner increment after each step, three members; FP32 rows of
    1024 sites run the register-resident four-step row pass, FP32 columns of 1024 sites the
    register-resident column pass with the batched site step (stages and step end)."""
    from polarism_gb300.engine import TABLEAU_NODES, Engine, MemberPhysics

    members = 3
    dx, dy, dt = 1.1, 0.9, 0.01
    rng = np.random.default_rng(21)
    psi0 = 0.1 * (rng.standard_normal((members, 1, ny, nx)) + 1j * rng.standard_normal((members, 1, ny, nx)))
    res0 = np.abs(rng.standard_normal((members, 1, ny, nx))) * 0.05
    env = np.exp(-0.5 * (((np.arange(nx) - nx / 2) * dx) ** 2)[None, :] / 9.0
                 - 0.5 * (((np.arange(ny) - ny / 2) * dy) ** 2)[:, None] / 9.0)
    phys = [MemberPhysics(**dict(P, R=0.02 + 0.01 * m)) for m in range(members)]
    eng = Engine(nx, ny, members, dx, dy, dt, phys, precision)
    eng.set_pump(env.astype(eng.real))
    seeds = [5, 6, 7]
    eng.set_noise(seeds, P["gamma_C"], [p.R for p in phys], 1.0, dt / (4 * dx * dy))
    eng.set_state(psi0.astype(eng.complex), res0.astype(eng.real))
    steps = 6
    coeff = lambda t: 0.2 * (1.0 + 0.3 * np.sin(10 * t))  # noqa: E731
    nodes = TABLEAU_NODES[tableau]
    scales = np.asarray([[[coeff(k * dt + c * dt)] * members for c in nodes] for k in range(steps)])
    eng.ifrk_advance(tableau, 0, steps, scales)
    psi, res = eng.get_state()
    tab = gpe.RK4_TABLEAU if tableau == "rk4" else gpe.DP5_TABLEAU
    k2 = _k2(nx, ny, dx, dy)
    for m in range(members):
        pm = dict(P, R=phys[m].R)
        noise = gpe.Noise([seeds[m]], [P["gamma_C"]], [pm["R"]], [1.0], dt, dx * dy, "double",
                          normals_precision=precision)
        state = gpe.IFRKState(psi=psi0[m:m + 1].copy(), fields=(res0[m:m + 1].copy(),))
        for k in range(steps):
            gpe.ifrk_step(state, dt, tab, lambda t: env * coeff(t), 0.0, pm, k2, dx, dy)
            field = state.real_space()
            noise.apply(field, state.fields[0], k)
            state.psi, state.psi_k = field, None
        assert rel_l2(psi[m], state.psi[0]) < tol, m
        assert rel_l2(res[m], state.fields[0][0]) < tol, m


@pytest.mark.parametrize("tableau", ["rk4", "dp5"])
def test_fast_column_pass_with_complex_potential(cuda_lib, tableau):
    """FP32 columns of 1024 sites with a complex potential, two members: the batched site step
    of the register-resident column pass reads V_re and V_im per site."""
    from polarism_gb300 import _lib
    from polarism_gb300.engine import TABLEAU_NODES, Engine, MemberPhysics

    members, ny, nx = 2, 1024, 16
    dx, dy, dt = 0.8, 0.5, 0.01
    rng = np.random.default_rng(34)
    psi0 = 0.1 * (rng.standard_normal((members, 1, ny, nx)) + 1j * rng.standard_normal((members, 1, ny, nx)))
    res0 = np.abs(rng.standard_normal((members, 1, ny, nx))) * 0.05
    y = (np.arange(ny) - ny / 2) * dy
    env = np.broadcast_to(np.exp(-0.5 * y[:, None] ** 2 / 900.0), (ny, nx))
    pot = (0.02 * np.cos(2 * np.pi * y / 64.0)[:, None] + 0.005j * np.sin(2 * np.pi * y / 96.0)[:, None]
           + np.zeros((1, nx)))
    phys = [MemberPhysics(**dict(P, R=0.02 + 0.01 * m)) for m in range(members)]
    eng = Engine(nx, ny, members, dx, dy, dt, phys, "single", potential=_lib.PG_POT_COMPLEX)
    eng.set_pump(env.astype(eng.real))
    eng.set_potential(pot.astype(eng.complex))
    eng.set_state(psi0.astype(eng.complex), res0.astype(eng.real))
    steps = 5
    coeff = lambda t: 0.3 * (1.0 + 0.2 * np.cos(7 * t))  # noqa: E731
    nodes = TABLEAU_NODES[tableau]
    scales = np.asarray([[[coeff(k * dt + c * dt)] * members for c in nodes] for k in range(steps)])
    eng.ifrk_advance(tableau, 0, steps, scales)
    psi, res = eng.get_state()
    eng.close()
    tab = gpe.RK4_TABLEAU if tableau == "rk4" else gpe.DP5_TABLEAU
    k2 = _k2(nx, ny, dx, dy)
    for m in range(members):
        pm = dict(P, R=phys[m].R)
        state = gpe.IFRKState(psi=psi0[m:m + 1].copy(), fields=(res0[m:m + 1].copy(),))
        for k in range(steps):
            gpe.ifrk_step(state, dt, tab, lambda t: env * coeff(t), pot, pm, k2, dx, dy)
        assert rel_l2(psi[m], state.real_space()[0]) < 1e-4, m
        assert rel_l2(res[m], state.fields[0][0]) < 1e-4, m


@pytest.mark.parametrize("ny,nx", [(32, 1024), (1024, 32)])
def test_dp5_trial_error_norm_on_the_1024_site_passes(cuda_lib, ny, nx):
    """The adaptive trial's error estimate on FP32 rows (a row pass over stored stage spectra
    only) or columns (stages and step end on the register-resident column pass, the error norm
    on the generic one) of 1024 sites against the FP64 engine's: the error norm within 1e-2
    and, away from the threshold, the same accept decision."""
    from polarism_gb300.engine import Engine, MemberPhysics

    dx, dy = 0.4, 0.4
    rng = np.random.default_rng(8)
    psi0 = 0.2 * (rng.standard_normal((1, 1, ny, nx)) + 1j * rng.standard_normal((1, 1, ny, nx)))
    res0 = np.abs(rng.standard_normal((1, 1, ny, nx))) * 0.05
    env = np.exp(-0.5 * (((np.arange(nx) - nx / 2) * dx) ** 2)[None, :] / 400.0
                 - 0.5 * (((np.arange(ny) - ny / 2) * dy) ** 2)[:, None] / 400.0)
    errs = {}
    for precision in ("double", "single"):
        eng = Engine(nx, ny, 1, dx, dy, 0.01, MemberPhysics(**P), precision)
        eng.set_pump(np.broadcast_to(env, (ny, nx)).astype(eng.real))
        eng.set_state(psi0.astype(eng.complex), res0.astype(eng.real))
        errs[precision] = eng.ifrk_trial(0.02, np.full((7, 1), 0.2), 1e-6, 1e-8)
        eng.close()
    # The estimate is a small combination of FP32 stage spectra: a few 1e-3 of it is rounding.
    assert abs(errs["single"][0] - errs["double"][0]) <= 1e-2 * errs["double"][0]
    if abs(errs["double"][0] - 1.0) > 1e-2:
        assert errs["single"][1] == errs["double"][1]


def test_dp5_adaptive_matches_reference_run(cuda_lib):
    """Accepted/rejected counts and the final state of the reference's adaptive DP5 run."""
    from polarism_gb300.engine import TABLEAU_NODES, Engine, MemberPhysics
    from polarism_gb300.step_control import StepController

    g = load_golden("dp5_p2")
    p = g["physics"]
    ny, nx = g["psi0"].shape[-2:]
    eng = Engine(nx, ny, 1, float(g["dx"]), float(g["dy"]), float(g["dt"]),
                 MemberPhysics.from_object(p), "double")
    eng.set_pump(g["envelope"])
    eng.set_state(g["psi0"], g["res0"][0])
    ctl = StepController(float(g["dt"]))
    t, target = 0.0, int(g["ticks"]) * float(g["dt"])
    while t < target:
        h, clamped, proposal = ctl.propose(t, target)
        scales = np.full((7, 1), float(g["p0"]))
        err, acc = eng.ifrk_trial(h, scales, float(g["rtol"]), float(g["atol"]))
        if acc:
            t = target if clamped else t + h
        ctl.update(h, clamped, proposal, acc, err)
    psi, res = eng.get_state()
    assert (ctl.accepted, ctl.rejected) == (int(g["accepted"]), int(g["rejected"]))
    assert rel_l2(psi, g["psi"]) < 1e-10 and rel_l2(res, g["res"][0]) < 1e-10
    assert len(TABLEAU_NODES["dp5"]) == 7


@pytest.mark.parametrize("precision,rtol", [("double", 1e-6), ("double", 1e-9), ("single", 1e-5)])
def test_dp5_uniform_decay_known_answer(cuda_lib, precision, rtol):
    """psi(t) = exp(-gamma t / 2 + i phi(t)) for a uniform field without reservoir."""
    from polarism_gb300.engine import Engine, MemberPhysics
    from polarism_gb300.step_control import StepController

    n = 4
    phys = MemberPhysics(g_C=2.0, g_R=0.0, R=0.0, gamma_C=0.7, gamma_R=0.0)
    eng = Engine(n, n, 1, 1.0, 1.0, 1.0, phys, precision, reservoir=False)
    eng.set_pump(np.zeros((n, n)))
    eng.set_state(np.ones((1, 1, n, n), dtype=eng.complex))
    for total, dt in ((2.0, 1.0), (5.0, 5.0)):
        eng.set_state(np.ones((1, 1, n, n), dtype=eng.complex))
        ctl = StepController(dt)
        t = 0.0
        while t < total:
            h, clamped, proposal = ctl.propose(t, total)
            err, acc = eng.ifrk_trial(h, np.zeros((7, 1)), rtol, rtol * 0.01)
            if acc:
                t = total if clamped else t + h
            ctl.update(h, clamped, proposal, acc, err)
        psi, _ = eng.get_state()
        phase = -2.0 / (0.6582119514 * 0.7) * (1 - np.exp(-0.7 * total))
        exact = np.exp(-0.7 * total / 2 + 1j * phase)
        tol = 50 * rtol if precision == "double" else 50 * rtol + 1e-5
        assert np.max(np.abs(psi - exact)) <= tol, (total, np.max(np.abs(psi - exact)))
        if dt == 5.0:
            assert ctl.rejected > 0
