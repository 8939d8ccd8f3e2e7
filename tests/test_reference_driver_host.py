"""The drop-in solvers driven by the reference's own objects (CPU; skipped without Polarism).

The reference's ``SimulationController`` builds the grid, ``Model`` (pump field, reservoir,
``NoiseApplier``), ``SimulationState`` and -- through the solver registry -- the solver, and
calls ``solver.advance(model, state, n)`` (``polarism/simulation_controller.py:163-310,
997-1130``; ``polarism/solver/abstract_solver.py:60-101``).  Here ``rk4-cuda``,
``split-step-fft`` and ``split-step-fft-cuda`` resolve to this package's classes, and the
device engine they drive is replaced by a recording stand-in that keeps every argument the
solver derived from the reference's objects and advances the state with the FP64 oracle.
The tests check those arguments against the reference objects (pump envelope, per-stage
coefficients, per-member seeds, gamma_C, R, strength, dt / 4 dV, physics constants), the
state bookkeeping (``state.step``, ``state.t``, the reservoir hand-back, the spectrum that
``split-step-fft-cuda`` leaves), and the whole trajectory against the reference's own CPU
solvers on the same controller configuration (``rk4-fdm``, ``split-step-fft``).
"""
from __future__ import annotations

import numpy as np
import pytest

from oracle import gpe
from tests.test_host import _reference_importable

STEPS = (5, 7)  # two advance calls: start step and time carry over between them


class RecordingEngine:
    """Stands in for ``polarism_gb300.engine.RK4Engine`` (same methods the solvers call)."""

    made: list = []

    def __init__(self, nx, ny, members, dx, dy, dt, physics, precision="single", reservoir=True,
                 potential=0, pump_per_member=False, potential_per_member=False, components=1,
                 reservoir_components=None, pump_terms=1):
        self.nx, self.ny, self.members = int(nx), int(ny), int(members)
        self.dx, self.dy, self.dt = float(dx), float(dy), float(dt)
        self.physics = list(physics)
        self.precision = precision
        self.real = np.float32 if precision == "single" else np.float64
        self.complex = np.complex64 if precision == "single" else np.complex128
        self.reservoir_kind = {True: "single", False: "none"}.get(reservoir, reservoir)
        self.potential_kind = int(potential)
        self.pump_terms = int(pump_terms)
        self.shape = (self.members, 1, self.ny, self.nx)
        self.res_shape = self.shape
        self.calls = []
        self.noise = None
        self.spectral = False
        RecordingEngine.made.append(self)

    # inputs ---------------------------------------------------------------------------------
    def close(self):
        pass

    def set_pump(self, envelope):
        self.envelope = np.array(envelope, dtype=np.float64)
        self.calls.append(("set_pump", self.envelope.copy()))

    def set_potential(self, potential):
        self.calls.append(("set_potential", np.array(potential)))

    def set_noise(self, seeds=None, gamma=None, scattering=None, strength=None, dt_over_4dv=0.0):
        self.noise = None if seeds is None else dict(
            seeds=np.asarray(seeds, dtype=np.uint64).reshape(-1),
            gamma=np.asarray(gamma, dtype=np.float64).reshape(-1),
            scattering=np.asarray(scattering, dtype=np.float64).reshape(-1),
            strength=np.asarray(strength, dtype=np.float64).reshape(-1),
            dt_over_4dv=float(dt_over_4dv))
        self.calls.append(("set_noise", self.noise))

    def set_state(self, psi, res=None):
        self.psi = np.array(psi, dtype=np.complex128).reshape(self.shape)
        self.res = None if res is None else np.array(res, dtype=np.float64).reshape(self.res_shape)
        self.calls.append(("set_state",))

    def set_state_kind(self, spectral):
        self.spectral = bool(spectral)
        self.calls.append(("set_state_kind", self.spectral))

    def get_state(self, psi_out=None, res_out=None):
        psi = self.psi.astype(self.complex)
        res = None if self.res is None else self.res.astype(self.real)
        if psi_out is not None:
            psi_out[...] = psi
            psi = psi_out
        if res_out is not None and res is not None:
            res_out[...] = res
            res = res_out
        self.returned_res = res
        return psi, res

    # stepping with the oracle --------------------------------------------------------------
    def _p(self):
        names = ("hbar", "m_eff", "g_C", "g_R", "g_I", "R", "gamma_C", "gamma_R")
        return {k: np.asarray([getattr(ph, k) for ph in self.physics]).reshape(-1, 1, 1, 1)
                for k in names}

    def _noise(self):
        if self.noise is None:
            return None
        n = self.noise
        # dt / (4 dV) fixes the cell volume the oracle's increment uses.
        return gpe.Noise(n["seeds"], n["gamma"], n["scattering"], n["strength"], self.dt,
                         self.dt / (4.0 * n["dt_over_4dv"]), "double")

    def _pump(self, scales, step, nodes, t):
        env = self.envelope.reshape((-1, 1, self.ny, self.nx) if self.envelope.ndim == 4
                                    else (self.ny, self.nx))

        def at(time):
            node = int(round((time - t) / self.dt * 4))  # quarter steps
            return scales[step][nodes[node]].reshape(-1, 1, 1, 1) * env
        return at

    def advance(self, start_step, n_steps, stage_scales, use_graphs=True):
        scales = np.asarray(stage_scales, dtype=np.float64)
        self.calls.append(("advance", int(start_step), int(n_steps), scales.copy()))
        p, noise = self._p(), self._noise()
        psi, fields = self.psi, (self.res,)
        for k in range(n_steps):
            step = start_step + k
            t = step * self.dt
            pump = self._pump(scales, k, {0: 0, 2: 1, 4: 2}, t)
            psi, fields = gpe.rk4_step(psi, fields, pump, 0.0, p, self.dx, self.dy, self.dt, t)
            if noise is not None:
                noise.apply(psi, fields[0], step)
        self.psi, self.res = psi, fields[0]

    def split_advance(self, ordering, start_step, n_steps, half_scales, use_graphs=True):
        scales = np.asarray(half_scales, dtype=np.float64)
        self.calls.append(("split_advance", int(ordering), int(start_step), int(n_steps),
                           scales.copy()))
        p, noise = self._p(), self._noise()
        kx = 2 * np.pi * np.fft.fftfreq(self.nx, self.dx)
        ky = 2 * np.pi * np.fft.fftfreq(self.ny, self.dy)
        k2 = kx[None, :] ** 2 + ky[:, None] ** 2
        psi = np.fft.ifft2(self.psi) if (ordering == 1 and self.spectral) else self.psi
        fields = (self.res,)
        step_fn = gpe.split_step_cpu if ordering == 0 else gpe.split_step_kouter
        for k in range(n_steps):
            step = start_step + k
            t = step * self.dt
            pump = self._pump(scales, k, {1: 0, 3: 1}, t)
            psi, fields = step_fn(psi, fields, pump, 0.0, p, k2, self.dx, self.dy, self.dt, t,
                                  step, "single", noise)
        # split-step-fft-cuda leaves the unnormalised spectrum in the state.
        self.psi = np.fft.fft2(psi) if ordering == 1 else psi
        self.res = fields[0]


@pytest.fixture()
def reference(monkeypatch):
    if _reference_importable() is None:
        pytest.skip("Polarism source tree not available on this host")
    import warnings

    import polarism_gb300
    from polarism_gb300 import _lib, solvers

    monkeypatch.setattr(solvers, "RK4Engine", RecordingEngine)
    monkeypatch.setattr(_lib, "load", lambda *a, **k: None)
    RecordingEngine.made.clear()
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        polarism_gb300.register()
    yield


def _controller(method, wigner=True):
    from polarism.config.simulation_parameters import Config
    from polarism.simulation_controller import SimulationController

    cfg = Config()
    cfg.grid.nx, cfg.grid.ny, cfg.grid.lx, cfg.grid.ly = 32, 16, 16.0, 8.0
    cfg.reservoir.reservoir_type = "single"
    cfg.potential.potential_type = "zero"
    cfg.laser.mode = "single"
    cfg.laser.laser_type = "continuous-gaussian"
    cfg.laser.P0, cfg.laser.sigma_space = 0.05, 4.0
    cfg.solver.method = method
    cfg.solver.dt = 2e-3
    cfg.solver.precision = "double"
    cfg.solver.total_time = 2e-3 * sum(STEPS)
    cfg.noise.seed = 3
    if wigner:
        cfg.noise.stochastic = "wigner"
    return SimulationController(cfg)


def _run(ctl):
    for n in STEPS:
        ctl.solver.advance(ctl.model, ctl.state, n)
    return np.array(ctl.state.field), np.array(ctl.reservoir.get_state()[0])


def _check_inputs(ctl, engine):
    """What the solver handed the engine equals the reference's own objects."""
    noise = ctl.model.noise
    assert engine.noise is not None
    np.testing.assert_array_equal(engine.noise["seeds"], np.asarray(noise.seeds, dtype=np.uint64))
    np.testing.assert_allclose(engine.noise["gamma"], noise.gamma, rtol=0, atol=0)
    np.testing.assert_allclose(engine.noise["scattering"], noise.scattering, rtol=0, atol=0)
    np.testing.assert_allclose(engine.noise["strength"], noise.strength, rtol=0, atol=0)
    assert engine.noise["dt_over_4dv"] == noise.dt / (4.0 * noise.volume)
    env, _ = ctl.model.pump.separable_term()
    np.testing.assert_array_equal(engine.envelope.reshape(np.shape(env)), np.asarray(env))
    phys = ctl.cfg.physics
    for name in ("hbar", "m_eff", "g_C", "g_R", "R", "gamma_C", "gamma_R"):
        assert getattr(engine.physics[0], name) == getattr(phys, name), name
    assert (engine.nx, engine.ny, engine.dx, engine.dy) == (ctl.grid.nx, ctl.grid.ny,
                                                            ctl.grid.dx, ctl.grid.dy)


def _coefficients(ctl, start, n, nodes):
    _, coefficient = ctl.model.pump.separable_term()
    dt = ctl.cfg.solver.dt
    return np.asarray([[np.asarray(coefficient(ctl.state.t0 + (start + k + c) * dt)).reshape(-1)
                        for c in nodes] for k in range(n)])


def test_rk4_cuda_under_the_reference_controller_matches_rk4_fdm(reference):
    from polarism_gb300.solvers import RK4CudaSolver

    ctl = _controller("rk4-cuda")
    assert isinstance(ctl.solver, RK4CudaSolver)
    psi, res = _run(ctl)
    engine = RecordingEngine.made[-1]
    _check_inputs(ctl, engine)
    advances = [c for c in engine.calls if c[0] == "advance"]
    assert [(c[1], c[2]) for c in advances] == [(0, STEPS[0]), (STEPS[0], STEPS[1])]
    start = 0
    for c in advances:  # coefficients at t, t + dt/2, t + dt of every step
        np.testing.assert_allclose(c[3], _coefficients(ctl, start, c[2], (0.0, 0.5, 1.0)),
                                   rtol=0, atol=0)
        start += c[2]
    assert ctl.state.step == sum(STEPS)
    assert ctl.state.t == ctl.state.t0 + sum(STEPS) * ctl.cfg.solver.dt
    # The reservoir the engine returned is what the reference's reservoir now holds.
    np.testing.assert_array_equal(res, np.asarray(engine.returned_res).reshape(res.shape))

    ref = _controller("rk4-fdm")
    psi_ref, res_ref = _run(ref)
    assert np.linalg.norm(psi - psi_ref) / np.linalg.norm(psi_ref) < 1e-12
    assert np.linalg.norm(res - res_ref) / np.linalg.norm(res_ref) < 1e-12


def test_split_step_fft_under_the_reference_controller_matches_its_cpu_solver(reference):
    from polarism_gb300.solvers import SplitStepFFTSolver

    ctl = _controller("split-step-fft")
    assert type(ctl.solver) is SplitStepFFTSolver
    psi, res = _run(ctl)
    engine = RecordingEngine.made[-1]
    _check_inputs(ctl, engine)
    calls = [c for c in engine.calls if c[0] == "split_advance"]
    assert [(c[1], c[2], c[3]) for c in calls] == [(0, 0, STEPS[0]), (0, STEPS[0], STEPS[1])]
    np.testing.assert_allclose(calls[1][4], _coefficients(ctl, STEPS[0], STEPS[1], (0.25, 0.75)),
                               rtol=0, atol=0)
    assert ctl.state.step == sum(STEPS)

    # The reference's own NumPy split-step solver (split_step_fft_solver.py:97-159).  The
    # drop-in's class now owns the name, so build the reference class directly.
    from polarism.solver.split_step_fft_solver import SplitStepFFTSolver as RefSplit

    ref = _controller("split-step-fft")
    ref.solver = RefSplit(ref.cfg, ref.grid, ref.model)
    psi_ref, res_ref = _run(ref)
    assert np.linalg.norm(psi - psi_ref) / np.linalg.norm(psi_ref) < 1e-12
    assert np.linalg.norm(res - res_ref) / np.linalg.norm(res_ref) < 1e-12


def test_split_step_fft_cuda_leaves_the_spectrum_and_matches_the_kouter_oracle(reference):
    from polarism_gb300.solvers import SplitStepFFTCudaSolver

    ctl = _controller("split-step-fft-cuda")
    assert isinstance(ctl.solver, SplitStepFFTCudaSolver)
    psi0 = np.array(ctl.state.field)
    res0 = np.array(ctl.reservoir.get_state()[0])
    for n in STEPS:
        ctl.solver.advance(ctl.model, ctl.state, n)
        # After each call the state holds the spectrum only, as the reference's solver leaves it.
        assert ctl.state._field is None and ctl.state.field_k is not None
    engine = RecordingEngine.made[-1]
    _check_inputs(ctl, engine)
    kinds = [c[1] for c in engine.calls if c[0] == "set_state_kind"]
    assert kinds == [False, True]  # real space on entry, the kept spectrum afterwards
    assert ctl.state.step == sum(STEPS)
    psi = np.array(ctl.state.field)  # the reference's state transforms field_k back

    g = ctl.grid
    phys = ctl.cfg.physics
    p = {k: getattr(phys, k) for k in ("hbar", "m_eff", "g_C", "g_R", "g_I", "R", "gamma_C",
                                       "gamma_R")}
    env, coefficient = ctl.model.pump.separable_term()
    noise = ctl.model.noise
    oracle_noise = gpe.Noise(noise.seeds, noise.gamma, noise.scattering, noise.strength,
                             noise.dt, noise.volume, "double")
    kx = 2 * np.pi * np.fft.fftfreq(g.nx, g.dx)
    ky = 2 * np.pi * np.fft.fftfreq(g.ny, g.dy)
    k2 = kx[None, :] ** 2 + ky[:, None] ** 2
    psi_o, f_o = gpe.split_advance("kouter", psi0, (res0,),
                                   lambda t: float(np.asarray(coefficient(t)).reshape(-1)[0]) * np.asarray(env),
                                   0.0, p, k2, g.dx, g.dy, ctl.cfg.solver.dt, 0, sum(STEPS),
                                   noise=oracle_noise)
    assert np.linalg.norm(psi - psi_o) / np.linalg.norm(psi_o) < 1e-12
    res = np.array(ctl.reservoir.get_state()[0])
    assert np.linalg.norm(res - f_o[0]) / np.linalg.norm(f_o[0]) < 1e-12
