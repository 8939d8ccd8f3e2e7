"""The steady-state stop of the controller's run loop kept on the device, with the real
library (``polarism_gb300.run_loop.DeviceSteadyMonitor`` over ``rk4-cuda`` and
``split-step-fft``).

``LoopController`` restates what ``SimulationController.run`` does around the stop
(``polarism/simulation_controller.py:1063-1130``: chunks that end on every check step,
``_check_steady_state`` :710-734 computed on the host from the state the drop-in hands back,
``_record_stops`` :698-708, the loop ending once every member has a stop time).  Members relax
to the fixed point of a near-uniform pump at three strengths, so they stop at different checks.

The run with the monitor installed must stop every member on the same step as the host-decided
run, end on the same step with a bitwise-equal state, and make no host wait between its first
chunk and the settle: the library's own counter (``pg_sync_counts``) does not move while the
chunks and the checks are queued.
"""
from __future__ import annotations

import copy

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N, DX, DT, INTERVAL, RTOL, STEPS = 16, 1.0, 0.05, 20, 5e-3, 4000
P0 = (4.0, 8.0, 16.0)


class LoopController:
    """The stop-related part of the reference's controller: ``cfg``, ``state``, ``model``,
    ``solver``, ``stop_times``, the ``_steady_*`` attributes, ``_check_steady_state`` and
    ``run``.  ``after_first_advance`` is called once, after the first chunk."""

    def __init__(self, cfg, grid, model, state, solver, accumulate_every=0):
        self.cfg, self.grid, self.model, self.state, self.solver = cfg, grid, model, state, solver
        self.accumulate_every = accumulate_every  # steps between g2 samples (0: none)
        self._accumulators = {"g2": G2Sums(state)} if accumulate_every else {}
        self.stop_times = np.full(state.batch_size, np.nan)
        self._steady_density = None
        self._steady_norm = None
        self._steady_last_step = -1
        self.after_first_advance = None
        self.margin = np.inf  # closest approach of a host decision to the threshold (relative)

    def _check_steady_state(self):
        density = np.abs(self.state.psi) ** 2
        norms = np.atleast_1d(density.sum(axis=(-2, -1)) * (self.grid.dx * self.grid.dy))
        if self._steady_density is not None:
            old, old_norms = self._steady_density, self._steady_norm
            rd = np.sqrt(((density - old) ** 2).sum(axis=(-2, -1))) / np.maximum(
                np.sqrt((old ** 2).sum(axis=(-2, -1))), 1e-30)
            rn = np.abs(norms - old_norms) / np.maximum(old_norms, 1e-30)
            self.margin = min(self.margin, float(np.min(np.abs(np.concatenate([rd, rn]) / RTOL - 1))))
            reached = (norms < 1e-30) | ((rn < self.cfg.stop.rtol) & (rd < self.cfg.stop.rtol))
            if self.state.t >= self.cfg.stop.min_time:
                self.stop_times[reached & np.isnan(self.stop_times)] = self.state.t
        self._steady_norm = norms.copy()
        self._steady_density = density.copy()
        self._steady_last_step = self.state.step

    def run(self):
        dt = self.cfg.solver.dt
        n_steps = round(self.cfg.solver.total_time / dt)
        interval = round(self.cfg.stop.check_every / dt)
        step = self.state.step
        first = True
        every = self.accumulate_every
        while step < n_steps and not np.isfinite(self.stop_times).all():
            end = min(n_steps, (step // interval + 1) * interval)
            if every:
                end = min(end, (step // every + 1) * every)
            self.solver.advance(self.model, self.state, end - step)
            if first and self.after_first_advance is not None:
                self.after_first_advance()
            first = False
            step = self.state.step
            if every and step % every == 0:
                self._accumulators["g2"].update(self.state, self.state.t)
            if step % interval == 0 and self._steady_last_step != step:
                self._check_steady_state()


class G2Sums:
    """The reference's G2Accumulator sums (``polarism/results/accumulators.py:134-160``):
    per-site FP64 sums of |psi|^2 and |psi|^4 with the sample count and times."""

    name = "g2"

    def __init__(self, state):
        self.sum_density = np.zeros(state.psi.shape)
        self.sum_density_squared = np.zeros(state.psi.shape)
        self.samples, self.t_first, self.t_last = 0, None, None

    def update(self, state, t):
        re, im = state.psi.real.astype(np.float64), state.psi.imag.astype(np.float64)
        density = re * re + im * im
        self.sum_density += density
        self.sum_density_squared += density * density
        if self.samples == 0:
            self.t_first = t
        self.t_last = t
        self.samples += 1

    def state_dict(self):
        return {"samples": self.samples, "t_first": self.t_first, "t_last": self.t_last,
                "sum_density": self.sum_density, "sum_density_squared": self.sum_density_squared}

    def load_state_dict(self, values):
        self.samples, self.t_first, self.t_last = values["samples"], values["t_first"], values["t_last"]
        self.sum_density = np.asarray(values["sum_density"], dtype=np.float64)
        self.sum_density_squared = np.asarray(values["sum_density_squared"], dtype=np.float64)


def _controller(method, precision, accumulate_every=0):
    from polarism_gb300 import solvers
    from polarism_gb300.host import Config, build_simulation

    cfg = Config()
    cfg.grid.nx = cfg.grid.ny = N
    cfg.grid.lx = cfg.grid.ly = N * DX
    cfg.physics.gamma_R = 0.5
    cfg.solver.dt = DT
    cfg.solver.total_time = STEPS * DT
    cfg.solver.precision = precision
    cfg.stop.steady_state = True
    cfg.stop.rtol = RTOL
    cfg.stop.check_every = INTERVAL * DT
    cfg.laser.sigma_space = 1e3  # a near-uniform pump
    cfg.noise.enabled = False
    members = []
    for p0 in P0:
        c = copy.deepcopy(cfg)
        c.laser.P0 = p0
        members.append(c)
    grid, model, state = build_simulation(cfg, members)
    x = (np.arange(N) - N / 2) * DX
    row = (1.0 + 0.02 * np.cos(2 * np.pi * x / (N * DX))).astype(state.field.dtype)
    state.field = np.ascontiguousarray(np.broadcast_to(row[None, :], state.field.shape))
    n0 = model.reservoir.get_state()[0]
    model.reservoir.set_state((np.full_like(n0, 4.0),))
    cls = {"rk4-cuda": solvers.RK4CudaSolver, "split-step-fft": solvers.SplitStepFFTSolver}[method]
    solver = cls(cfg, grid, model)
    return LoopController(cfg, grid, model, state, solver, accumulate_every)


@pytest.mark.parametrize("precision", ["single", "double"])
@pytest.mark.parametrize("method", ["rk4-cuda", "split-step-fft"])
def test_device_monitor_in_the_run_loop_matches_host_decisions_without_waits(cuda_lib, method,
                                                                              precision):
    from polarism_gb300.run_loop import DeviceSteadyMonitor

    host = _controller(method, precision)
    host.run()
    assert np.isfinite(host.stop_times).all() and host.state.step < STEPS
    assert len(set(host.stop_times.tolist())) == 3      # staggered stops
    assert host.margin > 1e-6                           # no decision sits on the threshold

    dev = _controller(method, precision)
    monitor = DeviceSteadyMonitor(dev).install()
    counts = {}

    def first_chunk_queued():
        counts["start"] = dev.solver.engine.sync_counts()

    dev.after_first_advance = first_chunk_queued
    settle = monitor.settle

    def settle_counted():
        counts.setdefault("settle", dev.solver.engine.sync_counts())
        settle()

    monitor.settle = settle_counted
    dev.run()
    engine = dev.solver.engine
    np.testing.assert_array_equal(dev.stop_times, host.stop_times)
    assert (dev.state.step, dev.state.t) == (host.state.step, host.state.t)
    assert np.array_equal(dev.state.field, host.state.field)
    assert np.array_equal(dev.model.reservoir.get_state()[0], host.model.reservoir.get_state()[0])
    # No host wait while the chunks and the checks were queued (the monitor's reset at the
    # first check is stream ordered too), until the settle.
    (syncs0, _), (syncs1, _) = counts["start"], counts["settle"]
    assert syncs1 == syncs0
    assert monitor.checks >= host.state.step // INTERVAL
    assert monitor.settles == 1
    stopped, done = engine.steady_poll()
    assert stopped == 3
    monitor.uninstall()


def test_host_decided_loop_waits_every_chunk(cuda_lib):
    """The same loop without the monitor: the drop-in copies the state in and out around every
    chunk, each a host wait the counter sees."""
    ctl = _controller("rk4-cuda", "single")
    counts = {}
    ctl.after_first_advance = lambda: counts.setdefault("start", ctl.solver.engine.sync_counts())
    ctl.run()
    chunks = ctl.state.step // INTERVAL
    syncs = ctl.solver.engine.sync_counts()[0] - counts["start"][0]
    assert syncs >= 2 * (chunks - 1)


@pytest.mark.parametrize("precision", ["single", "double"])
def test_device_accumulator_in_the_run_loop(cuda_lib, precision):
    """A g2 accumulator sampled every 50 steps: summed on the device under the monitor (no host
    wait while chunks, checks and samples are queued; samples after the halting check add
    nothing), it ends with the host loop's sample count, times and bitwise-equal sums."""
    from polarism_gb300.run_loop import DeviceSteadyMonitor

    host = _controller("rk4-cuda", precision, accumulate_every=50)
    host.run()
    dev = _controller("rk4-cuda", precision, accumulate_every=50)
    monitor = DeviceSteadyMonitor(dev).install()
    counts = {}
    dev.after_first_advance = lambda: counts.setdefault("start", dev.solver.engine.sync_counts())
    settle = monitor.settle

    def settle_counted():
        counts.setdefault("settle", dev.solver.engine.sync_counts())
        settle()

    monitor.settle = settle_counted
    dev.run()
    assert counts["settle"][0] == counts["start"][0]
    np.testing.assert_array_equal(dev.stop_times, host.stop_times)
    assert dev.state.step == host.state.step
    h, d = host._accumulators["g2"].state_dict(), dev._accumulators["g2"].state_dict()
    assert (d["samples"], d["t_first"], d["t_last"]) == (h["samples"], h["t_first"], h["t_last"])
    assert h["samples"] >= 10
    assert np.array_equal(d["sum_density"], h["sum_density"])
    assert np.array_equal(d["sum_density_squared"], h["sum_density_squared"])
    monitor.uninstall()
