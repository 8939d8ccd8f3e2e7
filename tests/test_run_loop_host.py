"""The device steady-state monitor under the reference's own ``SimulationController.run``
(CPU; skipped without Polarism).

The controller drives ``rk4-cuda`` / ``split-step-fft`` (this package's drop-ins) over a
recording engine that steps with the FP64 oracle and also stands in for the library's
steady-state monitor (``pg_steady_update`` / ``pg_steady_poll`` / ``pg_steady_results``:
the comparison of ``polarism/simulation_controller.py:710-734`` on the engine's state, the
first stop step, the halt once every member has stopped).  It counts the entry points that
make the library wait for the device: state copies in and out, results and exports.

One run uses the reference's host-side check (the drop-in copies the state back after every
chunk); the other installs :class:`polarism_gb300.run_loop.DeviceSteadyMonitor`.  Both must
give the same stop times, the same final step and time and the same final fields, and the
monitored run must make no synchronising call between its first upload and the deciding
check.
"""
from __future__ import annotations

import numpy as np
import pytest

from tests.test_reference_driver_host import RecordingEngine, reference  # noqa: F401

SYNCING = ("set_state", "get_state", "steady_results", "steady_export", "steady_import",
           "steady_reset", "synchronize", "accumulator_sums")


class MonitoringEngine(RecordingEngine):
    """RecordingEngine plus a host stand-in for the device steady-state monitor.  The
    progress word shows a halt only ``lag`` advance calls after it, as a device running
    behind the host would: the host queues chunks past the deciding check."""

    lag = 0

    def __init__(self, *args, **kwargs):
        super().__init__(*args, **kwargs)
        self.syncs = []          # (call, number of advance calls before it)
        self.advances = 0
        self.halted = False
        self.halted_at = None    # advance calls made when the halt was set
        self.after_halt = 0      # advance calls that found the halt set
        self._steady_reset_state()

    def _sync(self, name):
        self.syncs.append((name, self.advances))

    def _steady_reset_state(self):
        self.rho_old = None
        self.norm_old = None
        self.stop_step = np.full(self.members, -1, dtype=np.int64)
        self.halt_step = None
        self.updates = 0
        self.results = (np.full(self.members, np.inf),) * 3

    def set_state(self, psi, res=None):
        self._sync("set_state")
        super().set_state(psi, res)

    def get_state(self, psi_out=None, res_out=None):
        self._sync("get_state")
        return super().get_state(psi_out, res_out)

    def advance(self, start_step, n_steps, stage_scales, use_graphs=True):
        self.advances += 1
        if self.halted:  # every launch returns at once
            self.after_halt += 1
            return
        super().advance(start_step, n_steps, stage_scales, use_graphs)

    def split_advance(self, ordering, start_step, n_steps, half_scales, use_graphs=True):
        self.advances += 1
        if self.halted:
            self.after_halt += 1
            return
        super().split_advance(ordering, start_step, n_steps, half_scales, use_graphs)

    # the monitor's entry points ------------------------------------------------------------
    def steady_reset(self):
        self._sync("steady_reset")
        self.halted = False
        self._steady_reset_state()

    def steady_import(self, density, norms, stop_steps=None):
        self._sync("steady_import")
        self._steady_reset_state()
        if density is not None:
            self.rho_old = np.asarray(density, dtype=np.float64).reshape(self.members, self.ny, self.nx)
            self.norm_old = np.asarray(norms, dtype=np.float64).reshape(self.members)
        if stop_steps is not None:
            self.stop_step = np.asarray(stop_steps, dtype=np.int64).copy()

    def steady_update(self, step, record=True, rtol=1e-6, halt=False):
        if self.halted:
            return
        self.updates += 1
        rho = (np.abs(self.psi) ** 2).reshape(self.members, self.ny, self.nx)
        norms = rho.sum(axis=(-2, -1)) * (self.dx * self.dy)
        if self.rho_old is not None:
            rd = np.sqrt(((rho - self.rho_old) ** 2).sum(axis=(-2, -1))) / np.maximum(
                np.sqrt((self.rho_old ** 2).sum(axis=(-2, -1))), 1e-30)
            rn = np.abs(norms - self.norm_old) / np.maximum(self.norm_old, 1e-30)
            reached = (norms < 1e-30) | ((rn < rtol) & (rd < rtol))
            if record:
                self.stop_step[reached & (self.stop_step < 0)] = step
            self.results = (rd, rn, norms)
        self.rho_old, self.norm_old = rho, norms
        if halt and (self.stop_step >= 0).all():
            self.halted = True
            self.halt_step = int(step)
            self.halted_at = self.advances

    def steady_poll(self):
        stopped = int((self.stop_step >= 0).sum())
        if self.halted and self.advances - self.halted_at < self.lag:
            stopped -= 1  # the deciding check has not reached the progress word yet
        return stopped, self.updates

    def steady_results(self):
        self._sync("steady_results")
        rd, rn, nm = self.results
        halt = self.halt_step
        self.halted = False
        return rd, rn, nm, self.stop_step.copy(), halt

    # FP64 observable sums (pg_accumulate, pg_accumulator_zero, pg_accumulator_sums) --------
    def accumulator_zero(self):
        shape = (self.members, 1, self.ny, self.nx)
        self.sums = {"rho": np.zeros(shape), "rho2": np.zeros(shape), "k": np.zeros(shape)}

    def accumulate(self, density=True, momentum=False):
        if self.halted:  # the accumulation kernels return at once after the halt
            return
        if density:
            rho = self.psi.real.astype(np.float64) ** 2 + self.psi.imag.astype(np.float64) ** 2
            self.sums["rho"] += rho
            self.sums["rho2"] += rho * rho
        if momentum:
            fk = np.fft.fftn(self.psi, axes=(-2, -1))
            self.sums["k"] += fk.real.astype(np.float64) ** 2 + fk.imag.astype(np.float64) ** 2

    def accumulator_sums(self, kind):
        self._sync("accumulator_sums")
        return self.sums[kind].copy(), 0

    def steady_export(self):
        self._sync("steady_export")
        if self.rho_old is None:
            return None, None, self.stop_step.copy()
        return self.rho_old.copy(), self.norm_old.copy(), self.stop_step.copy()


@pytest.fixture(params=[0, 3], ids=["in-step", "lagging"])
def monitored(reference, monkeypatch, request):
    from polarism_gb300 import solvers

    monkeypatch.setattr(solvers, "RK4Engine", MonitoringEngine)
    monkeypatch.setattr(MonitoringEngine, "lag", request.param)
    yield request.param


MEMBERS = [{"laser.P0": 0.05}, {"noise.initial_amplitude": 0.0}, {"physics.gamma_C": 0.3}]


def _controller(method, steps=400, rtol=0.18, min_time=0.1, check_every=2e-2):
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
    cfg.solver.total_time = 2e-3 * steps
    cfg.stop.steady_state = True
    cfg.stop.rtol = rtol
    cfg.stop.check_every = check_every
    cfg.stop.min_time = min_time
    cfg.noise.seed = 3
    return SimulationController(cfg, members=MEMBERS)


def _final(ctl):
    return (np.array(ctl.state.field), np.array(ctl.reservoir.get_state()[0]), ctl.stop_times.copy(),
            ctl.state.step, ctl.state.t)


# rtol between the relative density changes the two integrators show for these members
# (the initial noise disperses faster under the exact kinetic step of the split-step method).
@pytest.mark.parametrize("method,rtol", [("rk4-cuda", 0.18), ("split-step-fft", 0.36)])
def test_device_monitor_under_the_reference_run_loop_matches_the_host_check(monitored, method,
                                                                            rtol):
    from polarism_gb300.run_loop import DeviceSteadyMonitor

    host = _controller(method, rtol=rtol)
    host.run()
    psi_h, res_h, stops_h, step_h, t_h = _final(host)
    engine_h = MonitoringEngine.made[-1]
    # The host check stops every member before the end (the comparison means something),
    # after copying the state back at every chunk.
    assert np.isfinite(stops_h).all() and step_h < 400
    assert sum(1 for name, _ in engine_h.syncs if name == "get_state") == engine_h.advances

    dev = _controller(method, rtol=rtol)
    monitor = DeviceSteadyMonitor(dev).install()
    dev.run()
    engine = MonitoringEngine.made[-1]
    psi, res, stops, step, t = _final(dev)
    np.testing.assert_array_equal(stops, stops_h)
    assert (step, t) == (step_h, t_h)
    np.testing.assert_array_equal(psi, psi_h)
    np.testing.assert_array_equal(res, res_h)
    assert monitor.checks >= step_h // 10
    # One upload before the first chunk; no synchronising call while chunks and checks are
    # queued; the waits after the last queued chunk are the settle (results, state, export).
    first, last = engine.syncs[0], engine.advances
    assert first == ("set_state", 0)
    during = [s for s in engine.syncs[1:] if s[1] < last]
    assert [name for name, _ in during] == ["steady_reset"]
    assert {name for name, _ in engine.syncs[1:]} <= set(SYNCING)
    assert monitor.settles == 1
    # The device halted at the deciding check; the chunks the host queued after it (as many
    # as the progress word lagged) did nothing, and the state is the deciding check's.
    assert engine.halt_step == step_h
    assert engine.after_halt == monitored
    # The controller keeps the last check's density for a later run, as its own check does.
    np.testing.assert_array_equal(dev._steady_density, host._steady_density)
    np.testing.assert_array_equal(dev._steady_norm, host._steady_norm)
    monitor.uninstall()


def test_device_monitor_settles_at_the_last_step_when_members_keep_changing(monitored):
    """rtol too small for two members: the run ends at total_time with their stop times NaN,
    the third member's recorded, and the final state is the last step's."""
    from polarism_gb300.run_loop import run_with_device_monitor

    host = _controller("rk4-cuda", steps=120, rtol=1e-3)
    host.run()
    dev = _controller("rk4-cuda", steps=120, rtol=1e-3)
    run_with_device_monitor(dev)
    psi_h, res_h, stops_h, step_h, t_h = _final(host)
    psi, res, stops, step, t = _final(dev)
    assert step_h == 120 and np.isnan(stops_h).sum() == 2
    np.testing.assert_array_equal(stops, stops_h)
    assert (step, t) == (step_h, t_h)
    np.testing.assert_array_equal(psi, psi_h)
    np.testing.assert_array_equal(res, res_h)


def test_device_monitor_refuses_a_solver_that_leaves_a_spectrum(monitored):
    from polarism_gb300.run_loop import DeviceSteadyMonitor

    ctl = _controller("split-step-fft-cuda")
    with pytest.raises(ValueError, match="cannot keep its state"):
        DeviceSteadyMonitor(ctl)


def test_device_monitor_copies_the_state_back_for_accumulators_and_events(monitored):
    """The controller's other readers of the state -- a scheduled accumulator (g2, every
    0.02 ps from 0.04 ps) and an event callback (every 0.04 ps) -- see the same states with the
    monitor installed as without it, and the event's stop decision still ends the run."""
    from polarism_gb300.run_loop import run_with_device_monitor

    def setup(ctl, seen):
        def event(view):
            seen.append((view.step, np.array(view.density)))
            return view.step >= 120  # every member "stops" by event at step 120
        ctl.add_event(event, 0.04)

    runs = {}
    for mode in ("host", "device"):
        ctl = _controller("rk4-cuda", steps=300, rtol=1e-9)  # the steady check never stops anyone
        ctl.cfg.result.accumulators = {"g2": {"start": 0.04, "every": 0.02}}
        from polarism.results.accumulators import G2Accumulator

        ctl._accumulators = {"g2": G2Accumulator(ctl, start=0.04, every=0.02)}
        seen = []
        setup(ctl, seen)
        if mode == "host":
            ctl.run()
        else:
            run_with_device_monitor(ctl)
        runs[mode] = (ctl, seen)
    (h, h_seen), (d, d_seen) = runs["host"], runs["device"]
    assert [s for s, _ in d_seen] == [s for s, _ in h_seen] and h_seen[-1][0] == 120
    for (_, a), (_, b) in zip(d_seen, h_seen):
        np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(d.stop_times, h.stop_times)
    assert d.state.step == h.state.step == 120
    np.testing.assert_array_equal(np.array(d.state.field), np.array(h.state.field))
    ah, ad = h._accumulators["g2"], d._accumulators["g2"]
    assert ad.samples == ah.samples > 0
    for x, y in zip(ad.results(), ah.results()):
        np.testing.assert_array_equal(np.asarray(x.value), np.asarray(y.value))
    # The results the controller gathered inside run() (its loop ended on the event, before
    # any settle of the monitor's) already hold the device sums.
    assert set(d.accumulated) == set(h.accumulated) and h.accumulated
    for key in h.accumulated:
        np.testing.assert_array_equal(np.asarray(d.accumulated[key].value),
                                      np.asarray(h.accumulated[key].value))


def test_device_monitor_continues_a_run_from_the_controllers_steady_reference(monitored):
    """A second run() that continues the first (total_time raised): the monitor starts from the
    density and stop times the controller kept, as the reference's own check continues from
    _steady_density, so both ways stop every member on the same steps."""
    from polarism_gb300.run_loop import DeviceSteadyMonitor

    results = {}
    for mode in ("host", "device"):
        ctl = _controller("rk4-cuda", steps=60, rtol=0.18)
        monitor = DeviceSteadyMonitor(ctl).install() if mode == "device" else None
        ctl.run()                                  # 60 steps: the zero member stops at 0.1 ps
        first = ctl.stop_times.copy()
        ctl.cfg.solver.total_time = 2e-3 * 400
        ctl.run()                                  # continues from step 60
        results[mode] = (first, ctl.stop_times.copy(), ctl.state.step, np.array(ctl.state.field))
        if monitor is not None:
            monitor.uninstall()
    (h1, h2, hs, hf), (d1, d2, ds, df) = results["host"], results["device"]
    np.testing.assert_array_equal(d1, h1)
    assert np.isfinite(h1).sum() == 1 and np.isfinite(h2).all()
    np.testing.assert_array_equal(d2, h2)
    assert ds == hs < 400
    np.testing.assert_array_equal(df, hf)


def test_device_accumulators_match_the_reference_accumulators(monitored):
    """g2 (from t = 0: its first sample is taken on the host before any chunk) and the
    momentum distribution summed on the device under the monitor, with the steady-state stop
    halting the run (and, in the lagging case, samples queued past the halt): the same sample
    counts, first and last times and sums as the reference's own accumulators."""
    from polarism.results.accumulators import G2Accumulator, MomentumDistribution

    from polarism_gb300.run_loop import run_with_device_monitor

    out = {}
    for mode in ("host", "device"):
        ctl = _controller("rk4-cuda", rtol=0.18)
        ctl._accumulators = {"g2": G2Accumulator(ctl, start=0.0, every=0.02),
                             "momentum-distribution": MomentumDistribution(ctl, start=0.04,
                                                                           every=0.04)}
        if mode == "host":
            ctl.run()
        else:
            monitor = run_with_device_monitor(ctl)
            assert set(monitor._device_accumulators) == {"g2", "momentum-distribution"}
        out[mode] = ctl
    h, d = out["host"], out["device"]
    assert d.state.step == h.state.step < 400
    for name in ("g2", "momentum-distribution"):
        sh, sd = h._accumulators[name].state_dict(), d._accumulators[name].state_dict()
        assert (sd["samples"], sd["t_first"], sd["t_last"]) == (sh["samples"], sh["t_first"],
                                                                  sh["t_last"]), name
        for key in sh:
            if key.startswith("sum"):
                np.testing.assert_allclose(sd[key], sh[key], rtol=1e-12, atol=0)
    assert set(d.accumulated) == set(h.accumulated) and h.accumulated
    for key in h.accumulated:
        np.testing.assert_allclose(np.asarray(d.accumulated[key].value),
                                   np.asarray(h.accumulated[key].value), rtol=1e-12, atol=1e-300)
