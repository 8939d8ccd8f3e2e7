"""The steady-state stop of ``SimulationController.run`` kept on the device.

``SimulationController.run`` (``polarism/simulation_controller.py:1063-1130``) advances the
solver to each ``stop.check_every`` boundary and then calls ``_check_steady_state``
(:710-734): it takes |psi|^2 on the host, compares it with the previous check's density and
norms, and records the first stop time of every member that meets the criterion
(``_record_stops``, :698-708); the loop ends once every member has one.  Driving a GB300
drop-in that way costs host waits every chunk: the solver copies the state back after each
``advance`` so that the check can read it.

:class:`DeviceSteadyMonitor` leaves the controller's loop as it is and changes what its
steps do:

* the solver keeps its state in device memory between ``advance`` calls (its resident mode),
  so a chunk is queued without a wait;
* ``_check_steady_state`` queues ``pg_steady_update`` behind the chunk -- the same relative
  density and norm changes (FP64 sums), the same criterion and the first stop step, kept in
  device memory -- and reads the monitor's mapped progress word without waiting;
* the check that finds every member stopped sets the solver's halt word, after which the
  steps the host has already queued leave the state as it was.  When the progress word shows
  it, the monitor waits once, fills ``controller.stop_times``, and puts the state of the
  deciding check back into the controller's state with that check's ``step`` and ``t``: the
  loop then ends where the reference's ends;
* the controller's ``g2`` and ``momentum-distribution`` accumulators sum on the device
  (``pg_accumulate``, FP64, queued behind the chunk like the checks; samples queued after the
  halting check add nothing) and receive the sums and sample counts when the run settles;
* whatever else of the controller reads the state (result recording, event views, checkpoints,
  other accumulators) first copies the device state back.

A run that ends before every member has stopped settles at its last step, before ``run``
prints and stores the stop times.  A run ended by a signal settles when ``run`` returns.
"""
from __future__ import annotations

import functools

import numpy as np

from polarism_gb300.sampling import check_interval


def _to_host(array):
    if hasattr(array, "__cuda_array_interface__"):
        return array.detach().cpu().numpy() if hasattr(array, "detach") else np.asarray(array.get())
    return np.asarray(array)


class DeviceSteadyMonitor:
    """Install on a ``SimulationController`` (the reference's, or any object with its ``cfg``,
    ``state``, ``model``, ``solver``, ``stop_times``, ``_steady_*`` attributes and ``run``)
    whose solver is a GB300 drop-in that can keep its state resident (``rk4-cuda``,
    ``split-step-fft``).  ``poll_every``: checks between reads of the progress word."""

    #: Controller methods that read the state and therefore copy the device state back first.
    READERS = ("_record_results", "_event_view", "save_checkpoint")
    #: Accumulators (``polarism/results/accumulators.py``) whose sums the library forms on the
    #: device: name -> the sums they hold.
    DEVICE_ACCUMULATORS = {"g2": ("sum_density", "sum_density_squared"),
                           "momentum-distribution": ("sum_k",)}

    def __init__(self, controller, poll_every: int = 1):
        solver = controller.solver
        if not getattr(solver, "supports_resident", False):
            raise ValueError(f"{getattr(solver, 'name', type(solver).__name__)} cannot keep its "
                             "state on the device between chunks")
        if not controller.cfg.stop.steady_state:
            raise ValueError("the controller's stop.steady_state is off")
        self.controller = controller
        self.solver = solver
        self.poll_every = max(1, int(poll_every))
        self.checks = 0          # checks queued in the current run
        self.settles = 0         # waits for the device's decisions
        self._saved = {}
        self._started = False
        self._settled = False
        self._halted = False
        self._n_steps = 0
        self._interval = 0
        self._accumulator_updates = []
        self._device_accumulators = {}   # name -> accumulator summed on the device
        self._samples = {}               # name -> [(step, t)] of the samples queued this run
        self._before = {}                # name -> (samples, t_first, t_last) before them
        self._zeroed = False

    # ------------------------------------------------------------------ installation
    def install(self):
        ctl = self.controller
        self._patch("_check_steady_state", self._check)
        for name in self.READERS:
            if hasattr(ctl, name):
                self._patch(name, self._flushing(getattr(ctl, name), timed=name == "_record_results"))
        self._patch("run", self._wrap_run(ctl.run))
        self._patch_object(self.solver, "advance", self._wrap_advance(self.solver.advance))
        self.solver.resident = True
        return self

    def uninstall(self):
        """Copy the state back, leave resident mode and restore the patched methods."""
        ctl = self.controller
        self.solver.release_resident(ctl.model, ctl.state)
        for (obj, name), (had, old) in self._saved.items():
            if had:
                setattr(obj, name, old)
            else:
                delattr(obj, name)
        self._saved.clear()

    def _patch(self, name, fn):
        self._patch_object(self.controller, name, fn)

    def _patch_object(self, obj, name, fn):
        key = (obj, name)
        if key not in self._saved:
            had = name in vars(obj)
            self._saved[key] = (had, vars(obj).get(name))
        setattr(obj, name, fn)

    def _flushing(self, method, timed=False):
        """``method`` after a copy back; ``timed``: its first argument is the time of the
        state it records, which after a halt is the deciding check's, not the step the host
        had queued up to."""
        @functools.wraps(method)
        def wrapper(*args, **kwargs):
            self.flush()
            if timed and args and self._halted:
                args = (self.controller.state.t,) + tuple(args[1:])
            return method(*args, **kwargs)
        return wrapper

    def _wrap_run(self, run):
        @functools.wraps(run)
        def wrapper(*args, **kwargs):
            self._begin()
            try:
                result = run(*args, **kwargs)
            except BaseException:
                try:
                    self.settle()
                except Exception:
                    pass
                raise
            finally:
                self._end()
            self.settle()
            return result
        return wrapper

    def _wrap_advance(self, advance):
        @functools.wraps(advance)
        def wrapper(model, state, n_steps):
            advance(model, state, n_steps)
            # The run's last step with no check after it: settle before the loop ends.
            if (self._n_steps and state.step >= self._n_steps
                    and (not self._interval or state.step % self._interval)):
                self.settle()
        return wrapper

    def _begin(self):
        ctl = self.controller
        dt = float(ctl.cfg.solver.dt)
        self._n_steps = int(round(float(ctl.cfg.solver.total_time) / dt))
        self._interval = check_interval(float(ctl.cfg.stop.check_every), dt)
        self._started = False
        self._settled = False
        self._halted = False
        self.checks = 0
        # Accumulators read the state after the advances they follow: g2 and the momentum
        # distribution (one of each) sum on the device, the others see the copied-back state.
        self._device_accumulators = {}
        self._samples = {}
        self._before = {}
        self._zeroed = False
        for accumulator in getattr(ctl, "_accumulators", {}).values():
            update = accumulator.update
            self._accumulator_updates.append((accumulator, "update", "update" in vars(accumulator),
                                              update))
            name = getattr(accumulator, "name", "")
            if name in self.DEVICE_ACCUMULATORS and name not in self._device_accumulators:
                self._device_accumulators[name] = accumulator
                self._samples[name] = []
                accumulator.update = self._device_update(name, update)
                # The controller asks for results when the loop ends (its sample counts are
                # kept current): the device sums come in first.
                results = getattr(accumulator, "results", None)
                if results is not None:
                    self._accumulator_updates.append((accumulator, "results",
                                                      "results" in vars(accumulator), results))
                    accumulator.results = self._settled_first(results)
            else:
                accumulator.update = self._flushing(update)

    def _end(self):
        for accumulator, attr, had, method in reversed(self._accumulator_updates):
            if had:
                setattr(accumulator, attr, method)
            else:
                delattr(accumulator, attr)
        self._accumulator_updates.clear()

    def _settled_first(self, method):
        @functools.wraps(method)
        def wrapper(*args, **kwargs):
            self.settle()
            return method(*args, **kwargs)
        return wrapper

    def _device_update(self, name, host_update):
        """An accumulator sample queued on the device (before any chunk there is no device
        state yet: that sample is taken on the host, as the reference takes it)."""
        def update(state, t):
            engine = self.solver.engine
            if engine is None or not self.solver._stale and self.solver._held is None:
                return host_update(state, t)
            if not self._zeroed:
                engine.accumulator_zero()
                self._zeroed = True
            accumulator = self._device_accumulators[name]
            if not self._samples[name]:
                self._before[name] = (accumulator.samples, accumulator.t_first, accumulator.t_last)
            engine.accumulate(density=name == "g2", momentum=name == "momentum-distribution")
            self._samples[name].append((int(state.step), t))
            # The sample count and times as the accumulator's own update keeps them.
            if accumulator.samples == 0:
                accumulator.t_first = t
            accumulator.t_last = t
            accumulator.samples += 1
        return update

    def _finish_accumulators(self, halt_step):
        """Add the device sums and the samples taken up to the halting check (all, without a
        halt) to each device-summed accumulator (one wait)."""
        if not self._zeroed:
            return
        engine = self.solver.engine
        kinds = {"sum_density": "rho", "sum_density_squared": "rho2", "sum_k": "k"}
        for name, accumulator in self._device_accumulators.items():
            if not self._samples[name]:
                continue
            taken = [(s, t) for s, t in self._samples[name] if halt_step is None or s <= halt_step]
            samples, t_first, t_last = self._before[name]
            values = dict(accumulator.state_dict())
            for key in self.DEVICE_ACCUMULATORS[name]:
                sums, _ = engine.accumulator_sums(kinds[key])
                host = _to_host(values[key])
                values[key] = host + sums.reshape(np.shape(host))
            values["samples"] = int(samples) + len(taken)
            values["t_first"] = t_first if samples else (taken[0][1] if taken else None)
            values["t_last"] = taken[-1][1] if taken else t_last
            accumulator.load_state_dict(values)
            self._samples[name] = []
        self._zeroed = False

    # ------------------------------------------------------------------ the check
    def _start(self, engine):
        """Reset the device monitor, carrying over a reference density and the stops the
        controller already has (a resumed or continued run)."""
        ctl = self.controller
        engine.steady_reset()
        density = getattr(ctl, "_steady_density", None)
        known = np.isfinite(ctl.stop_times)
        if density is not None or known.any():
            dt = float(ctl.cfg.solver.dt)
            stops = np.where(known, np.round((np.nan_to_num(ctl.stop_times) - ctl.state.t0) / dt),
                             -1).astype(np.int64)
            norms = None if density is None else np.atleast_1d(_to_host(ctl._steady_norm))
            engine.steady_import(None if density is None else _to_host(density), norms, stops)
        self._started = True

    def _check(self):
        """Replacement of ``SimulationController._check_steady_state``: queue the check."""
        ctl = self.controller
        state = ctl.state
        engine = self.solver.engine
        if not self._started:
            self._start(engine)
        stop = ctl.cfg.stop
        engine.steady_update(state.step, record=state.t >= stop.min_time, rtol=float(stop.rtol),
                             halt=True)
        ctl._steady_last_step = state.step
        self.checks += 1
        last = bool(self._n_steps) and state.step >= self._n_steps
        if last or self.checks % self.poll_every == 0:
            stopped, _ = engine.steady_poll()
            if last or stopped == engine.members:
                self.settle()

    # ------------------------------------------------------------------ settling
    def _collect(self):
        """Wait for the queued checks and copy their first stop steps into the controller's
        stop times (where it has none yet).  Returns the halting check's step, or None."""
        ctl = self.controller
        engine = self.solver.engine
        _, _, _, stops, halt_step = engine.steady_results()
        new = (stops >= 0) & np.isnan(ctl.stop_times)
        ctl.stop_times[new] = ctl.state.t0 + stops[new] * float(ctl.cfg.solver.dt)
        return halt_step

    def flush(self):
        """Before anything else of the controller reads the state: the device's stop
        decisions so far go into ``stop_times`` (an event that records stops must see them
        first, as it would after the reference's own checks), and the device state is copied
        back into the controller's state and reservoir.  If a check has halted the run, this
        settles it."""
        ctl = self.controller
        if self._started and not self._settled:
            halt_step = self._collect()
            if halt_step is not None:
                self._settle_halted_or_final(halt_step)
                return
        self.solver.flush(ctl.model, ctl.state)

    def settle(self):
        """Wait for the queued checks; record the stop times; when the device halted, move
        the state back to the deciding check."""
        if self._settled or not self._started:
            if not self._started:
                self._finish_accumulators(None)
                self.solver.flush(self.controller.model, self.controller.state)
            return
        self._settle_halted_or_final(self._collect())

    def _settle_halted_or_final(self, halt_step):
        ctl = self.controller
        state = ctl.state
        engine = self.solver.engine
        self.settles += 1
        self._finish_accumulators(halt_step)
        if halt_step is not None:
            state.step = int(halt_step)
            state.t = state.t0 + state.step * float(ctl.cfg.solver.dt)
            ctl._steady_last_step = state.step
            self._halted = True
        self.solver.flush(ctl.model, state)
        density, norms, _ = engine.steady_export()
        if density is not None:
            shape = np.shape(_to_host(state.psi))
            ctl._steady_density = density.reshape(shape)
            ctl._steady_norm = np.atleast_1d(norms).copy()
        self._settled = True


def run_with_device_monitor(controller, poll_every: int = 1):
    """``controller.run()`` with the steady-state stop on the device; returns the monitor."""
    monitor = DeviceSteadyMonitor(controller, poll_every).install()
    try:
        controller.run()
    finally:
        monitor.uninstall()
    return monitor
