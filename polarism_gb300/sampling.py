"""The sampling loop of ``SimulationController.run`` for the steady-state stop, kept on the
device (``polarism/simulation_controller.py:1063-1130``, ``_check_steady_state`` and
``_record_stops`` at :698-734).

The reference advances one chunk, copies the density to the host side of its array library,
compares it with the previous check and decides the stops before it queues the next chunk.
Here every check is a kernel pair queued behind the chunk it follows (``pg_steady_update``):
the comparison, the stop decision and the first stop step stay in device memory, the host
reads a mapped word (members stopped, newest finished check) without waiting, and the check
that finds every member stopped sets the solver's halt word, after which the RK4 steps the
host has already queued leave the state unchanged.  The run therefore ends on the step of the
deciding check, as the reference's loop does, without a host round trip per chunk.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np


@dataclass
class SteadyRun:
    stop_steps: np.ndarray     # per member, -1 when the member never stopped
    stop_times: np.ndarray     # t0 + stop_step * dt, NaN when the member never stopped
    final_step: int            # step of the state left in the engine
    halted: bool               # every member stopped before the last step
    checks: int                # checks queued
    rel_density: np.ndarray    # newest check's values
    rel_norm: np.ndarray
    norms: np.ndarray


def check_interval(check_every: float, dt: float) -> int:
    """Steps per check; ``check_every`` must be a whole number of steps
    (``polarism/config/validation.py:339-340``)."""
    steps = int(round(check_every / dt))
    if steps <= 0 or not math.isclose(steps * dt, check_every, rel_tol=1e-9):
        raise ValueError("stop.check_every must be a positive multiple of solver.dt")
    return steps


def chunk_ends(step: int, n_steps: int, interval: int):
    """Ends of the chunks the loop advances through: every check step, then ``n_steps``
    (the ``end = min(..., ((step // interval) + 1) * interval)`` rule of the reference)."""
    while step < n_steps:
        step = min(n_steps, (step // interval + 1) * interval)
        yield step


def run_to_steady(engine, start_step: int, n_steps: int, scales_for, dt: float, interval: int,
                  rtol: float, min_time: float = 0.0, t0: float = 0.0, halt: bool = True,
                  poll_every: int = 8, use_graphs: bool = True) -> SteadyRun:
    """Advance ``engine`` (an :class:`~polarism_gb300.engine.RK4Engine`) from ``start_step``
    to ``n_steps`` with a steady-state check every ``interval`` steps.

    ``scales_for(a, b)`` returns the pump coefficients of steps ``a..b-1``, shape
    ``(b - a, 3, members)``.  A check at step ``k`` records stops only when
    ``t0 + k dt >= min_time``.  With ``halt`` the run ends on the check that finds every
    member stopped; the host looks at the device's progress every ``poll_every`` checks
    (without waiting) only to stop queueing work that would do nothing."""
    engine.steady_reset()
    members = engine.members
    step = int(start_step)
    checks = 0
    for end in chunk_ends(step, int(n_steps), int(interval)):
        engine.advance(step, end - step, scales_for(step, end), use_graphs=use_graphs)
        step = end
        if step % interval == 0:
            engine.steady_update(step, record=t0 + step * dt >= min_time, rtol=rtol, halt=halt)
            checks += 1
            if halt and checks % poll_every == 0 and engine.steady_poll()[0] == members:
                break
    rd, rn, norms, stops, halt_step = engine.steady_results()
    final = step if halt_step is None else halt_step
    times = np.where(stops >= 0, t0 + stops * dt, np.nan)
    return SteadyRun(stops, times, int(final), halt_step is not None, checks, rd, rn, norms)
