"""Host logic of the device-resident sampling loop (``polarism_gb300/sampling.py``): the chunk
schedule of ``SimulationController.run`` (``polarism/simulation_controller.py:1063-1130``), the
``min_time`` gate and first-stop rule of ``_record_stops`` (:698-708), and the early end once
every member has stopped.  A scripted stand-in for the device monitor replaces the GPU."""
from __future__ import annotations

import numpy as np
import pytest

from polarism_gb300 import sampling


def test_chunk_ends_follow_the_check_grid():
    assert list(sampling.chunk_ends(0, 50, 20)) == [20, 40, 50]
    assert list(sampling.chunk_ends(15, 50, 20)) == [20, 40, 50]
    assert list(sampling.chunk_ends(40, 40, 20)) == []


def test_check_interval_requires_a_whole_number_of_steps():
    assert sampling.check_interval(10.0, 0.01) == 1000
    with pytest.raises(ValueError):
        sampling.check_interval(0.015, 0.01)


class ScriptedMonitor:
    """Stands in for RK4Engine: member m's criterion holds from step reach[m] on."""

    def __init__(self, reach):
        self.reach = np.asarray(reach)
        self.members = len(reach)
        self.step = 0
        self.advanced = []

    def steady_reset(self):
        self.stops = np.full(self.members, -1, dtype=np.int64)
        self.halt_step = None
        self.updates = 0
        self.have_old = False

    def advance(self, start, n, scales, use_graphs=True):
        assert np.shape(scales) == (n, 3, self.members)
        self.advanced.append((start, n))
        if self.halt_step is None:
            self.step = start + n

    def steady_update(self, step, record, rtol, halt):
        if self.halt_step is not None:
            return
        self.updates += 1
        if self.have_old and record:
            newly = (self.stops < 0) & (step >= self.reach)
            self.stops[newly] = step
        self.have_old = True
        if halt and (self.stops >= 0).all():
            self.halt_step = step

    def steady_poll(self):
        return int((self.stops >= 0).sum()), self.updates

    def steady_results(self):
        z = np.zeros(self.members)
        return z, z, z, self.stops.copy(), self.halt_step


def _scales(m):
    return lambda a, b: np.ones((b - a, 3, m))


def test_run_ends_on_the_deciding_check():
    eng = ScriptedMonitor([60, 140, 100])
    run = sampling.run_to_steady(eng, 0, 1000, _scales(3), 0.5, 20, 1e-6, poll_every=1)
    assert run.halted and run.final_step == 140
    assert run.stop_steps.tolist() == [60, 140, 100]
    np.testing.assert_allclose(run.stop_times, [30.0, 70.0, 50.0])
    assert eng.advanced[-1] == (120, 20)  # polled after every check: nothing queued past 140


def test_first_check_only_sets_the_reference_and_min_time_gates_records():
    eng = ScriptedMonitor([0, 0])
    run = sampling.run_to_steady(eng, 0, 200, _scales(2), 1.0, 20, 1e-6, min_time=70.0,
                                 poll_every=1)
    assert run.stop_steps.tolist() == [80, 80]  # checks at 20..60 are before min_time
    eng = ScriptedMonitor([0, 0])
    run = sampling.run_to_steady(eng, 0, 200, _scales(2), 1.0, 20, 1e-6, poll_every=1)
    assert run.stop_steps.tolist() == [40, 40]  # no decision on the first check


def test_lagging_poll_queues_extra_chunks_that_do_nothing():
    eng = ScriptedMonitor([60, 60])
    run = sampling.run_to_steady(eng, 0, 1000, _scales(2), 1.0, 20, 1e-6, poll_every=4)
    assert run.final_step == 60 and eng.step == 60
    assert len(eng.advanced) == 4  # the host learnt of the stop at its fourth check


def test_without_halt_the_run_reaches_the_end():
    eng = ScriptedMonitor([60, 60])
    run = sampling.run_to_steady(eng, 0, 200, _scales(2), 1.0, 20, 1e-6, halt=False)
    assert not run.halted and run.final_step == 200 and run.stop_steps.tolist() == [60, 60]
    assert np.isnan(sampling.run_to_steady(ScriptedMonitor([10 ** 6]), 0, 100, _scales(1), 1.0, 20,
                                           1e-6).stop_times).all()
