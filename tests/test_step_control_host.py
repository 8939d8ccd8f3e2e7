"""The product's adaptive trial-size controller against the oracle's (itself pinned to the
reference's accepted / rejected trial counts): the same trial sizes, decisions and landings on
output ticks for a synthetic error model, including rejections, tick clamping and dt_max."""
from __future__ import annotations

import math

import pytest

from oracle import gpe


class _State:
    def __init__(self):
        self.t = 0.0


def _error(h, t):
    # A smooth error model with a stiff stretch between t = 0.3 and t = 0.5.
    scale = 40.0 if 0.3 < t < 0.5 else 1.0
    return scale * (h / 0.013) ** 5


@pytest.mark.parametrize("dt,dt_max", [(0.01, None), (0.05, 0.02), (0.002, None)])
def test_controller_matches_oracle_trial_for_trial(dt, dt_max):
    from polarism_gb300.step_control import StepController

    ticks = [0.1 * k for k in range(1, 11)]
    ours = StepController(dt, dt_max)
    ref = gpe.StepControl(dt, dt_max, 5, 4)
    st = _State()
    trials_ours, trials_ref = [], []

    def step_fn(state, h):
        err = _error(h, state.t)
        trials_ref.append((state.t, h, err <= 1))
        if err <= 1:
            state.t += h
        return err

    t = 0.0
    for target in ticks:
        gpe.ifrk_adaptive_advance(st, ref, step_fn, target)
        while t < target:
            h, clamped, proposal = ours.propose(t, target)
            err = _error(h, t)
            accepted = err <= 1
            trials_ours.append((t, h, accepted))
            if accepted:
                t = target if clamped else t + h
            ours.update(h, clamped, proposal, accepted, err)
        assert math.isclose(t, st.t, rel_tol=0, abs_tol=0)
    assert len(trials_ours) == len(trials_ref)
    for a, b in zip(trials_ours, trials_ref):
        assert a[1] == b[1] and a[2] == b[2]
    assert ours.accepted == ref.accepted and ours.rejected == ref.rejected
    assert ours.rejected > 0
    if dt_max is not None:
        assert max(h for _, h, _ in trials_ours) <= dt_max


def test_controller_state_round_trip():
    from polarism_gb300.step_control import StepController

    a = StepController(0.01)
    for err in (0.5, 2.0, 0.1, 0.9):
        h, clamped, proposal = a.propose(0.0, 1.0)
        a.update(h, clamped, proposal, err <= 1, err)
    b = StepController(0.5)
    b.load_state_dict(a.state_dict())
    assert b.propose(0.2, 1.0) == a.propose(0.2, 1.0)
    assert b.statistics == a.statistics
