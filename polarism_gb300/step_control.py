"""Adaptive trial-size control for the Lawson IFRK solver.

Same PI feedback, clamping and tick landing as ``polarism/solver/step_controller.py:9-81``:
factor = 0.9 err^(-0.7/k) err_prev^(0.4/k) clamped to [0.2, 5] after an accepted trial,
max(0.2, 0.9 err^(-1/k)) (and no growth on the next success) after a rejection, with
k = min(order, embedded order) + 1; a trial that reaches the output tick is clamped to it.
Used when Polarism's own ``StepController`` is not installed.
"""
from __future__ import annotations

import math
import sys


class StepController:
    def __init__(self, dt, dt_max=None, order=5, embedded_order=4):
        self.dt_max = dt_max
        self.h_next = min(dt, dt_max or math.inf)
        self.k = min(order, embedded_order) + 1
        self.err_prev = 1.0
        self.no_growth = False
        self.accepted = 0
        self.rejected = 0
        self.dt_min = math.inf
        self.dt_max_used = 0.0
        self.dt_last = 0.0

    @property
    def statistics(self):
        return dict(accepted=self.accepted, rejected=self.rejected, dt_min=self.dt_min,
                    dt_max=self.dt_max_used, dt_last=self.dt_last)

    def state_dict(self):
        return dict(h_next=self.h_next, err_prev=self.err_prev, **self.statistics)

    def load_state_dict(self, values):
        self.h_next = float(values["h_next"])
        self.err_prev = float(values["err_prev"])
        self.no_growth = False
        self.accepted = int(values["accepted"])
        self.rejected = int(values["rejected"])
        self.dt_min = float(values["dt_min"])
        self.dt_max_used = float(values["dt_max"])
        self.dt_last = float(values["dt_last"])

    def propose(self, t, target):
        """Trial size and whether it lands on the tick."""
        proposal = self.h_next
        clamped = proposal >= target - t
        h = target - t if clamped else proposal
        if h < 16 * sys.float_info.epsilon * max(1, abs(t)):
            raise RuntimeError(f"adaptive step size underflow at t={t}")
        return h, clamped, proposal

    def update(self, h, clamped, proposal, accepted, error):
        if error is None or not math.isfinite(error) or error < 0:
            error = math.inf
        if accepted:
            self.accepted += 1
            self.dt_min = min(self.dt_min, h)
            self.dt_max_used = max(self.dt_max_used, h)
            self.dt_last = h
            factor = 5.0 if error == 0 else 0.9 * error ** (-0.7 / self.k) * self.err_prev ** (0.4 / self.k)
            factor = min(5.0, max(0.2, factor))
            if self.no_growth:
                factor = min(1.0, factor)
            self.err_prev = max(error, 1e-4)
            self.no_growth = False
        else:
            self.rejected += 1
            factor = min(1.0, max(0.2, 0.9 * error ** (-1 / self.k)))
            self.no_growth = True
        h_next = h * factor
        if accepted and clamped:
            h_next = max(h_next, proposal)
        self.h_next = min(h_next, self.dt_max or math.inf)
