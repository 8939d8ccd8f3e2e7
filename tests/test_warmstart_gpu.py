"""The learned warm start end to end on a small case (64^2, Gaussian pumps at 2-3 x threshold):
solver-made steady states, FNO training on the GPU kernels, and the judged comparison of
time to the steady-state criterion of ``SimulationController._check_steady_state``
(``polarism/simulation_controller.py:710-734``, rtol 1e-6 per 10 ps) from the plain noise start
and from the warm start, a warm result accepted only at steady density within 1e-3 (relative
L2) of the plain result, a rejected member charged both runs.  The warm start is the network's psi
rescaled to a steady state's particle balance, with n_R from the reservoir's stationary
relation (``warmstart.amplitude_balance``, ``reservoir_closure``).

The runs step in FP64: in FP32 the rounding of every step keeps the slowest condensate modes
moving by about the criterion itself, and most members never meet it (2 of 16 in 12000 ps,
against 16 of 16 within 3760 ps in FP64, on this family of pumps).
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _members(count, seed, total_time=6000.0):
    from polarism_gb300 import warmstart as ws

    cfgs = ws.pump_members(count, seed, n=64, length=64.0, dt=0.02, total_time=total_time,
                           kinds=("gaussian",))
    rng = np.random.default_rng(seed)
    p_th = ws.threshold(cfgs[0].physics)
    for c in cfgs:
        c.laser.profile = {"type": "gaussian", "sigma": float(rng.uniform(10.0, 14.0))}
        c.laser.P0 = float(rng.uniform(2.0, 3.0) * p_th)
    return cfgs


def test_warm_start_reaches_the_criterion_sooner_at_equal_steady_density(cuda_lib):
    from polarism_gb300 import warmstart as ws

    train, test = _members(48, seed=3), _members(8, seed=4)
    assert all(c.solver.precision == "double" for c in train + test)
    data = ws.run_uniform(train)
    keep = np.isfinite(data.stop_times) & (data.final_norms > 1e-6)
    assert keep.sum() >= 40  # the plain solver makes the training targets
    a = ws.features([c for c, k in zip(train, keep) if k])
    y = ws.targets(list(data.psi[keep]), list(data.reservoir[keep]))
    model = ws.WarmStart(64, width=32, modes=16, layers=4, hidden=64, seed=0)
    losses = model.fit(a, y, epochs=150, batch=8, lr=3e-3)
    assert np.mean(losses[-5:]) < 1e-2 * np.mean(losses[:5])

    plain = ws.run_uniform(test)
    valid = np.isfinite(plain.stop_times) & (plain.final_norms > 1e-6)
    assert valid.all()  # every held-out member lases and meets the criterion from noise
    ev = ws.evaluate(model, test, plain)
    print("plain stop (ps)", plain.stop_times.tolist(), "warm stop (ps)", ev.warm_time.tolist(),
          "density error", np.round(ev.density_error, 6).tolist(), "accepted", ev.accepted.tolist(),
          "time ratio", round(ev.speedup_time, 3))
    assert ev.accepted.sum() >= 6
    acc = ev.accepted
    assert np.all(ev.warm_time[acc] < ev.plain_time[acc])
    assert np.all(ev.density_error[acc] <= 1e-3)
    assert ev.speedup_time >= 2.8
