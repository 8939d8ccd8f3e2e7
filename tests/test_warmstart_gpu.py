"""The learned warm start end to end on a small case (64^2, Gaussian pumps): solver-made
targets, FNO training on the GPU kernels, prediction and the judged warm-start run.

What the trained network gains over the method without it is measured where it is
deterministic: the warm-start state is much closer to the solver's late-time state than the
plain noise start is (density relative L2), and the warm-started solver run ends near the
plain run's late-time density.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _members(count, seed):
    from polarism_gb300 import warmstart as ws

    cfgs = ws.pump_members(count, seed, n=64, length=64.0, dt=0.02, total_time=1200.0,
                           kinds=("gaussian",))
    rng = np.random.default_rng(seed)
    p_th = ws.threshold(cfgs[0].physics)
    for c in cfgs:
        c.laser.profile = {"type": "gaussian", "sigma": float(rng.uniform(10.0, 14.0))}
        c.laser.P0 = float(rng.uniform(2.0, 3.0) * p_th)
        c.stop.rtol = 0.0  # run every member to the total time
    return cfgs


def test_warm_start_beats_the_noise_start(cuda_lib):
    from polarism_gb300 import warmstart as ws

    train = _members(48, seed=3)
    test = _members(8, seed=4)
    data = ws.run_uniform(train)
    ref = ws.run_uniform(test)
    a, y = ws.features(train), ws.targets(list(data.psi), list(data.reservoir))
    model = ws.WarmStart(64, width=16, modes=8, layers=4, hidden=32, seed=0)
    losses = model.fit(a, y, epochs=60, batch=8, lr=3e-3)
    assert np.mean(losses[-6:]) < 0.5 * np.mean(losses[:6])  # last epoch vs first
    psi, n_r = model.predict(ws.features(test))
    warm_err = np.array([ws.density_error(psi[i], ref.psi[i]) for i in range(len(test))])
    from polarism_gb300 import host

    noise = [host.make_initial_psi((64, 64), 1e-3, c.noise.seed, np.complex64, np.float32) for c in test]
    plain_err = np.array([ws.density_error(noise[i], ref.psi[i]) for i in range(len(test))])
    lasing = ref.final_norms > 1e-3 * ref.final_norms.max()
    print("lasing", lasing, "prediction error", np.round(warm_err, 3), "noise-start error",
          np.round(plain_err, 3))
    assert lasing.sum() >= 4
    assert np.median(warm_err[lasing]) < 0.5 and np.all(plain_err[lasing] > 0.99)
    # The judged warm-start run ends near the plain run's late-time density.
    warm = ws.run_uniform(test, initial=(psi, n_r))
    final_err = np.array([ws.density_error(warm.psi[i], ref.psi[i]) for i in range(len(test))])
    print("after the warm-started run", np.round(final_err, 4))
    assert np.median(final_err[lasing]) < 0.5
