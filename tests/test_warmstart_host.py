"""Host logic of the learned warm-start protocol, without a GPU: the pump generator, the
network inputs and targets, the density error and the accounting of ``evaluate`` (acceptance
at equal steady density, rejected members charged both runs, decayed members left out)."""
from __future__ import annotations

import numpy as np


def test_pump_members_are_seeded_and_within_the_configured_ranges():
    from polarism_gb300 import warmstart as ws

    a = ws.pump_members(12, seed=3, n=32, length=32.0)
    b = ws.pump_members(12, seed=3, n=32, length=32.0)
    p_th = ws.threshold(a[0].physics)
    assert [c.laser.profile for c in a] == [c.laser.profile for c in b]
    assert [c.laser.P0 for c in a] == [c.laser.P0 for c in b]
    for c in a:
        assert 1.0 * p_th <= c.laser.P0 <= 3.0 * p_th
        assert c.laser.profile["type"] in ("gaussian", "ring", "lattice")
        assert c.physics.kinetic_relaxation_eta == 0.02 and c.noise.stochastic == "none"
        assert c.solver.precision == "double"
    assert len({c.noise.seed for c in a}) == len(a)


def test_reservoir_closure_is_the_stationary_reservoir_of_the_condensate():
    """n_R from psi makes dn_R/dt = P - (gamma_R + R |psi|^2) n_R vanish (single reservoir,
    polarism/reservoir/single_reservoir.py) and is P / gamma_R where psi = 0."""
    from polarism_gb300 import host
    from polarism_gb300 import warmstart as ws

    cfgs = ws.pump_members(3, seed=4, n=16, length=16.0)
    rng = np.random.default_rng(1)
    psi = rng.standard_normal((3, 16, 16)) + 1j * rng.standard_normal((3, 16, 16))
    psi[2] = 0
    n_r = ws.reservoir_closure(cfgs, psi)
    grid = host.PeriodicGrid(cfgs[0].grid)
    for m, c in enumerate(cfgs):
        pump = host.make_laser(c.laser, grid.X, grid.Y, "double")._spatial_envelope * c.laser.P0
        ph = c.physics
        rate = pump - (ph.gamma_R + ph.R * np.abs(psi[m]) ** 2) * n_r[m]
        assert np.max(np.abs(rate)) <= 1e-15 * np.max(pump)
    assert np.allclose(n_r[2], host.make_laser(cfgs[2].laser, grid.X, grid.Y, "double")._spatial_envelope
                       * cfgs[2].laser.P0 / cfgs[2].physics.gamma_R, rtol=1e-15)


def test_features_targets_and_phase_convention():
    from polarism_gb300 import warmstart as ws

    cfgs = ws.pump_members(3, seed=1, n=16, length=16.0)
    f = ws.features(cfgs)
    assert f.shape == (3, 3, 16, 16) and f.dtype == np.float32
    assert np.all(f[:, 0] >= 0) and np.allclose(f[0, 1], f[1, 1]) and np.abs(f[:, 1:]).max() <= 1.0
    rng = np.random.default_rng(0)
    psi = rng.standard_normal((16, 16)) + 1j * rng.standard_normal((16, 16))
    fixed = ws.phase_fixed(psi * np.exp(0.7j))
    k = np.argmax(np.abs(psi))
    assert abs(np.angle(fixed.reshape(-1)[k])) < 1e-12
    assert np.allclose(np.abs(fixed), np.abs(psi))
    t = ws.targets([psi], [np.abs(psi)])
    assert t.shape == (1, 3, 16, 16) and np.allclose(t[0, 0] ** 2 + t[0, 1] ** 2, np.abs(psi) ** 2,
                                                     rtol=1e-5)
    assert ws.density_error(psi, psi) == 0.0
    assert abs(ws.density_error(psi * np.sqrt(1.01), psi) - 0.01) < 1e-12


def test_evaluate_accounting(monkeypatch):
    """Four members: accepted (reached and within 1e-3), rejected for density, rejected for not
    reaching the criterion, and one whose plain run decayed (its warm result may be accepted, but
    a member without a plain steady state stays out of both ratios)."""
    from polarism_gb300 import warmstart as ws

    n, m = 8, 4
    cfgs = ws.pump_members(m, seed=2, n=n, length=8.0, total_time=100.0)
    rng = np.random.default_rng(5)
    steady = rng.standard_normal((m, n, n)) + 1j * rng.standard_normal((m, n, n))
    plain = ws.UniformResult(steady.astype(np.complex64), np.zeros((m, n, n), np.float32),
                             np.array([40.0, 50.0, 60.0, np.nan]),
                             np.array([1.0, 1.0, 1.0, 0.0]), 100.0, 8.0)
    warm_psi = steady.copy()
    warm_psi[1] *= np.sqrt(1.01)  # density 1 % off: rejected
    warm = ws.UniformResult(warm_psi.astype(np.complex64), np.zeros((m, n, n), np.float32),
                            np.array([10.0, 20.0, np.nan, 30.0]),
                            np.array([1.0, 1.0, 1.0, 1.0]), 100.0, 2.0)

    class Fake:
        def predict(self, feats):
            assert feats.shape == (m, 3, n, n)
            return np.zeros((m, n, n), np.complex64), np.zeros((m, n, n), np.float32)

    monkeypatch.setattr(ws, "run_uniform", lambda cfgs_, initial=None, total_time=None: warm)
    ev = ws.evaluate(Fake(), cfgs, plain)
    assert list(ev.accepted) == [True, False, False, True]
    # Charged time: the warm run, plus the plain run where the warm result is rejected; a member
    # that never reached the criterion is charged the whole run time.
    assert np.allclose(ev.warm_time, [10.0, 20.0, 100.0, 30.0])
    assert np.allclose(ev.cost_time[:3], [10.0, 20.0 + 50.0, 100.0 + 60.0])
    assert np.isclose(ev.speedup_time, (40.0 + 50.0 + 60.0) / (10.0 + 70.0 + 160.0))
    share = (50.0 + 60.0) / (40.0 + 50.0 + 60.0)
    assert np.isclose(ev.warm_wall, 2.0 + share * 8.0)
    assert np.isclose(ev.speedup_wall, 8.0 / (2.0 + share * 8.0))


def test_amplitude_balance_restores_the_uniform_steady_population():
    """A uniform condensate under a uniform pump is stationary when R n_R = gamma_C with
    n_R = P / (gamma_R + R |psi|^2), i.e. |psi|^2 = P / gamma_C - gamma_R / R; the balance
    rescales any uniform psi to that density (the Laplacian term vanishes)."""
    from polarism_gb300 import warmstart as ws

    cfgs = ws.pump_members(2, seed=6, n=16, length=16.0)
    for c in cfgs:
        c.laser.profile = {"type": "gaussian", "sigma": 1e9}  # uniform to double precision
    ph = cfgs[0].physics
    psi = np.full((2, 16, 16), 0.3 + 0.4j)
    out = ws.amplitude_balance(cfgs, psi)
    for m, c in enumerate(cfgs):
        expect = c.laser.P0 / ph.gamma_C - ph.gamma_R / ph.R
        assert np.allclose(np.abs(out[m]) ** 2, expect, rtol=1e-12)
        assert np.allclose(np.angle(out[m]), np.angle(psi[m]))
