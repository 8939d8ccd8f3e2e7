"""The host mirror of Polarism's objects (used where Polarism is not installed), on CPU:
batched pump slots, reservoir state semantics and batched simulation construction."""
from __future__ import annotations

import copy

import numpy as np
import pytest


def _cfg(n=16):
    from polarism_gb300.host import Config

    cfg = Config()
    cfg.grid.nx = cfg.grid.ny = n
    cfg.grid.lx = cfg.grid.ly = 20.0
    cfg.laser.P0, cfg.laser.sigma_space = 0.05, 4.0
    cfg.noise.seed = 7
    return cfg


def test_batched_pump_shares_equal_envelopes_and_stacks_different_ones():
    from polarism_gb300.host import build_simulation

    cfg = _cfg()
    same = [copy.deepcopy(cfg) for _ in range(3)]
    for m, c in enumerate(same):
        c.laser.P0 = 0.02 * (m + 1)
        c.noise.seed = 7 + m
    _, model, _ = build_simulation(cfg, same)
    (env, coeff), = model.pump.separable_terms()
    assert np.ndim(env) == 2
    assert np.allclose(coeff(0.3), [0.02, 0.04, 0.06])
    total = model.pump(0.3)
    assert total.shape == (3, 1, 16, 16) and np.allclose(total[2, 0], 0.06 * env)

    diff = [copy.deepcopy(c) for c in same]
    for m, c in enumerate(diff):
        c.laser.sigma_space = 3.0 + m
    _, model2, _ = build_simulation(cfg, diff)
    (env2, coeff2), = model2.pump.separable_terms()
    assert env2.shape == (3, 1, 16, 16)
    assert not np.allclose(env2[0], env2[2])
    assert np.allclose(model2.pump(0.0)[1], coeff2(0.0)[1] * env2[1])


@pytest.mark.parametrize("kind", ["single", "double", "quadratic-double"])
def test_reservoir_set_state_clamps_and_checks_shape(kind):
    from polarism_gb300.host import build_simulation

    cfg = _cfg()
    cfg.reservoir.reservoir_type = kind
    members = [copy.deepcopy(cfg) for _ in range(2)]
    for m, c in enumerate(members):
        c.noise.seed = 7 + m
    _, model, _ = build_simulation(cfg, members)
    res = model.reservoir
    state = tuple(np.asarray(f).copy() for f in res.get_state())
    assert len(state) == (1 if kind == "single" else 2)
    noisy = tuple(f - 0.5 + np.arange(f.size).reshape(f.shape) / f.size for f in state)
    res.set_state(noisy)
    for got, given in zip(res.get_state(), noisy):
        assert np.all(got >= 0)
        assert np.array_equal(got, np.maximum(given, 0).astype(got.dtype))
    with pytest.raises(ValueError):
        res.set_state(tuple(f[:1] for f in noisy))


def test_batched_simulation_state_and_seeds():
    from polarism_gb300.host import build_simulation

    cfg = _cfg()
    members = [copy.deepcopy(cfg) for _ in range(3)]
    for m, c in enumerate(members):
        c.noise.seed = 11 + m
    grid, model, state = build_simulation(cfg, members)
    assert state.field.shape == (3, 1, 16, 16)
    assert not np.allclose(state.field[0], state.field[1])
    single = build_simulation(members[1])[2]
    assert np.array_equal(state.field[1, 0], single.field[0, 0])
    assert grid.shape == (16, 16) and grid.dx == 20.0 / 16
