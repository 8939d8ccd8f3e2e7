"""Host logic of the uneven-size sweep (no GPU): member expansion, tile-shape candidates,
override validation.  Mirrors ``tests/unit/test_sweep.py`` of the reference for the
product/zip expansion and its errors (``polarism/sweep.py:98-138``)."""
from __future__ import annotations

import pytest

from polarism_gb300 import host
from polarism_gb300.sweep import Sweep, tiling_candidates


def test_product_and_zip_expansion_in_deterministic_order():
    cfg = host.Config()
    s = Sweep(cfg, {"grid.nx": [128, 256], "laser.P0": [0.1, 0.2, 0.3]})
    assert [m["grid.nx"] for m in s.members] == [128, 128, 128, 256, 256, 256]
    assert [m["laser.P0"] for m in s.members] == [0.1, 0.2, 0.3] * 2
    z = Sweep(cfg, {"grid.nx": [128, 256], "noise.seed": [4, 5]}, mode="zip")
    cfgs = z.member_configs()
    assert [(c.grid.nx, c.noise.seed) for c in cfgs] == [(128, 4), (256, 5)]
    assert cfg.grid.nx == 256  # the base config is untouched


def test_sweep_argument_errors():
    cfg = host.Config()
    with pytest.raises(ValueError):
        Sweep(cfg, {"grid.nx": [1]}, mode="cartesian")
    with pytest.raises(ValueError):
        Sweep(cfg, {"grid.nx": []})
    with pytest.raises(ValueError):
        Sweep(cfg, {"grid.nx": [1, 2], "laser.P0": [1]}, mode="zip")
    with pytest.raises(ValueError):
        Sweep(cfg, {"grid.unknown": [1]}).member_configs()


def test_tiling_candidates_respect_member_widths():
    grids = [(128, 128, 1, 1), (256, 256, 1, 1), (512, 512, 1, 1)]
    cands = tiling_candidates(grids)
    assert (512, 8) in cands and (512, 512) in cands and (1024, 512) in cands
    assert all(l in (512, 1024) for l, _ in cands)
    narrow = tiling_candidates([(64, 64, 1, 1), (512, 64, 1, 1)])
    assert {l for l, _ in narrow} == {512} and max(h for _, h in narrow) == 64
    assert tiling_candidates([(1024, 32, 1, 1), (64, 32, 1, 1)]) == []
