"""Uneven-size sweep: members of different grids in one persistent launch per RK4 step.

Checks, through the C ABI:
* each member matches the FP64 oracle (``oracle.gpe.rk4_advance``, the reference rk4-fdm
  restated, with the single-precision noise realisation) within 1e-4 relative L2;
* each member is bitwise identical to the same member stepped alone by the full-width kernel
  (the sweep kernel does the same arithmetic in the same order);
* tile shapes, graph vs plain launches and frozen members change nothing else, bitwise;
* the FP64 steady-state check matches NumPy, and the sweep driver records stop times as
  ``SimulationController._check_steady_state`` does (``polarism/simulation_controller.py:710-734``).
"""
from __future__ import annotations

import numpy as np
import pytest

from oracle import gpe
from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu

SIZES = [(128, 128), (256, 64), (64, 128), (128, 96), (512, 16), (256, 256), (64, 64)]


def _members(seed=3, sizes=SIZES):
    from polarism_gb300.engine import MemberPhysics

    rng = np.random.default_rng(seed)
    out = []
    for m, (nx, ny) in enumerate(sizes):
        dx = 0.8 + 0.1 * m
        dy = 0.7 + 0.05 * m
        phys = MemberPhysics(R=0.02 * (1 + 0.1 * m), gamma_C=0.083 * (1 - 0.05 * m), g_C=0.001 * (1 + 0.2 * m))
        x = (np.arange(nx) - nx / 2) * dx
        y = (np.arange(ny) - ny / 2) * dy
        X, Y = np.meshgrid(x, y)
        sigma = 6.0 + 2 * m
        envelope = np.exp(-0.5 * (X ** 2 + Y ** 2) / sigma ** 2)
        psi = 0.05 * (rng.standard_normal((ny, nx)) + 1j * rng.standard_normal((ny, nx)))
        psi += 0.3 * np.exp(-0.5 * (X ** 2 + Y ** 2) / (2 * sigma) ** 2)
        res = 0.5 * envelope * rng.uniform(0.5, 1.5, size=(ny, nx))
        out.append(dict(nx=nx, ny=ny, dx=dx, dy=dy, physics=phys, envelope=envelope,
                        psi=psi.astype(np.complex64), res=res.astype(np.float32),
                        p0=0.05 * (1 + 0.3 * m), seed=1000 + 17 * m, strength=1.0 + 0.5 * m))
    return out


def _sweep(members, dt=2e-3, noise=True):
    from polarism_gb300.sweep import SweepEngine

    eng = SweepEngine([(m["nx"], m["ny"], m["dx"], m["dy"]) for m in members],
                      [m["physics"] for m in members], dt)
    eng.set_pump([m["envelope"] for m in members])
    if noise:
        eng.set_noise([m["seed"] for m in members], [m["physics"].gamma_C for m in members],
                      [m["physics"].R for m in members], [m["strength"] for m in members])
    eng.set_state([m["psi"] for m in members], [m["res"] for m in members])
    return eng


def _scales(members, steps):
    p0 = np.asarray([m["p0"] for m in members])
    return np.broadcast_to(p0, (steps, 3, len(members))).copy()


def test_members_match_fp64_oracle(cuda_lib):
    members = _members()
    dt, steps = 2e-3, 12
    eng = _sweep(members, dt)
    eng.advance(0, steps, _scales(members, steps))
    psi, res = eng.get_state()
    for m, mem in enumerate(members):
        p = mem["physics"].__dict__
        noise = gpe.Noise([mem["seed"]], [p["gamma_C"]], [p["R"]], [mem["strength"]], dt,
                          mem["dx"] * mem["dy"], "double", normals_precision="single")
        pump = mem["envelope"] * mem["p0"]
        psi_ref, fields = gpe.rk4_advance(mem["psi"].astype(np.complex128)[None, None],
                                          (mem["res"].astype(np.float64)[None, None],),
                                          lambda t: pump, 0.0, p, mem["dx"], mem["dy"], dt, 0, steps,
                                          noise=noise)
        assert rel_l2(psi[m], psi_ref[0, 0]) < 1e-4, (m, mem["nx"], mem["ny"])
        assert rel_l2(res[m], fields[0][0, 0]) < 1e-4, (m, mem["nx"], mem["ny"])
    eng.close()


def test_members_bitwise_equal_full_width_kernel(cuda_lib):
    from polarism_gb300.engine import RK4Engine

    members = [m for m in _members() if m["nx"] in (128, 256, 512) and m["ny"] >= 4]
    dt, steps = 2e-3, 10
    eng = _sweep(members, dt)
    eng.advance(5, steps, _scales(members, steps))
    psi, res = eng.get_state()
    for m, mem in enumerate(members):
        alone = RK4Engine(mem["nx"], mem["ny"], 1, mem["dx"], mem["dy"], dt, mem["physics"], "single")
        alone.set_kernel(2)
        alone.set_pump(mem["envelope"].astype(np.float32))
        alone.set_noise([mem["seed"]], mem["physics"].gamma_C, mem["physics"].R, mem["strength"],
                        dt / (4 * mem["dx"] * mem["dy"]))
        alone.set_state(mem["psi"][None, None], mem["res"][None, None])
        alone.advance(5, steps, np.full((steps, 3, 1), mem["p0"]))
        p1, r1 = alone.get_state()
        assert np.array_equal(p1[0, 0], psi[m]), (mem["nx"], mem["ny"])
        assert np.array_equal(r1[0, 0], res[m]), (mem["nx"], mem["ny"])
        alone.close()
    eng.close()


def test_tilings_graphs_and_frozen_members_are_bitwise_neutral(cuda_lib):
    members = _members()
    steps = 9
    ref = _sweep(members)
    ref.advance(0, steps, _scales(members, steps), use_graphs=False)
    psi_ref, res_ref = ref.get_state()
    ref.close()
    for lanes, rows in [(512, 8), (512, 24), (512, 64), (1024, 16), (1024, 512)]:
        if lanes == 1024 and min(m["nx"] for m in members) < 128:
            continue
        eng = _sweep(members)
        eng.set_tiling(lanes, rows)
        assert eng.tiling["lanes"] == lanes and eng.tiling["strip_rows"] == rows
        eng.advance(0, steps, _scales(members, steps), use_graphs=True)
        psi, res = eng.get_state()
        for m in range(len(members)):
            assert np.array_equal(psi[m], psi_ref[m]) and np.array_equal(res[m], res_ref[m]), (lanes, rows, m)
        eng.close()
    wide = [m for m in members if m["nx"] >= 128]
    ref = _sweep(wide)
    ref.advance(0, steps, _scales(wide, steps))
    psi_w, res_w = ref.get_state()
    ref.close()
    eng = _sweep(wide)
    eng.set_tiling(1024, 32)
    eng.advance(0, steps, _scales(wide, steps))
    psi, res = eng.get_state()
    for m in range(len(wide)):
        assert np.array_equal(psi[m], psi_w[m]) and np.array_equal(res[m], res_w[m])
    eng.close()
    # A frozen member keeps its state; the others are unaffected by its absence.
    eng = _sweep(members)
    eng.advance(0, 3, _scales(members, 3))
    psi3, res3 = eng.get_state()
    active = np.ones(len(members), dtype=bool)
    active[1] = False
    eng.set_active(active)
    eng.advance(3, steps - 3, _scales(members, steps - 3))
    psi, res = eng.get_state()
    assert np.array_equal(psi[1], psi3[1]) and np.array_equal(res[1], res3[1])
    for m in range(len(members)):
        if m != 1:
            assert np.array_equal(psi[m], psi_ref[m]), m
    eng.set_active(None)
    assert eng.tiling["items"] > 0
    eng.close()


def test_steady_check_matches_numpy(cuda_lib):
    members = _members(seed=8)
    eng = _sweep(members)
    rd, rn, n0 = eng.steady_check()
    assert np.all(np.isinf(rd)) and np.all(np.isinf(rn))
    psi0, _ = eng.get_state()
    eng.advance(0, 4, _scales(members, 4))
    psi1, _ = eng.get_state()
    rd, rn, n1 = eng.steady_check()
    for m, mem in enumerate(members):
        rho0 = (psi0[m].real * psi0[m].real + psi0[m].imag * psi0[m].imag).astype(np.float64)
        rho1 = (psi1[m].real * psi1[m].real + psi1[m].imag * psi1[m].imag).astype(np.float64)
        cell = mem["dx"] * mem["dy"]
        # The device squares in FP32 (possibly fused), so densities agree to FP32 rounding;
        # the sums over them are FP64.
        assert abs(n0[m] - rho0.sum() * cell) <= 1e-6 * rho0.sum() * cell
        assert abs(n1[m] - rho1.sum() * cell) <= 1e-6 * rho1.sum() * cell
        d = np.sqrt(((rho1 - rho0) ** 2).sum()) / np.sqrt((rho0 ** 2).sum())
        assert abs(rd[m] - d) <= 1e-5 * d
        assert abs(rn[m] - abs(n1[m] - n0[m]) / n0[m]) <= 1e-12 + 1e-6 * rn[m]
    eng.close()


def test_autotune_restores_state_and_picks_a_candidate(cuda_lib, tmp_path, monkeypatch):
    from polarism_gb300.sweep import autotune_tiling, tiling_candidates

    monkeypatch.setenv("XDG_CACHE_HOME", str(tmp_path))
    members = _members(sizes=[(128, 128), (256, 256), (512, 64)])
    eng = _sweep(members)
    before = eng.get_packed_state()
    out = autotune_tiling(eng, steps=4, repeats=1)
    after = eng.get_packed_state()
    assert np.array_equal(before[0], after[0]) and np.array_equal(before[1], after[1])
    cands = tiling_candidates(eng.grids)
    assert (out["lanes"], out["strip_rows"]) in cands
    assert len(out["timings"]) == len(cands)
    assert eng.tiling["lanes"] == out["lanes"]
    cached = autotune_tiling(eng, steps=4, repeats=1)
    assert cached["timings"] is None and cached["lanes"] == out["lanes"]
    eng.close()


def test_run_sweep_records_stop_times_like_the_controller(cuda_lib, tmp_path, monkeypatch):
    from polarism_gb300 import host
    from polarism_gb300.sweep import Sweep

    monkeypatch.setenv("XDG_CACHE_HOME", str(tmp_path))
    cfg = host.Config()
    cfg.solver.precision = "single"
    cfg.solver.dt = 1e-3
    cfg.solver.total_time = 0.2
    cfg.noise.stochastic = "wigner"
    cfg.stop.steady_state = True
    cfg.stop.check_every = 0.05
    cfg.stop.rtol = 1e30           # every member passes at the first comparison
    cfg.laser.P0 = 0.03
    sweep = Sweep(cfg, {"grid.nx": [128, 256, 64], "grid.ny": [128, 64, 64],
                        "grid.lx": [100.0, 200.0, 50.0], "noise.seed": [1, 2, 3]}, mode="zip")
    results = sweep.run(autotune=False)
    assert len(results) == 3
    assert results[1]["psi"].shape == (1, 64, 256) and results[1]["reservoir"][0].shape == (64, 256)
    # First check (t = 0.05) only stores the reference; the first comparison is at t = 0.1.
    assert np.allclose(sweep.stop_times, 0.1)
    assert sweep.result.steps == 100
    # rtol = 0: nobody stops, the run goes to total_time.
    cfg.stop.rtol = 0.0
    sweep = Sweep(cfg, {"grid.nx": [128, 64], "grid.ny": [128, 64], "noise.seed": [1, 2]}, mode="zip")
    sweep.run(autotune=False, freeze_stopped=True)
    assert np.all(np.isnan(sweep.stop_times)) and sweep.result.steps == 200


def _relaxing_members():
    """Uneven members relaxing to the fixed point of a near-uniform pump at three strengths
    (they stop at different checks), with a smooth initial field and reservoir."""
    from polarism_gb300 import host

    cfgs, initial = [], []
    for (nx, ny), p0 in zip([(64, 64), (128, 64), (64, 128)], (4.0, 8.0, 16.0)):
        c = host.Config()
        c.grid.nx, c.grid.ny, c.grid.lx, c.grid.ly = nx, ny, float(nx), float(ny)
        c.physics.gamma_R = 0.5
        c.solver.precision = "single"
        c.solver.dt = 0.05
        c.solver.total_time = 200.0
        c.stop.steady_state = True
        c.stop.check_every = 1.0
        c.stop.rtol = 5e-3
        c.laser.P0, c.laser.sigma_space = p0, 1e4
        c.noise.enabled = False
        cfgs.append(c)
        x = np.arange(nx) - nx / 2
        row = (1.0 + 0.02 * np.cos(2 * np.pi * x / nx)).astype(np.complex64)
        initial.append((np.ascontiguousarray(np.broadcast_to(row, (ny, nx))),
                        np.full((ny, nx), 4.0, np.float32)))
    return cfgs, initial


def test_run_sweep_device_monitor_matches_host_decisions_without_waits(cuda_lib, tmp_path,
                                                                        monkeypatch):
    """The sweep's steady-state checks decided on the device stop every member on the same
    check as checks read back to the host, end on the same step with the same state, and make
    no host wait while the chunks and checks are queued (the sweep handle's own counter)."""
    from polarism_gb300.sweep import run_sweep

    monkeypatch.setenv("XDG_CACHE_HOME", str(tmp_path))
    cfgs, initial = _relaxing_members()
    host_run = run_sweep(cfgs, autotune=False, initial=initial, device_monitor=False)
    dev_run = run_sweep(cfgs, autotune=False, initial=initial, device_monitor=True)
    assert np.isfinite(host_run.stop_times).all() and host_run.steps < 4000
    assert len(set(host_run.stop_times.tolist())) == 3
    np.testing.assert_array_equal(dev_run.stop_times, host_run.stop_times)
    assert dev_run.steps == host_run.steps
    for a, b in zip(dev_run.psi + dev_run.reservoir, host_run.psi + host_run.reservoir):
        assert np.array_equal(a, b)
    assert dev_run.loop_syncs == 0
    assert host_run.loop_syncs >= host_run.steps // 20  # a wait at every check

    # Freezing members as their stops show: the same stop times, no wait per chunk.
    frozen = run_sweep(cfgs, autotune=False, initial=initial, freeze_stopped=True)
    np.testing.assert_array_equal(frozen.stop_times, host_run.stop_times)
    assert frozen.steps == host_run.steps and frozen.loop_syncs == 0
