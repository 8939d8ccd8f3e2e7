"""Learned warm start: an FNO proposes the steady state of a pump, the plain solver finishes.

Pipeline (none of it replaces reference code; Polarism has no learned component):

1. :func:`pump_members` draws sweep members with random pumps -- a Gaussian spot, a ring or a
   square lattice of spots (pitch 8-20 um) -- at P0 uniform in [1, 3] x the uniform-pump
   threshold ``gamma_R gamma_C / R`` (``polarism/analysis/condensation.py:52-57``).
2. The solver makes the training data: :func:`polarism_gb300.sweep.run_sweep` integrates every
   member from the reference's seeded noise start to the steady-state criterion of
   ``SimulationController._check_steady_state`` (``polarism/simulation_controller.py:710-734``).
   The stop times of this run are the plain-start times.
3. :class:`WarmStart` trains the FNO (:mod:`polarism_gb300.fno`, BF16 tensor-core GEMMs) to map
   ``(P(x)/P_th, x, y)`` to the steady ``(Re psi, Im psi, n_R)``, with psi's global phase fixed
   (the phase at the density maximum set to zero: steady states are stationary only up to a
   global phase rotation).
4. :func:`evaluate` starts held-out members from the prediction -- psi from the network,
   rescaled to the particle balance of a steady state (:func:`amplitude_balance`), n_R from psi
   through the reservoir's own steady-state relation (:func:`reservoir_closure`) --
   runs the same solver to the same criterion and accepts a warm result only when it reached
   the criterion (the stationarity residual) and its steady density is within ``density_tol``
   (relative L2) of the plain-start result; otherwise the member falls back to the plain start
   and is charged both runs.

The runs that make and judge steady states step in FP64 (``solver.precision = "double"``).  In
FP32 the rounding of every step keeps the slowest condensate modes moving by about the
criterion itself (relative density change 1e-6 per 10 ps): of sixteen 64^2 Gaussian-pump
members, two met it within 12000 ps in FP32 and all sixteen within 3760 ps in FP64, and the
FP32 states that had not met it still drifted by 1e-5 over the next 4000 ps.
"""
from __future__ import annotations

import copy
import math
import time
from dataclasses import dataclass

import numpy as np

from polarism_gb300 import host, sampling


def threshold(physics) -> float:
    return float(physics.gamma_R * physics.gamma_C / physics.R)


def pump_members(count, seed, n=256, length=128.0, dt=0.01, total_time=4000.0, check_every=10.0,
                 rtol=1e-6, kinds=("gaussian", "ring", "lattice"), eta=0.02, precision="double"):
    """Host-mirror configs of ``count`` members with random pumps (numpy ``default_rng(seed)``).

    The physics constants are Polarism's defaults plus kinetic relaxation ``eta`` (the
    ``kinetic_relaxation_eta`` term of ``polarism/model.py:89-127``): without energy relaxation
    the vortices seeded by the noise start keep moving and most lasing members never become
    stationary, so there would be no steady state to learn."""
    rng = np.random.default_rng(seed)
    base = host.Config()
    base.physics.kinetic_relaxation_eta = eta
    p_th = threshold(base.physics)
    out = []
    for i in range(count):
        c = copy.deepcopy(base)
        c.grid.nx = c.grid.ny = n
        c.grid.lx = c.grid.ly = length
        c.solver.dt, c.solver.precision, c.solver.total_time = dt, precision, total_time
        c.noise.seed = int(seed) * 1_000_003 + i
        c.noise.stochastic = "none"
        c.stop.steady_state, c.stop.rtol, c.stop.check_every = True, rtol, check_every
        kind = kinds[int(rng.integers(len(kinds)))]
        c.laser.laser_type = "profile"
        if kind == "gaussian":
            c.laser.profile = {"type": "gaussian", "sigma": float(rng.uniform(8.0, 20.0))}
        elif kind == "ring":
            c.laser.profile = {"type": "ring", "radius": float(rng.uniform(0.12, 0.27) * length),
                               "width": float(rng.uniform(3.0, 6.0))}
        else:
            pitch = float(rng.uniform(8.0, 20.0))
            c.laser.profile = {"type": "lattice", "constant": pitch, "width": pitch / 4.0}
        c.laser.P0 = float(rng.uniform(1.0, 3.0) * p_th)
        out.append(c)
    return out


def features(cfgs):
    """Network inputs (M, 3, n, n) float32: the pump in threshold units and the coordinates."""
    grid = host.PeriodicGrid(cfgs[0].grid)
    half = 0.5 * cfgs[0].grid.lx
    out = np.empty((len(cfgs), 3, grid.ny, grid.nx), dtype=np.float32)
    for m, c in enumerate(cfgs):
        laser = host.make_laser(c.laser, grid.X, grid.Y, "double")
        out[m, 0] = laser._spatial_envelope * (c.laser.P0 / threshold(c.physics))
        out[m, 1] = grid.X / half
        out[m, 2] = grid.Y / half
    return out


def phase_fixed(psi):
    """psi with the phase at its density maximum rotated to zero."""
    psi = np.asarray(psi)
    k = int(np.argmax(np.abs(psi)))
    ref = psi.reshape(-1)[k]
    return psi * (np.conj(ref) / abs(ref)) if abs(ref) > 0 else psi


def targets(psi_list, n_list):
    out = np.empty((len(psi_list), 3) + np.shape(psi_list[0]), dtype=np.float32)
    for m, (psi, n) in enumerate(zip(psi_list, n_list)):
        p = phase_fixed(psi)
        out[m, 0], out[m, 1], out[m, 2] = p.real, p.imag, n
    return out


class WarmStart:
    """The FNO plus the per-channel output scales it was trained with."""

    def __init__(self, n, width=32, modes=16, layers=4, hidden=128, seed=0):
        from polarism_gb300.fno import FNO2d

        self.net = FNO2d(n, c_in=3, c_out=3, width=width, modes=modes, layers=layers, hidden=hidden,
                         seed=seed)
        self.scale = np.ones(3, dtype=np.float32)

    def fit(self, a, y, epochs=20, batch=16, lr=1e-3, seed=0, log=None):
        """Adam on the scaled squared error; cosine-decayed learning rate.  Returns losses."""
        torch = self.net.torch
        self.scale = np.maximum(np.sqrt(np.mean(y.astype(np.float64) ** 2, axis=(0, 2, 3))), 1e-12).astype(np.float32)
        ys = y / self.scale.reshape(1, 3, 1, 1)
        dev = self.net.device
        A = torch.tensor(np.ascontiguousarray(a), device=dev)
        Y = torch.tensor(np.ascontiguousarray(ys, dtype=np.float32), device=dev)
        rng = np.random.default_rng(seed)
        steps = epochs * max(1, len(a) // batch)
        losses, k = [], 0
        for epoch in range(epochs):
            order = rng.permutation(len(a))
            for s in range(0, len(order) - batch + 1, batch):
                idx = torch.tensor(order[s:s + batch], device=dev)
                xa, xy = A.index_select(0, idx).contiguous(), Y.index_select(0, idx).contiguous()
                out, cache = self.net.forward(xa)
                loss, grad = self.net.mse(out, xy)
                rate = lr * 0.5 * (1 + math.cos(math.pi * k / steps))
                self.net.adam_step(self.net.backward(cache, grad), lr=rate)
                losses.append(loss)
                k += 1
            if log:
                log(f"epoch {epoch}: loss {np.mean(losses[-max(1, len(a) // batch):]):.4e}")
        return losses

    def predict(self, a, batch=16):
        """(psi (M, n, n) complex64, n_R (M, n, n) float32, clamped at zero)."""
        torch = self.net.torch
        dev = self.net.device
        outs = []
        for s in range(0, len(a), batch):
            x = torch.tensor(np.ascontiguousarray(a[s:s + batch]), device=dev)
            out, _ = self.net.forward(x, keep=False)
            outs.append(out.cpu().numpy())
        o = np.concatenate(outs) * self.scale.reshape(1, 3, 1, 1)
        psi = (o[:, 0] + 1j * o[:, 1]).astype(np.complex64)
        return psi, np.maximum(o[:, 2], 0).astype(np.float32)

    def loss(self, a, y, batch=16):
        torch = self.net.torch
        ys = (y / self.scale.reshape(1, 3, 1, 1)).astype(np.float32)
        total = 0.0
        for s in range(0, len(a), batch):
            x = torch.tensor(np.ascontiguousarray(a[s:s + batch]), device=self.net.device)
            t = torch.tensor(np.ascontiguousarray(ys[s:s + batch]), device=self.net.device)
            out, _ = self.net.forward(x, keep=False)
            total += self.net.mse(out, t, want_grad=False)[0] * len(x)
        return total / len(a)


@dataclass
class UniformResult:
    psi: np.ndarray          # (M, n, n) complex64
    reservoir: np.ndarray    # (M, n, n) float32
    stop_times: np.ndarray   # NaN where the criterion was not reached
    final_norms: np.ndarray
    t: float
    wall_time: float


def run_uniform(cfgs, initial=None, total_time=None):
    """Advance same-size members (one ``pg_solver``, per-member pumps and constants; the tiled
    RK4 kernel carries the kinetic-relaxation term) to the steady-state criterion of
    ``SimulationController._check_steady_state``.  Every member keeps stepping until all have
    a stop time or the total time is reached, as in the reference; a member's stop time is its
    first qualifying check (the first comparison is at the second check)."""
    from polarism_gb300.engine import Engine, MemberPhysics

    c0 = cfgs[0]
    grid = host.PeriodicGrid(c0.grid)
    dt = float(c0.solver.dt)
    total = float(c0.solver.total_time if total_time is None else total_time)
    interval = int(round(c0.stop.check_every / dt))
    rtol = float(c0.stop.rtol)
    m = len(cfgs)
    precision = getattr(c0.solver, "precision", "single")
    real = np.float64 if precision == "double" else np.float32
    cplx = np.complex128 if precision == "double" else np.complex64
    lasers = [host.make_laser(c.laser, grid.X, grid.Y, precision) for c in cfgs]
    env = np.stack([l._spatial_envelope for l in lasers])[:, None].astype(real)
    eng = Engine(grid.nx, grid.ny, m, grid.dx, grid.dy, dt,
                 [MemberPhysics.from_object(c.physics) for c in cfgs], precision, pump_per_member=True)
    try:
        eng.set_pump(env)
        if initial is None:
            psi0 = np.stack([host.make_initial_psi(grid.shape, c.noise.initial_amplitude, c.noise.seed,
                                                   cplx, real) for c in cfgs])[:, None]
            n0 = np.zeros((m, 1) + grid.shape, real)
        else:
            psi0 = np.ascontiguousarray(np.asarray(initial[0], cplx).reshape(m, 1, *grid.shape))
            n0 = np.ascontiguousarray(np.asarray(initial[1], real).reshape(m, 1, *grid.shape))
        eng.set_state(psi0, n0)
        p0 = np.asarray([c.laser.P0 for c in cfgs])
        n_total = int(round(total / dt))
        t0 = time.perf_counter()
        run = sampling.run_to_steady(
            eng, 0, n_total, lambda a, b: np.broadcast_to(p0, (b - a, 3, m)), dt, interval, rtol,
            min_time=float(getattr(c0.stop, "min_time", 0.0)))
        wall = time.perf_counter() - t0
        psi, res = eng.get_state()
        return UniformResult(psi[:, 0].copy(), res[:, 0].copy(), run.stop_times, run.norms,
                             run.final_step * dt, wall)
    finally:
        eng.close()


@dataclass
class Evaluation:
    plain_time: np.ndarray
    warm_time: np.ndarray
    accepted: np.ndarray
    density_error: np.ndarray
    cost_time: np.ndarray
    plain_wall: float
    warm_wall: float
    speedup_time: float
    speedup_wall: float


def reservoir_closure(cfgs, psi):
    """n_R where the single reservoir is stationary for the condensate psi:
    dn_R/dt = P - (gamma_R + R |psi|^2) n_R = 0 (``polarism/reservoir/single_reservoir.py``),
    so n_R = P(x) / (gamma_R + R |psi|^2).  It is exact at the steady state, so the warm start
    carries no reservoir error of its own: the reservoir relaxes on the slowest time scale of
    the model (1 / gamma_R = 200 ps with the default constants)."""
    grid = host.PeriodicGrid(cfgs[0].grid)
    out = np.empty((len(cfgs), grid.ny, grid.nx), dtype=np.float64)
    for m, (c, p) in enumerate(zip(cfgs, psi)):
        env = host.make_laser(c.laser, grid.X, grid.Y, "double")._spatial_envelope * c.laser.P0
        out[m] = env / (c.physics.gamma_R + c.physics.R * np.abs(np.asarray(p, np.complex128)) ** 2)
    return out


def amplitude_balance(cfgs, psi, lo=0.25, hi=4.0, iters=60):
    """psi rescaled so that the condensate neither gains nor loses particles with the reservoir
    of :func:`reservoir_closure`: at a steady state of polarism/model.py:89-127,
    dN/dt = sum (R n_R - gamma_C) |psi|^2 + eta (hbar / m) sum n_R Re(psi* lap psi) = 0 (the
    Hamiltonian part conserves N).  With psi -> sqrt(s) psi and n_R = P / (gamma_R + R s |psi|^2)
    this is sum n_R(s) w - gamma_C sum |psi|^2 = 0, w = R |psi|^2 + eta (hbar / m)
    Re(psi* lap psi) (the solver's five-point Laplacian), solved for s by bisection in log s.
    The total population is the slowest thing for a start to get right (it relaxes through the
    reservoir), so a start with the right shape but the wrong amount converges slowly.
    Members without a root in [lo, hi] keep their psi."""
    grid = host.PeriodicGrid(cfgs[0].grid)
    dx, dy = grid.dx, grid.dy
    out = []
    for c, p in zip(cfgs, psi):
        p = np.asarray(p, np.complex128)
        ph = c.physics
        pump = host.make_laser(c.laser, grid.X, grid.Y, "double")._spatial_envelope * c.laser.P0
        rho = np.abs(p) ** 2
        lap = ((np.roll(p, 1, 1) + np.roll(p, -1, 1) - 2 * p) / dx ** 2
               + (np.roll(p, 1, 0) + np.roll(p, -1, 0) - 2 * p) / dy ** 2)
        eta = float(getattr(ph, "kinetic_relaxation_eta", 0.0) or 0.0)
        w = ph.R * rho + eta * (ph.hbar / ph.m_eff) * np.real(np.conj(p) * lap)
        loss = ph.gamma_C * rho.sum()

        def g(s):
            return np.sum(pump * w / (ph.gamma_R + ph.R * s * rho)) - loss

        a, b = np.log(lo), np.log(hi)
        ga, gb = g(lo), g(hi)
        if loss <= 0 or not (ga > 0 > gb):
            out.append(p)
            continue
        for _ in range(iters):
            mid = 0.5 * (a + b)
            if g(np.exp(mid)) > 0:
                a = mid
            else:
                b = mid
        out.append(p * np.sqrt(np.exp(0.5 * (a + b))))
    return np.stack(out)


def density_error(psi_a, psi_b):
    ra, rb = np.abs(psi_a) ** 2, np.abs(psi_b) ** 2
    return float(np.sqrt(np.sum((ra - rb) ** 2)) / max(np.sqrt(np.sum(rb ** 2)), 1e-30))


def evaluate(ws, cfgs, plain, density_tol=1e-3, closure=True, balance=True):
    """Warm-start the members of ``cfgs`` (whose plain-start result is ``plain``, from
    :func:`run_uniform`) and compare.  Only members whose plain run reached a lasing steady
    state enter the ratios (decayed members have no condensate to predict).  ``closure``: the
    warm n_R is :func:`reservoir_closure` of the predicted psi instead of the network's n_R;
    ``balance``: psi is first rescaled by :func:`amplitude_balance`."""
    psi, n_r = ws.predict(features(cfgs))
    if balance:
        psi = amplitude_balance(cfgs, psi)
    if closure:
        n_r = reservoir_closure(cfgs, psi)
    warm = run_uniform(cfgs, initial=(psi, n_r))
    total = float(cfgs[0].solver.total_time)
    m = len(cfgs)
    err = np.array([density_error(warm.psi[i], plain.psi[i]) for i in range(m)])
    reached = np.isfinite(warm.stop_times)
    accepted = reached & (err <= density_tol)
    warm_t = np.where(reached, warm.stop_times, total)
    plain_t = plain.stop_times
    cost = np.where(accepted, warm_t, warm_t + plain_t)
    valid = np.isfinite(plain_t) & (plain.final_norms > 1e-6)
    speed_t = float(np.sum(plain_t[valid]) / max(np.sum(cost[valid]), 1e-30))
    # Wall time: the warm sweep plus, for rejected members, their share of the plain sweep.
    share = np.sum(plain_t[valid & ~accepted]) / max(np.sum(plain_t[valid]), 1e-30)
    warm_wall = warm.wall_time + share * plain.wall_time
    return Evaluation(plain_t, warm_t, accepted, err, cost, plain.wall_time, warm_wall, speed_t,
                      plain.wall_time / max(warm_wall, 1e-30))
