"""FP64 NumPy restatement of the reference's GPE time steppers (oracle; test infrastructure).

All arrays use the reference's canonical layout: condensate ``(B, C, ny, nx)``
complex, reservoir fields ``(B, C_res, ny, nx)`` real.  Physics constants are a
mapping (``hbar``, ``m_eff``, ``g_C`` ...) whose values are scalars or
member-broadcast arrays of shape ``(B, 1, 1, 1)``.

Functions and the reference code each one restates:

* ``laplacian``          -- ``polarism/model.py:210-225`` (periodic five-point)
* ``reservoir_derivatives`` -- ``polarism/reservoir/single_reservoir.py:81-98``,
  ``polarism/reservoir/double_reservoir.py:106-130``
* ``gpe_rhs``            -- ``polarism/model.py:89-127``
* ``rk4_step``           -- ``polarism/solver/rk4_fdm_solver.py:36-82`` plus the
  non-negative clamp of ``single_reservoir.py:70-73``
* ``rk4_advance``        -- ``polarism/solver/abstract_solver.py:83-101`` (noise
  after each accepted step; counter step = pre-step index, density = post-step)
* ``split_step_cpu``     -- ``polarism/solver/split_step_fft_solver.py:97-159``
  (R/2 K/2 N noise K/2 R/2)
* ``split_step_kouter``  -- ``polarism/solver/split_step_fft_cuda_solver.py:106-184``
  and ``:1144-1325`` (K/2 [R/2 N R/2 noise] K/2), the same composition as the
  reference's independent check ``tests/crosscheck/test_split_step_fft_cuda.py:46-70``
* ``ifrk_step``          -- ``polarism/solver/ifrk_fft_cuda_solver.py:96-109,128-241``
  (Lawson integrating-factor RK, stage-coupled reservoir)
* ``ifrk_error``         -- ``polarism/solver/ifrk_fft_cuda_solver.py:243-293``
* ``StepControl``        -- ``polarism/solver/step_controller.py:48-81``
"""
from __future__ import annotations

import math
import sys
from fractions import Fraction

import numpy as np

from oracle.philox import wigner_increment


# --------------------------------------------------------------------------- stencils
def laplacian(f, dx: float, dy: float):
    """Periodic five-point Laplacian over the last two axes."""
    return ((np.roll(f, -1, axis=-2) - 2 * f + np.roll(f, 1, axis=-2)) / dy ** 2
            + (np.roll(f, -1, axis=-1) - 2 * f + np.roll(f, 1, axis=-1)) / dx ** 2)


def _get(p, name, default=0.0):
    return p.get(name, default)


def reservoir_derivatives(kind: str, fields, rho, pump, p, dx, dy):
    """Reservoir time derivatives; state order is (n_R,) or (n_A, n_I)."""
    if kind == "none":
        return ()
    if kind == "single":
        (n,) = fields
        dn = pump - (_get(p, "gamma_R") + _get(p, "R") * rho) * n
        if np.any(_get(p, "reservoir_diffusion_R")):
            dn = dn + _get(p, "reservoir_diffusion_R") * laplacian(n, dx, dy)
        return (dn,)
    if kind == "double":
        n_a, n_i = fields
        dn_i = pump - (_get(p, "gamma_I") + _get(p, "R_IA")) * n_i + _get(p, "R_AI") * n_a
        dn_a = _get(p, "R_IA") * n_i - (_get(p, "gamma_A") + _get(p, "R_AI") + _get(p, "R") * rho) * n_a
        if np.any(_get(p, "reservoir_diffusion_I")):
            dn_i = dn_i + _get(p, "reservoir_diffusion_I") * laplacian(n_i, dx, dy)
        if np.any(_get(p, "reservoir_diffusion_A")):
            dn_a = dn_a + _get(p, "reservoir_diffusion_A") * laplacian(n_a, dx, dy)
        return (dn_a, dn_i)
    if kind == "quadratic-double":
        # polarism/reservoir/quadratic_double_reservoir.py:13-14,160-164: state (n_R, n_I).
        n_r, n_i = fields
        transfer = _get(p, "kappa") * n_i * n_i
        dn_r = transfer - _get(p, "gamma_R") * n_r - _get(p, "R") * n_r * rho
        dn_i = pump - transfer - _get(p, "gamma_I") * n_i
        return (dn_r, dn_i)
    raise ValueError(f"unsupported reservoir {kind!r}")


def _active(kind, fields):
    return 0.0 if kind == "none" else fields[0]


def _inactive(kind, fields):
    return fields[1] if kind in ("double", "quadratic-double") else 0.0


def gpe_rhs(psi, fields, pump, potential, p, dx, dy, kind="single"):
    """Finite-difference scalar right-hand side d(psi, fields)/dt."""
    hbar, m = _get(p, "hbar"), _get(p, "m_eff")
    rho = psi.real * psi.real + psi.imag * psi.imag
    dres = reservoir_derivatives(kind, fields, rho, pump, p, dx, dy)
    n_a, n_i = _active(kind, fields), _inactive(kind, fields)
    lap = laplacian(psi, dx, dy)
    kinetic = -(hbar ** 2) / (2 * m) * lap
    eff = potential + _get(p, "g_C") * np.abs(psi) ** 2 + _get(p, "g_R") * n_a + _get(p, "g_I") * n_i
    gain = (_get(p, "R") * n_a - _get(p, "gamma_C")) / 2.0
    dpsi = (-1j / hbar) * (kinetic + eff * psi) + gain * psi
    eta = _get(p, "kinetic_relaxation_eta")
    if np.any(eta):
        dpsi = dpsi + eta * n_a * (hbar / (2.0 * m)) * lap
    return dpsi, dres


# --------------------------------------------------------------------------- RK4 (rk4-fdm)
def rk4_step(psi, fields, pump_at, potential, p, dx, dy, dt, t, kind="single"):
    """One classic RK4 step with the reservoir advanced through the same stages.

    ``pump_at(t)`` returns the pump array at time ``t``.  Intermediate reservoir
    stages are not clamped; the final reservoir is clamped at zero.
    """
    def add(a, b, s):
        return tuple(x + s * y for x, y in zip(a, b))

    k1, r1 = gpe_rhs(psi, fields, pump_at(t), potential, p, dx, dy, kind)
    k2, r2 = gpe_rhs(psi + 0.5 * dt * k1, add(fields, r1, 0.5 * dt), pump_at(t + 0.5 * dt),
                     potential, p, dx, dy, kind)
    k3, r3 = gpe_rhs(psi + 0.5 * dt * k2, add(fields, r2, 0.5 * dt), pump_at(t + 0.5 * dt),
                     potential, p, dx, dy, kind)
    k4, r4 = gpe_rhs(psi + dt * k3, add(fields, r3, dt), pump_at(t + dt), potential, p, dx, dy, kind)
    psi_new = psi + (dt / 6.0) * (k1 + 2 * k2 + 2 * k3 + k4)
    fields_new = tuple(np.maximum(f0 + (dt / 6.0) * (a + 2 * b + 2 * c + d), 0)
                       for f0, a, b, c, d in zip(fields, r1, r2, r3, r4))
    return psi_new, fields_new


class Noise:
    """Per-member Wigner noise parameters (``polarism/noise/stochastic.py:15-37``)."""

    def __init__(self, seeds, gamma, scattering, strength, dt, cell_volume,
                 precision="double", normals_precision=None):
        self.seeds = np.asarray(seeds, dtype=np.uint64)
        self.gamma = np.asarray(gamma, dtype=np.float64)
        self.scattering = np.asarray(scattering, dtype=np.float64)
        self.strength = np.asarray(strength, dtype=np.float64)
        self.dt = float(dt)
        self.cell_volume = float(cell_volume)
        self.precision = precision
        self.normals_precision = normals_precision

    def apply(self, field, active, step):
        wigner_increment(field, active, step, self.seeds, self.gamma, self.scattering,
                         self.strength, self.dt, self.cell_volume, self.precision,
                         self.normals_precision)


def rk4_advance(psi, fields, pump_at, potential, p, dx, dy, dt, start_step, n_steps,
                t0=0.0, kind="single", noise: Noise | None = None, norm_trace=None):
    """Advance ``n_steps`` RK4 steps; returns (psi, fields).

    ``norm_trace`` (a list) receives the per-member norm sum |psi|^2 dx dy after each step.
    """
    for k in range(n_steps):
        step = start_step + k
        psi, fields = rk4_step(psi, fields, pump_at, potential, p, dx, dy, dt, t0 + step * dt, kind)
        if noise is not None:
            noise.apply(psi, _active(kind, fields), step)
        if norm_trace is not None:
            norm_trace.append(norm(psi, dx, dy))
    return psi, fields


def norm(psi, dx, dy):
    """Per-member total density sum |psi|^2 dV (``simulation_controller.py:92-103``)."""
    return np.sum(np.abs(psi) ** 2, axis=tuple(range(1, psi.ndim))) * dx * dy


# --------------------------------------------------------------------------- split step
def kinetic_half(k_squared, p, dt):
    """exp(-i hbar k^2 (dt/2) / (2 m)) (``split_step_fft_solver.py:54-61``)."""
    return np.exp(-1j * _get(p, "hbar") * k_squared * (dt / 2) / (2 * _get(p, "m_eff")))


def _kick(psi, half):
    return np.fft.ifft2(np.fft.fft2(psi, axes=(-2, -1)) * half, axes=(-2, -1))


def reservoir_half_step(kind, fields, psi, pump, h, p, dx, dy):
    """Midpoint RK2 over ``h`` at frozen psi with the final clamp
    (``single_reservoir.py:100-111``)."""
    if kind == "none":
        return ()
    rho = psi.real * psi.real + psi.imag * psi.imag
    k1 = reservoir_derivatives(kind, fields, rho, pump, p, dx, dy)
    mid = tuple(f + 0.5 * h * k for f, k in zip(fields, k1))
    k2 = reservoir_derivatives(kind, mid, rho, pump, p, dx, dy)
    return tuple(np.maximum(f + h * k, 0) for f, k in zip(fields, k2))


def nonlinear_step(psi, fields, potential, p, dt, kind="single"):
    """Exact local step psi * exp(g dt - i phi) with the expm1 phase time."""
    hbar = _get(p, "hbar")
    n_a, n_i = _active(kind, fields), _inactive(kind, fields)
    rho = np.abs(psi) ** 2
    gain = (_get(p, "R") * n_a - _get(p, "gamma_C")) / 2.0 + np.imag(potential) / hbar
    x = 2 * gain * dt
    small = np.abs(x) < 1e-6
    phase_time = dt * np.where(small, 1 + x / 2 + x * x / 6, np.expm1(x) / np.where(small, 1, x))
    phase = ((np.real(potential) + _get(p, "g_R") * n_a + _get(p, "g_I") * n_i) * dt
             + _get(p, "g_C") * rho * phase_time) / hbar
    return psi * np.exp(gain * dt - 1j * phase)


def split_step_cpu(psi, fields, pump_at, potential, p, k_squared, dx, dy, dt, t, step,
                   kind="single", noise: Noise | None = None):
    """The reference CPU ordering R/2 K/2 N [noise] K/2 R/2."""
    half = kinetic_half(k_squared, p, dt)
    fields = reservoir_half_step(kind, fields, psi, pump_at(t + dt / 4), dt / 2, p, dx, dy)
    psi = _kick(psi, half)
    psi = nonlinear_step(psi, fields, potential, p, dt, kind)
    if noise is not None:
        noise.apply(psi, _active(kind, fields), step)
    psi = _kick(psi, half)
    fields = reservoir_half_step(kind, fields, psi, pump_at(t + 3 * dt / 4), dt / 2, p, dx, dy)
    return psi, fields


def split_step_kouter(psi, fields, pump_at, potential, p, k_squared, dx, dy, dt, t, step,
                      kind="single", noise: Noise | None = None):
    """The reference GPU ordering K/2 R/2 N R/2 [noise] K/2."""
    half = kinetic_half(k_squared, p, dt)
    psi = _kick(psi, half)
    fields = reservoir_half_step(kind, fields, psi, pump_at(t + dt / 4), dt / 2, p, dx, dy)
    psi = nonlinear_step(psi, fields, potential, p, dt, kind)
    fields = reservoir_half_step(kind, fields, psi, pump_at(t + 3 * dt / 4), dt / 2, p, dx, dy)
    if noise is not None:
        noise.apply(psi, _active(kind, fields), step)
    psi = _kick(psi, half)
    return psi, fields


def split_advance(ordering, psi, fields, pump_at, potential, p, k_squared, dx, dy, dt,
                  start_step, n_steps, t0=0.0, kind="single", noise=None, norm_trace=None):
    step_fn = split_step_cpu if ordering == "cpu" else split_step_kouter
    for k in range(n_steps):
        step = start_step + k
        psi, fields = step_fn(psi, fields, pump_at, potential, p, k_squared, dx, dy, dt,
                              t0 + step * dt, step, kind, noise)
        if norm_trace is not None:
            norm_trace.append(norm(psi, dx, dy))
    return psi, fields


# --------------------------------------------------------------------------- IFRK (Lawson)
RK4_TABLEAU = dict(
    A=[[0, 0, 0, 0], [Fraction(1, 2), 0, 0, 0], [0, Fraction(1, 2), 0, 0], [0, 0, 1, 0]],
    b=[Fraction(1, 6), Fraction(1, 3), Fraction(1, 3), Fraction(1, 6)],
    c=[0, Fraction(1, 2), Fraction(1, 2), 1], b_hat=None, order=4, embedded_order=None)

DP5_TABLEAU = dict(
    A=[[0] * 7,
       [Fraction(1, 5)] + [0] * 6,
       [Fraction(3, 40), Fraction(9, 40)] + [0] * 5,
       [Fraction(44, 45), Fraction(-56, 15), Fraction(32, 9)] + [0] * 4,
       [Fraction(19372, 6561), Fraction(-25360, 2187), Fraction(64448, 6561),
        Fraction(-212, 729)] + [0] * 3,
       [Fraction(9017, 3168), Fraction(-355, 33), Fraction(46732, 5247), Fraction(49, 176),
        Fraction(-5103, 18656)] + [0] * 2,
       [Fraction(35, 384), 0, Fraction(500, 1113), Fraction(125, 192), Fraction(-2187, 6784),
        Fraction(11, 84), 0]],
    b=[Fraction(35, 384), 0, Fraction(500, 1113), Fraction(125, 192), Fraction(-2187, 6784),
       Fraction(11, 84), 0],
    c=[0, Fraction(1, 5), Fraction(3, 10), Fraction(4, 5), Fraction(8, 9), 1, 1],
    b_hat=[Fraction(5321, 57600), 0, Fraction(7429, 16695), Fraction(1321, 1920),
           Fraction(-126603, 339200), Fraction(121, 700), Fraction(-1, 40)],
    order=5, embedded_order=4)

TABLEAUS = {"rk4": RK4_TABLEAU, "dp5": DP5_TABLEAU}


class IFRKState:
    """Condensate kept as a spectrum between steps, as the reference's state does."""

    def __init__(self, psi=None, psi_k=None, fields=(), t=0.0):
        self.psi = psi
        self.psi_k = psi_k
        self.fields = tuple(fields)
        self.t = t

    def real_space(self):
        return self.psi if self.psi is not None else np.fft.ifft2(self.psi_k, axes=(-2, -1))


def _fft(x):
    return np.fft.fft2(x, axes=(-2, -1))


def _ifft(x):
    return np.fft.ifft2(x, axes=(-2, -1))


def spinor_exponential(kx, ky, p, tau):
    """exp(-i H tau / hbar) of the circular-basis spinor Hamiltonian on the FFT grid,
    H = [[E + Z/2, beta (kx - i ky)^2], [beta (kx + i ky)^2, E - Z/2]], E = hbar^2 k^2 / 2m
    (``polarism/dispersion.py:34-63``), from the identity
    exp(-i t (e I + B)) = exp(-i e t) (cos(w t) I - i sin(w t) / w B) for traceless B with
    B^2 = w^2 I (``polarism/dispersion.py:66-83``).  Returns the (2, 2, ny, nx) matrix."""
    hbar, m = _get(p, "hbar"), _get(p, "m_eff")
    energy = hbar ** 2 * (kx * kx + ky * ky) / (2.0 * m)
    z = _get(p, "zeeman") / 2.0
    upper = _get(p, "te_tm") * (kx - 1j * ky) ** 2
    lower = np.conj(upper)
    omega = np.sqrt(z * z + (upper * lower).real)
    t = tau / hbar
    phase = np.exp(-1j * energy * t)
    cos = np.cos(omega * t)
    sin_over = t * np.sinc(omega * t / np.pi)
    return np.stack((np.stack((phase * (cos - 1j * sin_over * z), -1j * phase * sin_over * upper)),
                     np.stack((-1j * phase * sin_over * lower, phase * (cos + 1j * sin_over * z)))))


def _apply2(matrix, field):
    return np.stack((matrix[0, 0] * field[:, 0] + matrix[0, 1] * field[:, 1],
                     matrix[1, 0] * field[:, 0] + matrix[1, 1] * field[:, 1]), axis=1)


def ifrk_step(state: IFRKState, h, tableau, pump_at, potential, p, k_squared, dx, dy,
              kind="single", adaptive=False, rtol=1e-6, atol=1e-8, spinor=None):
    """One Lawson step of size ``h``.

    Returns the embedded error for adaptive steps (and accepts the step only if
    it is <= 1), otherwise ``None``.

    ``spinor`` (a dict with ``kx``, ``ky`` -- the FFT wavenumber grids -- and ``weights``,
    the per-member pump weights ``(B, 2)`` used when the reservoir has one field per
    component) switches to the two-component field of ``ifrk_fft_cuda_solver.py:96-142``:
    the matrix Lawson factor, the cross-spin term alpha_2 |psi_-+|^2 and per-component
    (or shared, summed-density) reservoirs (``ifrk_fft_cuda_solver.py:118-126``).
    """
    A, b, c = tableau["A"], tableau["b"], tableau["c"]
    hbar, m = _get(p, "hbar"), _get(p, "m_eff")
    rate = -hbar / (2.0 * m)
    spin_cache = {}

    def phase(fraction):
        if spinor is not None:
            key = float(fraction)
            if key not in spin_cache:
                spin_cache[key] = spinor_exponential(spinor["kx"], spinor["ky"], p, h * key)
            return spin_cache[key]
        return np.exp(1j * rate * (h * float(fraction)) * k_squared)

    def lin(fraction, field):
        return _apply2(phase(fraction), field) if spinor is not None else phase(fraction) * field

    def res_derivs(res_i, rho, pump):
        if spinor is None:
            return reservoir_derivatives(kind, res_i, rho, pump, p, dx, dy)
        if kind == "none":
            return ()
        if res_i[0].shape[1] == 2:
            weights = np.asarray(spinor["weights"], dtype=np.float64).reshape(-1, 2, 1, 1)
            return reservoir_derivatives(kind, res_i, rho, pump * weights, p, dx, dy)
        return reservoir_derivatives(kind, res_i, rho.sum(axis=1, keepdims=True), pump, p, dx, dy)

    psi0 = state.psi
    psi0_k = state.psi_k if state.psi_k is not None else _fft(psi0)
    if state.psi_k is not None:
        psi0 = None
    res0 = state.fields
    f, derivs = [], []
    for i, ci in enumerate(c):
        stage_time = state.t + float(ci) * h
        if i == 0 and psi0 is not None:
            psi_i, psi_i_k = psi0, psi0_k
        else:
            psi_i_k = lin(ci, psi0_k)
            for j in range(i):
                if A[i][j]:
                    psi_i_k = psi_i_k + (h * float(A[i][j])) * lin(ci - c[j], f[j])
            psi_i = _ifft(psi_i_k)
        res_i = tuple(r0 + sum((h * float(A[i][j])) * derivs[j][q] for j in range(i) if A[i][j])
                      for q, r0 in enumerate(res0))
        rho = psi_i.real * psi_i.real + psi_i.imag * psi_i.imag
        n_a, n_i = _active(kind, res_i), _inactive(kind, res_i)
        eff = potential + _get(p, "g_C") * rho + _get(p, "g_R") * n_a + _get(p, "g_I") * n_i
        if spinor is not None:
            eff = eff + _get(p, "alpha_2") * rho[:, ::-1]
        gain = 0.5 * (_get(p, "R") * n_a - _get(p, "gamma_C"))
        rhs = (-1j / hbar) * eff * psi_i + gain * psi_i
        eta = _get(p, "kinetic_relaxation_eta")
        if np.any(eta):
            lap = _ifft(-k_squared * psi_i_k)
            rhs = rhs + eta * n_a * (hbar / (2.0 * m)) * lap
        f.append(_fft(rhs))
        derivs.append(res_derivs(res_i, rho, pump_at(stage_time)))
    psi_new_k = lin(1, psi0_k)
    for j, bj in enumerate(b):
        if bj:
            psi_new_k = psi_new_k + (h * float(bj)) * lin(1 - c[j], f[j])
    res_new = tuple(np.maximum(r0 + sum((h * float(bj)) * derivs[j][q]
                                        for j, bj in enumerate(b) if bj), 0)
                    for q, r0 in enumerate(res0))
    if not adaptive:
        state.psi, state.psi_k, state.fields = None, psi_new_k, res_new
        state.t = state.t + h
        return None
    psi_start = state.psi if state.psi is not None else _ifft(psi0_k)
    psi_new = _ifft(psi_new_k)
    weights = [float(bj - bh) for bj, bh in zip(b, tableau["b_hat"])]
    err = ifrk_error(h, psi_start, psi_new, psi0_k, f, res0, res_new, derivs, weights, c,
                     lin, rtol, atol)
    if err <= 1:
        state.psi, state.psi_k, state.fields = psi_new, psi_new_k, res_new
        state.t = state.t + h
    return err


def ifrk_error(h, psi_start, psi_new, psi0_k, f, res0, res_new, derivs, weights, c, lin,
               rtol, atol):
    """Embedded RMS error, scaled by atol + rtol max(|y0|, |y1|), max over members.
    ``lin(fraction, field)`` applies the Lawson factor of ``(1 - c_j) h``."""
    e_k = np.zeros_like(psi0_k)
    for j, w in enumerate(weights):
        if w:
            e_k = e_k + (h * w) * lin(1 - c[j], f[j])
    e = _ifft(e_k)
    axes = tuple(range(1, psi_new.ndim))

    def scaled(mag, scale):
        return np.where(scale > 0, mag / np.where(scale > 0, scale, 1),
                        np.where(mag == 0, 0, np.inf))

    s = scaled(np.abs(e), atol + rtol * np.maximum(np.abs(psi_start), np.abs(psi_new)))
    squares = np.sum(s * s, axis=axes)
    count = psi_new[0].size
    for q, (r0, r1) in enumerate(zip(res0, res_new)):
        value = np.zeros_like(r0)
        for j, w in enumerate(weights):
            if w:
                value = value + (h * w) * derivs[j][q]
        s = scaled(np.abs(value), atol + rtol * np.maximum(np.abs(r0), np.abs(r1)))
        squares = squares + np.sum(s * s, axis=axes)
        count += r0[0].size
    return float(np.max(np.sqrt(squares / count)))


class StepControl:
    """PI trial-size control with exact landing on output ticks."""

    def __init__(self, dt, dt_max, order, embedded_order):
        self.dt_max = dt_max
        self.h_next = min(dt, dt_max or math.inf)
        self.k = min(order, embedded_order) + 1
        self.err_prev = 1.0
        self.no_growth = False
        self.accepted = 0
        self.rejected = 0

    def trial(self, step_fn, state, target):
        proposal = self.h_next
        clamped = proposal >= target - state.t
        h = target - state.t if clamped else proposal
        if h < 16 * sys.float_info.epsilon * max(1, abs(state.t)):
            raise RuntimeError(f"adaptive step size underflow at t={state.t}")
        err = step_fn(state, h)
        accepted = err is not None and err <= 1
        if accepted and clamped:
            state.t = target
        error = err if (err is not None and math.isfinite(err) and err >= 0) else math.inf
        if accepted:
            self.accepted += 1
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
        return accepted


def ifrk_adaptive_advance(state, control, step_fn, target):
    """Run trials until ``state.t`` lands on ``target``."""
    while state.t < target:
        control.trial(step_fn, state, target)
    return state
