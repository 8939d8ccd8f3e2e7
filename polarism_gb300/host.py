"""Host-side mirror of the Polarism objects the time-stepping path consumes.

When the Polarism package is installed, its own ``Config``, grid, pump, reservoir,
noise and state objects drive the solvers in :mod:`polarism_gb300.solvers`
directly.  Without it (a bare GPU machine), the classes here provide the same
attribute names and meaning for the part of the API the hot path touches, so the
solvers, tests and benchmark run unchanged:

* ``PhysicsConstants`` and the parameter sections -- ``polarism/config/simulation_parameters.py:30-238``
  (same field names and defaults)
* ``PeriodicGrid`` -- ``polarism/grid/periodic_grid.py:17-69`` (cell-centred
  coordinates, ``k^2`` from ``fftfreq``)
* ``ContinuousGaussian`` / ``PumpField`` -- ``polarism/laser/continuous_gaussian.py:15-46``,
  ``polarism/laser/abstract_laser.py:74-79``, ``polarism/laser/pump_field.py:37-89``
* ``SingleReservoir`` / ``NoReservoir`` -- ``polarism/reservoir/single_reservoir.py:22-111``
  (non-negative clamp in ``set_state``)
* ``NoiseParametersArrays`` -- ``polarism/noise/stochastic.py:15-37``
* ``make_initial_psi`` -- ``polarism/noise/initial_field.py:82-90`` (NumPy
  ``default_rng`` on the host, zero mean, RMS-normalised)
* ``SimulationState`` -- ``polarism/simulation_state.py:20-196`` (canonical ``(B, C, ny, nx)``)
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field, fields
from typing import Any

import numpy as np


# --------------------------------------------------------------------------- config
@dataclass
class GridParameters:
    nx: int = 256
    ny: int = 256
    lx: float = 100.0
    ly: float = 100.0
    grid_type: str = "periodic"
    ndim: int = 2


@dataclass
class PhysicsConstants:
    hbar: float = 0.6582119514
    m_eff: float = 0.284
    gamma_R: float = 0.005
    gamma_C: float = 0.083
    g_C: float = 0.001
    g_R: float = 0.002
    g_I: float = 0.0
    gamma_I: float = 0.001
    gamma_A: float = 0.005
    R: float = 0.02
    R_IA: float = 5e-2
    R_AI: float = 2.5e-3
    kappa: float = 0.05
    kinetic_relaxation_eta: float = 0.0
    reservoir_diffusion_I: float = 0.0
    reservoir_diffusion_A: float = 0.0
    reservoir_diffusion_R: float = 0.0
    dispersion: str = "parabolic"
    spin: str = "scalar"
    alpha_2: float = 0.0
    zeeman: float = 0.0
    te_tm: float = 0.0


@dataclass
class NoiseParameters:
    enabled: bool = True
    seed: int | None = None
    initial: str = "complex_gaussian_zero_mean"
    initial_amplitude: float = 1e-3
    initial_k_cutoff_um: float | None = None
    stochastic: str = "none"
    stochastic_strength: float = 1.0


@dataclass
class LaserParameters:
    laser_type: str = "continuous-gaussian"
    P0: float = 0.4
    x0: float = 0.0
    y0: float = 0.0
    sigma_space: float = 15.0
    delay: float = 0.0
    circular_polarization: float = 0.0
    profile: dict = field(default_factory=dict)
    # pulse-gaussian (polarism/laser/pulse_gaussian.py, peak-amplitude definition)
    Pmax: float = 1.2
    sigma_time: float = 0.1
    pulse_separation: float = 0.6
    cutoff_sigma: float = 3.0
    n_pulses: int = 0
    # mode "multiple": the lasers listed here (the reference reads them from a YAML file,
    # polarism/laser/laser_factory.py:28-34,55-80)
    mode: str = "single"
    lasers: list = field(default_factory=list)


@dataclass
class ReservoirParameters:
    reservoir_type: str = "single"
    components: int | None = None


@dataclass
class PotentialParameters:
    potential_type: str = "zero"


@dataclass
class SolverParameters:
    total_time: float = 5.0
    dt: float = 1e-3
    method: str = "rk4-cuda"
    tableau: str = "rk4"
    precision: str = "double"
    laplacian: str = "five-point"
    cuda_graphs: bool = True
    adaptive: bool = False
    rtol: float = 1e-6
    atol: float = 1e-8
    dt_max: float | None = None


@dataclass
class StopParameters:
    steady_state: bool = False
    rtol: float = 1e-6
    check_every: float = 10.0
    min_time: float = 0.0


@dataclass
class Config:
    grid: GridParameters = field(default_factory=GridParameters)
    physics: PhysicsConstants = field(default_factory=PhysicsConstants)
    noise: NoiseParameters = field(default_factory=NoiseParameters)
    laser: LaserParameters = field(default_factory=LaserParameters)
    reservoir: ReservoirParameters = field(default_factory=ReservoirParameters)
    potential: PotentialParameters = field(default_factory=PotentialParameters)
    solver: SolverParameters = field(default_factory=SolverParameters)
    stop: StopParameters = field(default_factory=StopParameters)


def physics_float_fields():
    return [f.name for f in fields(PhysicsConstants) if f.type in (float, "float")]


# --------------------------------------------------------------------------- grid
class PeriodicGrid:
    """Two-dimensional periodic grid with cell-centred coordinates."""

    boundary = "periodic"
    grid_type = "periodic"
    ndim = 2

    def __init__(self, cfg: GridParameters):
        self.nx, self.ny = int(cfg.nx), int(cfg.ny)
        self.lx, self.ly = float(cfg.lx), float(cfg.ly)
        self.dx = self.lx / self.nx
        self.dy = self.ly / self.ny
        self.shape = (self.ny, self.nx)
        self.spacing = (self.dy, self.dx)
        self.lengths = (self.ly, self.lx)
        x = (np.arange(self.nx, dtype=np.float64) - (self.nx - 1) * 0.5) * self.dx
        y = (np.arange(self.ny, dtype=np.float64) - (self.ny - 1) * 0.5) * self.dy
        self.X, self.Y = np.meshgrid(x, y, indexing="xy")
        self.kx = 2 * np.pi * np.fft.fftfreq(self.nx, d=self.dx)
        self.ky = 2 * np.pi * np.fft.fftfreq(self.ny, d=self.dy)
        self.KX, self.KY = np.meshgrid(self.kx, self.ky, indexing="xy")
        self.k_squared = self.KX ** 2 + self.KY ** 2


def real_dtype(precision: str):
    return np.float32 if precision == "single" else np.float64


def complex_dtype(precision: str):
    return np.complex64 if precision == "single" else np.complex128


# --------------------------------------------------------------------------- pump
class ContinuousGaussian:
    """P(r, t) = coeff(t) exp(-r^2 / (2 sigma^2)), coeff = P0 for t >= delay."""

    time_independent = True

    def __init__(self, cfg: LaserParameters, X, Y, precision="double"):
        self.P0, self.x0, self.y0 = float(cfg.P0), float(cfg.x0), float(cfg.y0)
        self.delay = float(cfg.delay)
        self.sigma_space = float(cfg.sigma_space)
        r2 = (X - self.x0) ** 2 + (Y - self.y0) ** 2
        self._spatial_envelope = np.exp(-0.5 * r2 / self.sigma_space ** 2).astype(
            real_dtype(precision), copy=False)

    def power_coefficient(self, t: float) -> float:
        return 0.0 if t < self.delay else self.P0


class ProfileLaser:
    """P(r, t) = P0 profile(r) for t >= delay with the ``gaussian`` and ``ring`` profiles
    (``polarism/laser/profile_laser.py:26-52``, ``polarism/profiles/builtin_profiles.py:34-73``:
    ring = exp(-((r - radius) / width)^2 / 2))."""

    time_independent = True

    def __init__(self, cfg: LaserParameters, X, Y, precision="double"):
        spec = dict(cfg.profile)
        kind = spec.get("type")
        x0, y0 = float(spec.get("x0", cfg.x0)), float(spec.get("y0", cfg.y0))
        r2 = (X - x0) ** 2 + (Y - y0) ** 2
        if kind == "ring":
            shape = np.exp(-0.5 * ((np.sqrt(r2) - float(spec["radius"])) / float(spec["width"])) ** 2)
        elif kind == "gaussian":
            shape = np.exp(-0.5 * r2 / float(spec["sigma"]) ** 2)
        elif kind == "lattice":
            shape = square_lattice(X, Y, float(spec["constant"]), float(spec["width"]), x0, y0)
        else:
            raise ValueError(f"unsupported profile {kind!r}")
        self.P0 = float(cfg.P0)
        self.delay = float(cfg.delay)
        self._spatial_envelope = shape.astype(real_dtype(precision), copy=False)

    def power_coefficient(self, t: float) -> float:
        return 0.0 if t < self.delay else self.P0


def square_lattice(X, Y, constant, width, x0=0.0, y0=0.0):
    """Unit-depth Gaussian wells of ``width`` on a square lattice of pitch ``constant`` with a
    site at (x0, y0), covering the box plus one cell (the square case of the ``lattice``
    profile, ``polarism/profiles/builtin_profiles.py:180-237``, without disorder)."""
    dx = float(X[0, 1] - X[0, 0]) if X.shape[1] > 1 else 1.0
    dy = float(Y[1, 0] - Y[0, 0]) if Y.shape[0] > 1 else 1.0
    half_x = 0.5 * (X.max() - X.min() + dx) + constant
    half_y = 0.5 * (Y.max() - Y.min() + dy) + constant
    out = np.zeros(X.shape)
    for i in range(-int(half_x // constant) - 1, int(half_x // constant) + 2):
        for j in range(-int(half_y // constant) - 1, int(half_y // constant) + 2):
            sx, sy = x0 + i * constant, y0 + j * constant
            if abs(sx) > half_x or abs(sy) > half_y:
                continue
            out += np.exp(-0.5 * ((X - sx) ** 2 + (Y - sy) ** 2) / width ** 2)
    return out


class PulseGaussian:
    """Gaussian spot with a train of Gaussian pulses in time, peak-amplitude definition
    (``polarism/laser/pulse_gaussian.py:34-55,101-135``): pulse n is centred at
    delay + phase + n * separation with phase = cutoff * sigma_t, cut at cutoff * sigma_t, its
    amplitude min(P0 + n (Pmax - P0), Pmax); n_pulses <= 0 means an endless train."""

    time_independent = False

    def __init__(self, cfg: LaserParameters, X, Y, precision="double"):
        self.P0, self.Pmax = float(cfg.P0), float(cfg.Pmax)
        self.x0, self.y0 = float(cfg.x0), float(cfg.y0)
        self.delay, self.sigma_space = float(cfg.delay), float(cfg.sigma_space)
        self.sigma_time, self.cutoff_sigma = float(cfg.sigma_time), float(cfg.cutoff_sigma)
        self.pulse_separation, self.n_pulses = float(cfg.pulse_separation), int(cfg.n_pulses)
        self.phase = self.cutoff_sigma * self.sigma_time
        r2 = (X - self.x0) ** 2 + (Y - self.y0) ** 2
        self._spatial_envelope = np.exp(-0.5 * r2 / self.sigma_space ** 2).astype(
            real_dtype(precision), copy=False)

    def power_coefficient(self, t: float) -> float:
        if t < self.delay:
            return 0.0
        t_eff = t - self.delay
        n = max(0, round((t_eff - self.phase) / self.pulse_separation))
        if self.n_pulses > 0 and n >= self.n_pulses:
            return 0.0
        offset = t_eff - n * self.pulse_separation - self.phase
        if abs(offset) > self.cutoff_sigma * self.sigma_time:
            return 0.0
        amplitude = min(self.P0 + n * (self.Pmax - self.P0), self.Pmax)
        return amplitude * math.exp(-0.5 * (offset / self.sigma_time) ** 2)


def make_lasers(cfg: LaserParameters, X, Y, precision="double"):
    """The lasers of one config: one, or every entry of ``lasers`` in mode "multiple"."""
    if cfg.mode == "multiple":
        if not cfg.lasers:
            raise ValueError("laser mode 'multiple' needs a non-empty lasers list")
        return [make_laser(item, X, Y, precision) for item in cfg.lasers]
    return [make_laser(cfg, X, Y, precision)]


def make_laser(cfg: LaserParameters, X, Y, precision="double"):
    if cfg.laser_type == "profile":
        return ProfileLaser(cfg, X, Y, precision)
    if cfg.laser_type == "continuous-gaussian":
        return ContinuousGaussian(cfg, X, Y, precision)
    if cfg.laser_type == "pulse-gaussian":
        return PulseGaussian(cfg, X, Y, precision)
    raise ValueError(f"unsupported laser_type {cfg.laser_type!r}")


class PumpField:
    """Total pump with one cached separable (envelope, coefficient) term."""

    def __init__(self, lasers, grid, precision):
        self.lasers = list(lasers)
        self.grid = grid
        self.precision = precision

    def separable_term(self):
        if len(self.lasers) != 1:
            return None
        laser = self.lasers[0]
        return laser._spatial_envelope, laser.power_coefficient

    def separable_terms(self):
        return [(laser._spatial_envelope, laser.power_coefficient) for laser in self.lasers]

    def __call__(self, t: float):
        total = 0
        for envelope, coefficient in self.separable_terms():
            total = total + envelope * coefficient(t)
        return total


class BatchedPumpField:
    """Laser slots matched across members (``polarism/laser/pump_field.py:92-152``): slot l
    holds every member's l-th laser, its envelope shared when all are equal (else stacked per
    member) and its coefficient a member vector."""

    def __init__(self, member_lasers, grid, precision):
        self.member_lasers = [list(lasers) for lasers in member_lasers]
        if len({len(lasers) for lasers in self.member_lasers}) != 1:
            raise ValueError("every member needs the same number of lasers")
        self.lasers = self.member_lasers[0]
        self.grid = grid
        self.precision = precision
        self._terms = []
        for slot in zip(*self.member_lasers):
            envelopes = [laser._spatial_envelope for laser in slot]
            shared = all(np.array_equal(envelopes[0], e) for e in envelopes[1:])
            envelope = envelopes[0] if shared else np.stack(envelopes)[:, None]
            self._terms.append((envelope, self._slot_coefficient(slot)))

    def _slot_coefficient(self, slot):
        dtype = real_dtype(self.precision)

        def coefficient(t):
            return np.asarray([laser.power_coefficient(t) for laser in slot], dtype=dtype)
        return coefficient

    def separable_terms(self):
        return list(self._terms)

    def separable_term(self):
        return None

    def __call__(self, t):
        total = 0
        for envelope, coefficient in self._terms:
            total = total + envelope * coefficient(t).reshape(-1, 1, 1, 1)
        return total


# --------------------------------------------------------------------------- reservoir
class SingleReservoir:
    """dn/dt = P - (gamma_R + R |psi|^2) n with the non-negative clamp on set_state."""

    state_names = ("nR",)

    def __init__(self, physics: PhysicsConstants, grid, precision="double", batch_size=None,
                 components=1):
        self.components = components
        self._dtype = real_dtype(precision)
        self.nR = np.zeros((batch_size or 1, components, *grid.shape), dtype=self._dtype)
        self._batched = batch_size is not None

    def get_state(self):
        return (self.nR,)

    def set_state(self, state):
        (n,) = state
        if n.shape != self.nR.shape:
            raise ValueError(f"reservoir state shape must be {self.nR.shape}")
        if n is self.nR and n.dtype == self._dtype:
            np.maximum(n, 0, out=n)
            return
        self.nR = np.maximum(n, 0).astype(self._dtype, copy=False)

    def get_active_density(self, state):
        return state[0]

    def get_inactive_density(self, state):
        return state[0] * 0.0


class DoubleReservoir:
    """Active and inactive reservoirs (``polarism/reservoir/double_reservoir.py:22-130``):
    dn_I = P - (gamma_I + R_IA) n_I + R_AI n_A, dn_A = R_IA n_I - (gamma_A + R_AI + R |psi|^2) n_A;
    both clamped at zero on set_state; one pair per field component or one shared pair."""

    state_names = ("nA", "nI")

    def __init__(self, physics: PhysicsConstants, grid, precision="double", batch_size=None,
                 components=1):
        self.components = components
        self._dtype = real_dtype(precision)
        shape = (batch_size or 1, components, *grid.shape)
        self.nA = np.zeros(shape, dtype=self._dtype)
        self.nI = np.zeros(shape, dtype=self._dtype)

    def get_state(self):
        return (self.nA, self.nI)

    def set_state(self, state):
        n_a, n_i = state
        if n_a.shape != self.nA.shape or n_i.shape != self.nI.shape:
            raise ValueError(f"reservoir state shapes must be {self.nA.shape}")
        self.nA = np.maximum(n_a, 0).astype(self._dtype, copy=False)
        self.nI = np.maximum(n_i, 0).astype(self._dtype, copy=False)

    def get_active_density(self, state):
        return state[0]

    def get_inactive_density(self, state):
        return state[1]


class QuadraticDoubleReservoir(DoubleReservoir):
    """n_R fed by kappa n_I^2 from the inactive reservoir
    (``polarism/reservoir/quadratic_double_reservoir.py:13-14``); state (n_R, n_I)."""

    state_names = ("nR", "nI")


class NoReservoir:
    state_names = ()

    def __init__(self, *args, **kwargs):
        self.components = 1

    def get_state(self):
        return ()

    def set_state(self, state):
        if tuple(state):
            raise ValueError("the 'none' reservoir has no state")

    def get_active_density(self, state):
        return 0.0

    def get_inactive_density(self, state):
        return 0.0


# --------------------------------------------------------------------------- noise
class NoiseParametersArrays:
    """Per-member Wigner parameters: seeds, gamma_C, R, strength, dt, cell volume."""

    def __init__(self, config, grid, members=None):
        members = members or [config]
        self.precision = config.solver.precision
        self.spatial_n = int(np.prod(grid.shape))
        self.volume = float(np.prod(grid.spacing))
        self.dt = float(config.solver.dt)
        self.seeds = np.asarray([m.noise.seed for m in members], dtype=np.uint64)
        self.gamma = np.asarray([m.physics.gamma_C for m in members], dtype=np.float64)
        self.scattering = np.asarray([m.physics.R for m in members], dtype=np.float64)
        self.strength = np.asarray([m.noise.stochastic_strength for m in members], dtype=np.float64)
        self.active = bool(config.noise.enabled and config.noise.stochastic == "wigner"
                           and np.any(self.strength > 0.0))


# --------------------------------------------------------------------------- state
def make_initial_psi(shape, eps, seed, cdtype=np.complex128, rdtype=np.float64,
                     mode="complex_gaussian_zero_mean"):
    """Seeded complex-Gaussian field with zero mean and RMS ``eps``."""
    if mode == "none":
        return np.zeros(shape, dtype=cdtype)
    if mode != "complex_gaussian_zero_mean":
        raise ValueError(f"unsupported initial field mode {mode!r}")
    rng = np.random.default_rng(seed)
    re = rng.standard_normal(shape).astype(rdtype)
    im = rng.standard_normal(shape).astype(rdtype)
    psi = re + 1j * im
    psi -= np.mean(psi)
    rms = float(np.sqrt(np.mean(np.abs(psi) ** 2)))
    if rms < 1e-30:
        rms = 1.0
    return ((eps / rms) * psi).astype(cdtype)


class SimulationState:
    """Canonical ``(B, C, ny, nx)`` field with time bookkeeping."""

    def __init__(self, field, batched=False):
        self.batch_size = field.shape[0]
        self.components = field.shape[1]
        self.batched = batched
        self._field = field
        self._field_k = None
        self.t = 0.0
        self.t0 = 0.0
        self.step = 0

    @property
    def field(self):
        if self._field is None and self._field_k is not None:
            self._field = np.fft.ifft2(self._field_k, axes=(-2, -1))
        return self._field

    @field.setter
    def field(self, value):
        self._field = value
        self._field_k = None

    @property
    def field_k(self):
        return self._field_k

    @field_k.setter
    def field_k(self, value):
        self._field_k = value

    @property
    def psi(self):
        return self.field[:, 0] if self.batched else self.field[0, 0]


class BatchPhysicsLite:
    """``get(name)`` returns the scalar, or the ``(B, 1, 1, 1)`` array when members differ."""

    def __init__(self, physics: PhysicsConstants, members=None):
        self.physics = physics
        self.host = {}
        if members and len(members) > 1:
            for name in physics_float_fields():
                values = np.asarray([getattr(m.physics, name) for m in members], dtype=np.float64)
                if np.any(values != values[0]):
                    self.host[name] = values
        self.size = len(members) if members and len(members) > 1 and self.host else None

    def get(self, name):
        if name in self.host:
            return self.host[name].reshape(-1, 1, 1, 1)
        return getattr(self.physics, name, 0.0)

    def any_nonzero(self, name):
        if name in self.host:
            return bool(np.any(self.host[name]))
        return getattr(self.physics, name, 0.0) != 0.0

    def check(self, field, components=1):
        if field.ndim != 4 or field.shape[1] != components:
            raise ValueError(f"batch_physics requires canonical field shape; got {field.shape}")


class _NoAbsorption:
    after_step_is_noop = True


class _Boundary:
    absorption = _NoAbsorption()

    @staticmethod
    def after_step_action(psi):
        return psi


@dataclass
class Model:
    grid: Any
    physics: Any
    precision: str
    potential: Any
    pump: Any
    reservoir: Any
    noise: Any = None
    components: int = 1
    boundary: Any = field(default_factory=_Boundary)
    terms: tuple = ()
    drive: Any = None
    time_dependent_potential: bool = False
    reservoir_components: int = 1
    member_configs: list | None = None
    pump_weights: Any = None


def build_simulation(cfg: Config, members: list[Config] | None = None):
    """Build (grid, model, state) for a config, or a batch of member configs that
    share the grid -- the subset of ``SimulationController.__init__``
    (``polarism/simulation_controller.py:163-341``) this path needs."""
    grid = PeriodicGrid(cfg.grid)
    precision = cfg.solver.precision
    batched = members is not None and len(members) >= 2
    member_cfgs = members if members else [cfg]
    for m in member_cfgs:
        if m.noise.seed is None:
            m.noise.seed = cfg.noise.seed if cfg.noise.seed is not None else 0
    components = 2 if cfg.physics.spin == "spinor" else 1
    res_components = cfg.reservoir.components or components
    lasers = [make_lasers(m.laser, grid.X, grid.Y, precision) for m in member_cfgs]
    pump = BatchedPumpField(lasers, grid, precision) if batched else PumpField(lasers[0], grid, precision)
    res_cls = {"single": SingleReservoir, "double": DoubleReservoir,
               "quadratic-double": QuadraticDoubleReservoir,
               "none": NoReservoir}[cfg.reservoir.reservoir_type]
    reservoir = res_cls(cfg.physics, grid, precision, batch_size=len(member_cfgs) if batched else None,
                        components=res_components)

    def initial(m, seed):
        return make_initial_psi(grid.shape, m.noise.initial_amplitude if m.noise.enabled else 0.0,
                                seed, complex_dtype(precision), real_dtype(precision),
                                m.noise.initial if m.noise.enabled else "none")

    # The second component draws with seed + 1 (polarism/simulation_state.py:59-73).
    field_ = np.stack([np.stack([initial(m, m.noise.seed + c) for c in range(components)])
                       for m in member_cfgs])
    state = SimulationState(np.ascontiguousarray(field_), batched=batched)
    noise = NoiseParametersArrays(cfg, grid, member_cfgs)
    weights = None
    if components == 2:
        weights = np.asarray([[(1 + m.laser.circular_polarization) / 2,
                               (1 - m.laser.circular_polarization) / 2] for m in member_cfgs],
                             dtype=real_dtype(precision)).reshape(len(member_cfgs), 2, 1, 1)
    model = Model(grid=grid, physics=BatchPhysicsLite(cfg.physics, member_cfgs), precision=precision,
                  potential=np.zeros((), dtype=real_dtype(precision)), pump=pump,
                  reservoir=reservoir, noise=noise if noise.active else None,
                  member_configs=member_cfgs, components=components,
                  reservoir_components=res_components, pump_weights=weights)
    return grid, model, state


def threshold_pump(physics: PhysicsConstants) -> float:
    """Uniform-pump condensation threshold P_th = gamma_R gamma_C / R
    (``polarism/analysis/condensation.py:52-57``)."""
    return physics.gamma_R * physics.gamma_C / physics.R


def copy_config(cfg: Config) -> Config:
    import copy

    return copy.deepcopy(cfg)


def isclose(a, b):
    return math.isclose(a, b, rel_tol=1e-12, abs_tol=0.0)
