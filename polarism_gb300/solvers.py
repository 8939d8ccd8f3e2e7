"""Polarism solver-registry drop-ins backed by the sm_103a kernels.

``RK4CudaSolver`` replaces ``polarism/solver/rk4_cuda_solver.py:2197-3919``
(registered as ``"rk4-cuda"``).  It keeps the reference contract of
``AbstractSolver`` (``polarism/solver/abstract_solver.py:60-101``):
``__init__(config, grid, model)``, ``step(model, state, dt) -> StepReport`` and
``advance(model, state, n_steps)``, with ``state.step`` advanced and
``state.t = state.t0 + state.step * dt`` (``rk4_cuda_solver.py:3641-3642``).
The Wigner increment is injected inside the step kernel (``injects_noise = True``).

The classes accept both the reference's own objects (``Config``, grid, ``Model``,
``SimulationState``) and the mirrors in :mod:`polarism_gb300.host`.  There is no
CPU path: construction fails with ``RuntimeError`` when the CUDA library or a GPU
is missing, like the reference's GPU-only solvers (``split_step_fft_cuda_solver.py:525-526``).
"""
from __future__ import annotations

import numpy as np

from polarism_gb300 import _lib
from polarism_gb300.engine import MemberPhysics, RK4Engine

try:  # Subclass the reference's contract when Polarism is installed.
    from polarism.solver.abstract_solver import ACCEPTED, AbstractSolver, SolverCapabilities, StepReport
except Exception:  # pragma: no cover - exercised on hosts without Polarism
    from polarism_gb300.contract import ACCEPTED, AbstractSolver, SolverCapabilities, StepReport


def _member_count(state) -> int:
    return int(state.field.shape[0]) if state.field is not None else int(state.field_k.shape[0])


def _is_device(array) -> bool:
    return hasattr(array, "__cuda_array_interface__")


def _host(array):
    """Return a NumPy view/copy of a host or device array."""
    if _is_device(array):
        return array.detach().cpu().numpy() if hasattr(array, "detach") else np.asarray(array.get())
    return np.asarray(array)


class _GB300Solver(AbstractSolver):
    """Shared engine management of the GB300 drop-in solvers."""

    name = "gb300"
    injects_noise = True
    #: Two-component fields run on the IFRK passes only.
    spinor_and_double = False
    #: Reservoir types the class steps.
    reservoir_types = ("single", "none")

    def __init__(self, config, grid, model):
        super().__init__(config, grid, model)
        self._components = int(getattr(model, "components", 1))
        if self._components not in ((1, 2) if self.spinor_and_double else (1,)):
            raise ValueError(f"{self.name} (GB300) supports scalar fields only")
        if getattr(grid, "ndim", 2) != 2 or getattr(grid, "boundary", "periodic") != "periodic":
            raise ValueError(f"{self.name} (GB300) supports two-dimensional periodic grids")
        reservoir_type = getattr(getattr(config, "reservoir", None), "reservoir_type", "single")
        if reservoir_type not in self.reservoir_types:
            raise ValueError(f"{self.name} (GB300) does not support reservoir_type={reservoir_type!r}")
        self._reservoir_type = reservoir_type
        self._res_components = int(getattr(model, "reservoir_components", None)
                                   or getattr(model.reservoir, "components", None) or 1)
        self._grid = grid
        self._precision = getattr(config.solver, "precision", "double")
        self._dt = float(config.solver.dt)
        self._engine = None
        self._engine_key = None
        self._pump_key = None
        self._noise_key = None
        self._potential_key = None
        _lib.load()

    # ------------------------------------------------------------------ helpers
    def _physics_list(self, members, model=None):
        bp = self.batch_physics
        out = [MemberPhysics.from_object(bp, m) for m in range(members)]
        weights = getattr(model, "pump_weights", None) if model is not None else None
        if weights is not None:
            w = np.asarray(_host(weights), dtype=np.float64).reshape(-1, 2)
            for m, phys in enumerate(out):
                phys.pump_weight_plus, phys.pump_weight_minus = (float(v) for v in w[m if len(w) > 1 else 0])
        return out

    def _ensure_engine(self, model, members, pump_envs, potential):
        pump_per_member = any(np.ndim(e) == 4 and e.shape[0] > 1 for e in pump_envs)
        pump_terms = len(pump_envs)
        pot_kind = _lib.PG_POT_NONE
        pot_per_member = False
        if potential is not None and np.ndim(potential) > 0 and np.any(potential != 0):
            pot_kind = _lib.PG_POT_COMPLEX if np.iscomplexobj(potential) else _lib.PG_POT_REAL
            pot_per_member = np.ndim(potential) == 4 and potential.shape[0] > 1
        key = (members, pump_per_member, pot_kind, pot_per_member, pump_terms)
        if self._engine is None or self._engine_key != key:
            if self._engine is not None:
                self._engine.close()
            g = self._grid
            self._engine = RK4Engine(g.nx, g.ny, members, g.dx, g.dy, self._dt,
                                     self._physics_list(members, model), self._precision,
                                     reservoir=self._reservoir_type, potential=pot_kind,
                                     pump_per_member=pump_per_member,
                                     potential_per_member=pot_per_member,
                                     components=self._components,
                                     reservoir_components=self._res_components,
                                     pump_terms=pump_terms)
            self._engine_key = key
            self._pump_key = self._noise_key = self._potential_key = None
        return self._engine

    @staticmethod
    def _pump_terms(pump):
        """Every laser's (envelope, coefficient(t)) (``pump_field.py:81-89``): the kernels sum
        the terms per site, so any number of separable lasers runs on the GPU."""
        terms = pump.separable_terms() if hasattr(pump, "separable_terms") else None
        if terms is None and hasattr(pump, "separable_term"):
            term = pump.separable_term()
            terms = [term] if term is not None else None
        if not terms:
            raise ValueError("rk4-cuda (GB300) needs separable pump terms "
                             "(envelope x coefficient(t) per laser)")
        return list(terms)

    def _upload_inputs(self, engine, model, envelopes, potential):
        envs = [_host(e) for e in envelopes]
        key = tuple((id(e), h.shape) for e, h in zip(envelopes, envs))
        if self._pump_key != key:
            if len(envs) == 1:
                env = np.ascontiguousarray(envs[0], dtype=engine.real)
            else:
                per_member = engine.members > 1 and any(np.ndim(h) == 4 and h.shape[0] > 1
                                                        for h in envs)
                shape = (engine.members, 1, engine.ny, engine.nx) if per_member else (engine.ny, engine.nx)
                env = np.ascontiguousarray(np.stack([
                    np.broadcast_to(np.asarray(h).reshape(shape if np.size(h) == np.prod(shape)
                                                          else (engine.ny, engine.nx)), shape)
                    for h in envs]), dtype=engine.real)
            engine.set_pump(env)
            self._pump_key = key
        if engine.potential_kind != _lib.PG_POT_NONE:
            pkey = id(potential)
            if self._potential_key != pkey:
                engine.set_potential(np.ascontiguousarray(_host(potential)))
                self._potential_key = pkey
        noise = model.noise
        active = bool(noise is not None and getattr(noise, "active", True))
        nkey = (id(noise), active)
        if self._noise_key != nkey:
            if active:
                engine.set_noise(noise.seeds, noise.gamma, noise.scattering, noise.strength,
                                 noise.dt / (4.0 * noise.volume))
            else:
                engine.set_noise(None)
            self._noise_key = nkey

    @staticmethod
    def _coefficient_row(coefficients, time, members):
        """(L, B) coefficients of the L lasers at ``time`` (scalar or per-member values)."""
        row = np.empty((len(coefficients), members), dtype=np.float64)
        for term, coefficient in enumerate(coefficients):
            value = np.asarray(coefficient(time), dtype=np.float64).reshape(-1)
            row[term] = value if value.size == members else value[0]
        return row

    def _sampled(self, coefficients, times, members):
        """Coefficients at each (step, sample) time: (n, S, B), or (n, S, L, B) with several
        lasers (the layout of ``pg_rk4_advance`` / ``pg_split_advance`` / ``pg_ifrk_*``)."""
        if callable(coefficients):  # one laser given as its coefficient function
            coefficients = [coefficients]
        times = np.asarray(times, dtype=np.float64)
        out = np.empty(times.shape + (len(coefficients), members), dtype=np.float64)
        for index in np.ndindex(times.shape):
            out[index] = self._coefficient_row(coefficients, float(times[index]), members)
        return out[..., 0, :] if len(coefficients) == 1 else out

    def stage_scales(self, coefficients, t0, start_step, n_steps, members):
        """Pump coefficients at t, t + dt/2, t + dt of each step (shape (n, 3, [L,] B))."""
        dt = self._dt
        t = t0 + (start_step + np.arange(n_steps, dtype=np.float64)) * dt
        return self._sampled(coefficients, t[:, None] + np.array([0.0, 0.5, 1.0]) * dt, members)

    #: Write results back into the caller's host arrays (for example pinned buffers)
    #: instead of returning fresh arrays each call.
    inplace_host = False

    @staticmethod
    def _writable(array, dtype):
        return (isinstance(array, np.ndarray) and array.dtype == dtype
                and array.flags.c_contiguous and array.flags.writeable)

    def half_scales(self, coefficients, t0, start_step, n_steps, members):
        """Pump coefficients at t + dt/4 and t + 3 dt/4 of each step (shape (n, 2, [L,] B))."""
        dt = self._dt
        t = t0 + (start_step + np.arange(n_steps, dtype=np.float64)) * dt
        return self._sampled(coefficients, t[:, None] + np.array([0.25, 0.75]) * dt, members)

    # ------------------------------------------------------------------ contract
    def step(self, model, state, dt):
        self.advance(model, state, 1)
        return ACCEPTED

    def _prepare(self, model, state):
        """Create/refresh the device handle and upload pump, potential and noise."""
        field = state.field if state.field_k is None or getattr(state, "_field", None) is not None \
            else state.field_k
        members = int(field.shape[0])
        terms = self._pump_terms(model.pump)
        envelopes = [e for e, _ in terms]
        potential = getattr(model, "potential", None)
        engine = self._ensure_engine(model, members, [np.asarray(_host(e)) for e in envelopes],
                                     None if potential is None else _host(potential))
        self._upload_inputs(engine, model, envelopes, potential)
        return engine, members, [c for _, c in terms]

    def _reservoir_array(self, engine, model, device):
        """The reservoir fields in the engine's layout: the single field itself, the two
        fields of the double reservoirs stacked as (2, B, Cr, ny, nx), None without one."""
        res_state = model.reservoir.get_state()
        if self._reservoir_type == "single":
            return res_state[0]
        if self._reservoir_type in ("double", "quadratic-double"):
            if device:
                import torch

                return torch.stack(list(res_state))
            return np.stack([np.asarray(f, dtype=engine.real) for f in res_state])
        return None

    def _upload_state(self, engine, model, array):
        device = _is_device(array)
        res0 = self._reservoir_array(engine, model, device)
        if res0 is not None:
            engine.set_state(array if device else np.ascontiguousarray(array, dtype=engine.complex),
                             res0 if device else np.ascontiguousarray(res0, dtype=engine.real))
        else:
            engine.set_state(array if device else np.ascontiguousarray(array, dtype=engine.complex))
        return device, res0

    def _download_state(self, engine, like, res_in, device):
        if device:
            psi_out = like.new_empty(like.shape) if hasattr(like, "new_empty") else None
            res_out = res_in.new_empty(res_in.shape) if res_in is not None else None
            return engine.get_state(psi_out, res_out)
        if self.inplace_host and self._writable(like, engine.complex) and (
                res_in is None or self._writable(res_in, engine.real)):
            return engine.get_state(like, res_in)
        return engine.get_state()

    def _finish(self, model, state, res, n_steps):
        self._hand_back(model, res)
        state.step += n_steps
        state.t = state.t0 + state.step * self._dt

    def _hand_back(self, model, res):
        # Every kernel leaves n_R clamped at zero at the end of a step, as the reservoir's
        # set_state would.  When the result went in place into the reservoir's own host array
        # (inplace_host), handing it back through set_state would only repeat that clamp over
        # the whole array (for 32 x 1024^2 sites as long as 64 device steps), so it is skipped.
        if (self.inplace_host and self._reservoir_type == "single" and isinstance(res, np.ndarray)
                and res is model.reservoir.get_state()[0]):
            pass
        elif self._reservoir_type == "single":
            model.reservoir.set_state((res,))
        elif self._reservoir_type in ("double", "quadratic-double"):
            model.reservoir.set_state((res[0], res[1]))

    # ------------------------------------------------------------------ resident state
    #: Keep the state in device memory between ``advance`` calls (switched on by
    #: :class:`polarism_gb300.run_loop.DeviceSteadyMonitor`).  The state's field and the
    #: reservoir's arrays then keep their contents from before the first resident chunk until
    #: :meth:`flush` copies the device state back, so that a chunk waits for nothing: the
    #: steps and the steady-state checks are queued behind one another on the solver's
    #: stream.  ``state.step`` and ``state.t`` advance as usual.
    resident = False
    #: Whether the class can keep its state resident (a real-space state between calls).
    supports_resident = False
    _held = None    # (field, reservoir arrays) that the device state stands for
    _stale = False  # the device state is newer than those arrays

    def _holds(self, model, state, field):
        """The device state stands for the arrays the state and the reservoir hold now:
        nothing has replaced them since the last resident chunk or flush."""
        if not self.resident or self._held is None or self._engine is None:
            return False
        held_field, held_res = self._held
        current = tuple(model.reservoir.get_state())
        return (held_field is field and len(held_res) == len(current)
                and all(a is b for a, b in zip(held_res, current)))

    def _keep(self, model, state, field, n_steps):
        """Bookkeeping of a resident chunk: no copy back, the step and time advance."""
        self._held = (field, tuple(model.reservoir.get_state()))
        self._stale = True
        state.step += n_steps
        state.t = state.t0 + state.step * self._dt

    def flush(self, model, state):
        """Copy a resident device state back into ``state`` and the reservoir (one host
        wait); the device keeps it, so the next resident chunk uploads nothing."""
        if not self._stale:
            return
        engine = self._engine
        field = state.field
        device = _is_device(field)
        res_in = self._reservoir_array(engine, model, device)
        psi, res = self._download_state(engine, field, res_in, device)
        state.field = psi
        self._hand_back(model, res)
        self._stale = False
        self._held = (state.field, tuple(model.reservoir.get_state()))

    def release_resident(self, model, state):
        """Flush and leave resident mode."""
        self.flush(model, state)
        self.resident = False
        self._held = None

    @property
    def engine(self):
        return self._engine


class RK4CudaSolver(_GB300Solver):
    """Fused whole-step RK4 on GB300 with in-kernel Philox Wigner noise (``rk4-cuda``)."""

    name = "rk4-cuda"
    supports_resident = True
    reservoir_types = ("single", "none", "double", "quadratic-double")
    capabilities = SolverCapabilities(
        components=frozenset({1}), ndim=frozenset({2}), grid_types=frozenset({"periodic"}),
        reservoirs=frozenset({"single", "double", "quadratic-double", "none"}),
        custom_reservoirs="unsupported",
        potential=True, kinetic_relaxation=True, dispersion=frozenset({"parabolic"}),
        terms=False, noise=frozenset({"none", "wigner"}), adaptive=False,
        quantitative_reservoirs=frozenset({"single", "double", "quadratic-double", "none"}),
        description="GB300 fused RK4 (one sm_103a kernel per step, stage-coupled reservoir, "
                    "Philox Wigner noise in registers).")

    def __init__(self, config, grid, model):
        super().__init__(config, grid, model)
        if getattr(config.solver, "laplacian", "five-point") != "five-point":
            raise ValueError("rk4-cuda (GB300) implements the five-point Laplacian")

    def advance(self, model, state, n_steps: int) -> None:
        if n_steps <= 0:
            return
        field = state.field
        self.batch_physics.check(field, 1)
        engine, members, coefficient = self._prepare(model, state)
        if not self._holds(model, state, field):
            device, res_in = self._upload_state(engine, model, field)
        scales = self.stage_scales(coefficient, state.t0, state.step, n_steps, members)
        engine.advance(state.step, n_steps, scales,
                       use_graphs=bool(getattr(self.config.solver, "cuda_graphs", True)))
        if self.resident:
            self._keep(model, state, field, n_steps)
            return
        psi, res = self._download_state(engine, field, res_in, device)
        state.field = psi
        self._finish(model, state, res, n_steps)


class SplitStepFFTSolver(_GB300Solver):
    """Strang splitting R/2 K/2 N K/2 R/2 on hand-written Stockham FFT passes
    (``split-step-fft``; ``polarism/solver/split_step_fft_solver.py:24-159``).

    The Wigner increment is drawn after the nonlinear step with the reservoir after the
    first half step, as the reference does (``split_step_fft_solver.py:147-148``)."""

    name = "split-step-fft"
    ordering = 0
    supports_resident = True
    reservoir_types = ("single", "none", "double", "quadratic-double")
    capabilities = SolverCapabilities(
        components=frozenset({1}), ndim=frozenset({2}), grid_types=frozenset({"periodic"}),
        reservoirs=frozenset({"single", "double", "quadratic-double", "none"}),
        custom_reservoirs="unsupported",
        potential=True, kinetic_relaxation=False, dispersion=frozenset({"parabolic"}),
        terms=False, noise=frozenset({"none", "wigner"}), adaptive=False,
        quantitative_reservoirs=frozenset({"single", "double", "quadratic-double", "none"}),
        description="GB300 split-step Fourier (R/2 K/2 N K/2 R/2) with shared-memory Stockham "
                    "FFT passes fused with the propagator and the local step; nx, ny powers "
                    "of two.")

    def __init__(self, config, grid, model):
        super().__init__(config, grid, model)
        for n in (grid.nx, grid.ny):
            if n & (n - 1) or not 4 <= n <= 4096:
                raise ValueError(f"{self.name} (GB300) needs power-of-two grid sizes in [4, 4096]")

    def advance(self, model, state, n_steps: int) -> None:
        if n_steps <= 0:
            return
        field = state.field  # materialises psi from a cached spectrum if needed
        self.batch_physics.check(field, 1)
        engine, members, coefficient = self._prepare(model, state)
        if not self._holds(model, state, field):
            device, res_in = self._upload_state(engine, model, field)
        engine.set_state_kind(False)
        scales = self.half_scales(coefficient, state.t0, state.step, n_steps, members)
        engine.split_advance(self.ordering, state.step, n_steps, scales,
                             use_graphs=bool(getattr(self.config.solver, "cuda_graphs", True)))
        if self.resident:
            self._keep(model, state, field, n_steps)
            return
        psi, res = self._download_state(engine, field, res_in, device)
        state.field = psi
        self._finish(model, state, res, n_steps)


class SplitStepFFTCudaSolver(SplitStepFFTSolver):
    """K(dt/2) [R(dt/2) N(dt) R(dt/2)] K(dt/2) keeping the spectrum between steps
    (``split-step-fft-cuda``; ``polarism/solver/split_step_fft_cuda_solver.py:1144-1393``).

    After ``advance`` the state holds ``field_k`` (the unnormalised 2-D spectrum) and no
    real-space field, as the reference leaves it."""

    name = "split-step-fft-cuda"
    ordering = 1
    supports_resident = False  # leaves a spectrum, which the steady check cannot read

    def advance(self, model, state, n_steps: int) -> None:
        if n_steps <= 0:
            return
        spectral = getattr(state, "_field", None) is None and state.field_k is not None
        source = state.field_k if spectral else state.field
        self.batch_physics.check(source, 1)
        engine, members, coefficient = self._prepare(model, state)
        device, res_in = self._upload_state(engine, model, source)
        engine.set_state_kind(spectral)
        scales = self.half_scales(coefficient, state.t0, state.step, n_steps, members)
        engine.split_advance(self.ordering, state.step, n_steps, scales,
                             use_graphs=bool(getattr(self.config.solver, "cuda_graphs", True)))
        spec, res = self._download_state(engine, source, res_in, device)
        state.field = None
        state.field_k = spec
        self._finish(model, state, res, n_steps)


class IFRKFFTCudaSolver(_GB300Solver):
    """Lawson interaction-picture RK on the Stockham FFT passes (``ifrk-fft-cuda``;
    ``polarism/solver/ifrk_fft_cuda_solver.py:23-329``), tableaus ``rk4`` and ``dp5``.

    Fixed steps run the fused stage passes with the Wigner increment after each step.
    With ``solver.adaptive`` the Dormand-Prince trials run on the device (FP64 error
    norm) and the PI controller of ``polarism/solver/step_controller.py`` runs on the host
    while the state stays in device memory for the whole ``advance`` call."""

    name = "ifrk-fft-cuda"
    tableau_name = None
    spinor_and_double = True
    reservoir_types = ("single", "none", "double", "quadratic-double")
    capabilities = SolverCapabilities(
        components=frozenset({1, 2}), ndim=frozenset({2}), grid_types=frozenset({"periodic"}),
        reservoirs=frozenset({"single", "double", "quadratic-double", "none"}),
        custom_reservoirs="unsupported",
        potential=True, kinetic_relaxation=False, dispersion=frozenset({"parabolic"}),
        terms=False, noise=frozenset({"none", "wigner"}), adaptive=True,
        quantitative_reservoirs=frozenset({"single", "double", "quadratic-double", "none"}),
        description="GB300 Lawson IFRK (rk4, dp5) with fused Stockham stage passes, FP64 "
                    "embedded error norm, spinor (TE-TM, Zeeman, cross-spin) and double "
                    "reservoirs; nx, ny powers of two.")

    def __init__(self, config, grid, model):
        super().__init__(config, grid, model)
        self.tableau = self.tableau_name or getattr(config.solver, "tableau", "rk4")
        if self.tableau not in ("rk4", "dp5"):
            raise ValueError(f"{self.name} (GB300) implements the rk4 and dp5 tableaus")
        for n in (grid.nx, grid.ny):
            if n & (n - 1) or not 4 <= n <= 4096:
                raise ValueError(f"{self.name} (GB300) needs power-of-two grid sizes in [4, 4096]")
        if MemberPhysics.from_object(self.batch_physics, 0).kinetic_relaxation_eta != 0.0:
            raise ValueError(f"{self.name} (GB300) does not evaluate kinetic_relaxation_eta")
        self.adaptive = bool(getattr(config.solver, "adaptive", False))
        if self.adaptive and self.tableau != "dp5":
            raise ValueError("solver.adaptive requires the embedded dp5 tableau")
        if self.adaptive and getattr(model, "noise", None) is not None and \
                getattr(model.noise, "active", True):
            raise ValueError("solver.adaptive requires stochastic noise off")

    def _stage_scales(self, coefficients, times, members):
        return self._sampled(coefficients, times, members)

    def advance(self, model, state, n_steps: int) -> None:
        from polarism_gb300.engine import TABLEAU_NODES

        if n_steps <= 0:
            return
        field = state.field
        self.batch_physics.check(field, self._components)
        engine, members, coefficient = self._prepare(model, state)
        device, res_in = self._upload_state(engine, model, field)
        engine.set_state_kind(False)
        nodes = TABLEAU_NODES[self.tableau]
        if not self.adaptive:
            dt = self._dt
            scales = np.stack([
                self._stage_scales(coefficient,
                                   [state.t0 + (state.step + k) * dt + c * dt for c in nodes], members)
                for k in range(n_steps)])
            engine.ifrk_advance(self.tableau, state.step, n_steps, scales)
        else:
            controller = getattr(self, "step_controller", None)
            if controller is None:
                from polarism_gb300.step_control import StepController

                controller = StepController(self._dt, getattr(self.config.solver, "dt_max", None))
                self.step_controller = controller
            rtol = float(self.config.solver.rtol)
            atol = float(self.config.solver.atol)
            target = state.t0 + (state.step + n_steps) * self._dt
            t = state.t
            while t < target:
                h, clamped, proposal = controller.propose(t, target)
                scales = self._stage_scales(coefficient, [t + c * h for c in nodes], members)
                err, accepted = engine.ifrk_trial(h, scales, rtol, atol)
                if accepted:
                    t = target if clamped else t + h
                controller.update(h, clamped, proposal, accepted, err)
        psi, res = self._download_state(engine, field, res_in, device)
        state.field = psi
        self._finish(model, state, res, n_steps)

    def step(self, model, state, dt):
        if not self.adaptive:
            self.advance(model, state, 1)
            return ACCEPTED
        from polarism_gb300.engine import TABLEAU_NODES

        field = state.field
        engine, members, coefficient = self._prepare(model, state)
        device, res_in = self._upload_state(engine, model, field)
        engine.set_state_kind(False)
        scales = self._stage_scales(coefficient, [state.t + c * dt for c in TABLEAU_NODES["dp5"]],
                                    members)
        err, accepted = engine.ifrk_trial(dt, scales, float(self.config.solver.rtol),
                                          float(self.config.solver.atol))
        if accepted:
            psi, res = self._download_state(engine, field, res_in, device)
            state.field = psi
            if self._reservoir_type == "single":
                model.reservoir.set_state((res,))
            elif self._reservoir_type in ("double", "quadratic-double"):
                model.reservoir.set_state((res[0], res[1]))
            state.t += dt
        return StepReport(accepted, err, None)


class IFRK4FFTCudaSolver(IFRKFFTCudaSolver):
    """``ifrk4-fft-cuda``: the RK4 tableau whatever ``solver.tableau`` says."""

    name = "ifrk4-fft-cuda"
    tableau_name = "rk4"
    capabilities = SolverCapabilities(**{**IFRKFFTCudaSolver.capabilities.__dict__, "adaptive": False})
