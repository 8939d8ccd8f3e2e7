"""Generate the golden fixtures in this folder by running the reference itself.

Run where the Polarism v0.9.2 source tree is available, naming it::

    python tests/golden/make_golden.py PATH/TO/POLARISM     # or set POLARISM_REFERENCE
    python tests/golden/make_golden.py PATH/TO/POLARISM accumulators   # one case only

Every fixture records both the inputs (initial fields, pump arrays at the
stage times, physics constants) and the reference's outputs, so the tests can
replay them through the oracle and the CUDA library without the reference.
The reference's non-numeric imports (``yaml``, ``h5py``, ``tyro``,
``matplotlib``) are replaced by inert modules; none of them is on the numeric
path.  The reference's shipped IFRK golden file is loaded and compared with a
fresh run so the recorded vectors are pinned to it.
"""
from __future__ import annotations

import copy
import importlib.abc
import importlib.machinery
import json
import sys
from dataclasses import asdict
from pathlib import Path
from unittest import mock

import numpy as np

HERE = Path(__file__).resolve().parent


class _InertModules(importlib.abc.MetaPathFinder, importlib.abc.Loader):
    roots = ("yaml", "h5py", "tyro", "matplotlib", "mpl_toolkits")

    def find_spec(self, name, path, target=None):
        if name.split(".")[0] in self.roots:
            return importlib.machinery.ModuleSpec(name, self, is_package=True)
        return None

    def create_module(self, spec):
        module = mock.MagicMock(name=spec.name)
        module.__path__ = []
        module.__spec__ = spec
        return module

    def exec_module(self, module):
        return None


def reference_root() -> str | None:
    """Location of the Polarism source tree: ``POLARISM_REFERENCE`` when set, else a checkout
    named ``reference`` beside this repository's directory, else None."""
    import os

    if os.environ.get("POLARISM_REFERENCE"):
        return os.environ["POLARISM_REFERENCE"]
    beside = Path(__file__).resolve().parents[3] / "reference"
    return str(beside) if (beside / "polarism" / "__init__.py").exists() else None


def _import_reference(root: str):
    sys.meta_path.insert(0, _InertModules())
    sys.path.insert(0, root)
    import polarism  # noqa: F401
    return polarism


def _physics_json(cfg):
    return json.dumps(asdict(cfg.physics))


def philox_cases(out):
    from polarism.noise.philox import counter_words, normal_pair, philox4x32
    import tests.unit.test_noise as tn

    kat = None
    for mark in getattr(tn.test_philox_random123_vectors, "pytestmark", []):
        if mark.name == "parametrize":
            kat = mark.args[1]
    keys = np.asarray([int(k) for k, _, _ in kat], dtype=np.uint64)
    counters = np.asarray([c for _, c, _ in kat], dtype=np.uint32)
    expected = np.asarray([e for _, _, e in kat], dtype=np.uint32)
    for key, ctr, exp in zip(keys, counters, expected):
        assert tuple(philox4x32(ctr, int(key))) == tuple(int(v) for v in exp)
    batch_key = 0x123456789ABCDEF0
    batch_step = (1 << 40) + 7
    batch_counters = counter_words(np.arange(4096), batch_step)
    batch_words = philox4x32(batch_counters, batch_key)
    re_s, im_s = normal_pair(batch_words, "single")
    re_d, im_d = normal_pair(batch_words, "double")
    np.savez_compressed(out / "philox.npz", kat_keys=keys, kat_counters=counters,
                        kat_expected=expected, batch_key=np.uint64(batch_key),
                        batch_step=np.uint64(batch_step),
                        batch_words=batch_words, normals_single=np.stack([re_s, im_s]),
                        normals_double=np.stack([re_d, im_d]))


def wigner_cases(out):
    from types import SimpleNamespace

    from polarism.compute_engine import compute_engine
    from polarism.config.simulation_parameters import Config
    from polarism.noise.stochastic import NoiseApplier

    compute_engine.xp = np
    compute_engine.use_gpu = False
    result = {}
    for precision in ("single", "double"):
        members = []
        for seed, gamma, strength in ((11, 0.083, 1.0), (2 ** 40 + 3, 0.05, 2.0)):
            cfg = Config()
            cfg.solver.precision = precision
            cfg.solver.dt = 5e-4
            cfg.noise.seed = seed
            cfg.noise.stochastic = "wigner"
            cfg.noise.stochastic_strength = strength
            cfg.physics.gamma_C = gamma
            cfg.physics.R = 0.02
            members.append(cfg)
        grid = SimpleNamespace(shape=(6, 10), spacing=(0.4, 0.3))
        rdt = np.float32 if precision == "single" else np.float64
        cdt = np.complex64 if precision == "single" else np.complex128
        rng = np.random.default_rng(5)
        field = (rng.standard_normal((2, 1, 6, 10)) + 1j * rng.standard_normal((2, 1, 6, 10))).astype(cdt) * 0.01
        active = np.abs(rng.standard_normal((2, 1, 6, 10))).astype(rdt)
        before = field.copy()
        NoiseApplier(members[0], grid, members).apply_arrays(field, active, 12345)
        result[f"{precision}_before"] = before
        result[f"{precision}_active"] = active
        result[f"{precision}_after"] = field
    result["seeds"] = np.asarray([11, 2 ** 40 + 3], dtype=np.uint64)
    result["gamma"] = np.asarray([0.083, 0.05])
    result["R"] = np.asarray([0.02, 0.02])
    result["strength"] = np.asarray([1.0, 2.0])
    result["dt"] = np.float64(5e-4)
    result["cell_volume"] = np.float64(0.4 * 0.3)
    result["step"] = np.uint64(12345)
    np.savez_compressed(out / "wigner.npz", **result)


def _controller(method, nx, ny, lx, ly, dt, p0, sigma, seed, wigner, precision="double",
                reservoir="single"):
    from polarism.config.simulation_parameters import Config
    from polarism.simulation_controller import SimulationController

    cfg = Config()
    cfg.grid.nx, cfg.grid.ny, cfg.grid.lx, cfg.grid.ly = nx, ny, lx, ly
    cfg.reservoir.reservoir_type = reservoir
    cfg.potential.potential_type = "zero"
    cfg.laser.mode = "single"
    cfg.laser.laser_type = "continuous-gaussian"
    cfg.laser.P0 = p0
    cfg.laser.sigma_space = sigma
    cfg.solver.method = method
    cfg.solver.dt = dt
    cfg.solver.precision = precision
    cfg.solver.total_time = dt * 10
    cfg.noise.seed = seed
    if wigner:
        cfg.noise.stochastic = "wigner"
    return SimulationController(cfg)


def trajectory_case(out, name, method, steps, **kw):
    ctl = _controller(method, **kw)
    if ctl.reservoir.get_state() and len(ctl.reservoir.get_state()) == 2:
        # Start the two-field reservoirs away from zero so both fields take part.
        g = ctl.grid
        blob = np.exp(-0.5 * (g.X ** 2 + g.Y ** 2) / 8.0 ** 2)
        ctl.reservoir.set_state(tuple(np.asarray((0.5 + 0.5 * q) * np.broadcast_to(blob, f.shape), dtype=f.dtype)
                                      for q, f in enumerate(ctl.reservoir.get_state())))
    grid = ctl.grid
    psi0 = np.array(ctl.state.field, copy=True)
    res0 = tuple(np.array(f, copy=True) for f in ctl.reservoir.get_state())
    env = np.asarray(ctl.lasers[0]._spatial_envelope)
    norms = []
    for _ in range(steps):
        ctl.solver.advance(ctl.model, ctl.state, 1)
        norms.append(float(np.sum(np.abs(ctl.state.field) ** 2) * grid.dx * grid.dy))
    np.savez_compressed(
        out / f"{name}.npz", psi0=psi0, res0=np.stack(res0), envelope=env,
        p0=np.float64(kw["p0"]), dt=np.float64(kw["dt"]), dx=np.float64(grid.dx),
        dy=np.float64(grid.dy), k_squared=np.asarray(grid.k_squared), steps=np.int64(steps),
        reservoir=kw.get("reservoir", "single"),
        seed=np.uint64(kw["seed"]), wigner=np.bool_(kw["wigner"]),
        physics=_physics_json(ctl.cfg), psi=np.asarray(ctl.state.field),
        res=np.stack([np.asarray(f) for f in ctl.reservoir.get_state()]),
        norms=np.asarray(norms))


def two_laser_case(out, name, method, steps, **kw):
    """Two separable lasers (``pump_field.py:81-89``): the controller's continuous Gaussian plus
    a pulsed Gaussian off centre, built directly (the reference's multiple-laser mode reads a
    YAML file).  Stores both envelopes and every stage-time coefficient the reference used."""
    from polarism.laser.laser_registry import available_lasers

    ctl = _controller(method, **kw)
    grid = ctl.grid
    pulse = copy.deepcopy(ctl.cfg.laser)
    pulse.laser_type, pulse.mode = "pulse-gaussian", "single"
    pulse.x0, pulse.y0, pulse.sigma_space = 6.0, -3.0, 5.0
    pulse.P0 = pulse.Pmax = 0.4
    pulse.sigma_time, pulse.cutoff_sigma, pulse.pulse_separation, pulse.n_pulses = 0.01, 3.0, 0.05, 0
    pulse.delay = 0.002
    second = available_lasers.lookup("pulse-gaussian")(pulse, grid.X, grid.Y, ctl.cfg.solver.precision)
    ctl.lasers = [ctl.lasers[0], second]
    ctl.pump_field.lasers = ctl.lasers
    assert len(ctl.pump_field.separable_terms()) == 2
    psi0 = np.array(ctl.state.field, copy=True)
    res0 = tuple(np.array(f, copy=True) for f in ctl.reservoir.get_state())
    dt = kw["dt"]
    nodes = (0.0, 0.5, 1.0) if method == "rk4-fdm" else (0.25, 0.75)
    coeffs = np.asarray([[[laser.power_coefficient(k * dt + c * dt) for laser in ctl.lasers]
                          for c in nodes] for k in range(steps)])
    norms = []
    for _ in range(steps):
        ctl.solver.advance(ctl.model, ctl.state, 1)
        norms.append(float(np.sum(np.abs(ctl.state.field) ** 2) * grid.dx * grid.dy))
    np.savez_compressed(
        out / f"{name}.npz", psi0=psi0, res0=np.stack(res0),
        envelopes=np.stack([np.asarray(l._spatial_envelope) for l in ctl.lasers]),
        coefficients=coeffs, nodes=np.asarray(nodes), dt=np.float64(dt), dx=np.float64(grid.dx),
        dy=np.float64(grid.dy), k_squared=np.asarray(grid.k_squared), steps=np.int64(steps),
        seed=np.uint64(kw["seed"]), wigner=np.bool_(kw["wigner"]), physics=_physics_json(ctl.cfg),
        pulse=json.dumps({k: getattr(pulse, k) for k in ("P0", "Pmax", "x0", "y0", "sigma_space",
                                                         "sigma_time", "cutoff_sigma",
                                                         "pulse_separation", "n_pulses", "delay")}),
        psi=np.asarray(ctl.state.field), res=np.stack([np.asarray(f) for f in ctl.reservoir.get_state()]),
        norms=np.asarray(norms))


def kouter_case(out):
    """The reference's own NumPy composition check for the GPU ordering."""
    import tests.crosscheck.test_split_step_fft_cuda as ts
    from polarism.config.simulation_parameters import Config
    from polarism.grid.create_grid import create_grid

    cfg = Config()
    cfg.grid.nx, cfg.grid.ny, cfg.grid.lx, cfg.grid.ly = 12, 10, 12.0, 10.0
    cfg.solver.dt = 0.02
    cfg.reservoir.reservoir_type = "single"
    grid = create_grid(cfg.grid)
    rng = np.random.default_rng(3)
    psi = 0.2 * (rng.standard_normal((1, 1, 10, 12)) + 1j * rng.standard_normal((1, 1, 10, 12)))
    fields = (np.abs(rng.standard_normal((1, 1, 10, 12))) * 0.1,)
    x, y = np.asarray(grid.X), np.asarray(grid.Y)
    pumps = [0.4 * np.exp(-0.5 * (x ** 2 + y ** 2) / 3.0 ** 2) * (1.0 + 0.1 * k) for k in range(6)]
    potential = 0.01 * np.cos(2 * np.pi * x / 12.0) - 0.002j
    psi_in, fields_in = psi.copy(), fields[0].copy()
    for k in range(3):
        psi, fields = ts.reference_step(psi, fields, potential, pumps[2 * k], pumps[2 * k + 1],
                                        cfg, grid)
    np.savez_compressed(out / "split_kouter.npz", psi0=psi_in, res0=fields_in[None],
                        pumps=np.stack(pumps), potential=potential, dt=np.float64(cfg.solver.dt),
                        dx=np.float64(grid.dx), dy=np.float64(grid.dy),
                        k_squared=np.asarray(grid.k_squared), physics=_physics_json(cfg),
                        psi=psi, res=np.stack(fields))


def ifrk4_cases(out, root):
    """Replay the reference's IFRK4 golden generator, recording every stage input."""
    from polarism.config.simulation_parameters import ComputeEngineParameters
    from polarism.simulation_controller import SimulationController
    from tests.unit.conftest import small_config

    shipped = np.load(Path(root) / "tests/data/ifrk4_reference/reference.npz")
    result = {}
    for precision in ("single", "double"):
        for reservoir_type in ("single",):
            for eta in (0.0, 0.04):
                cfg = small_config(
                    solver__method="ifrk4-fft-cuda", solver__precision=precision,
                    solver__dt=0.007, solver__total_time=0.035,
                    reservoir__reservoir_type=reservoir_type,
                    physics__kinetic_relaxation_eta=eta,
                    compute_engine=ComputeEngineParameters(use_gpu=False))
                cfg.laser.laser_type = "pulse-gaussian"
                cfg.laser.sigma_time = 0.03
                cfg.laser.cutoff_sigma = 3.0
                ctl = SimulationController(cfg)
                x, y = ctl.grid.X, ctl.grid.Y
                dtype = np.complex64 if precision == "single" else np.complex128
                real = np.float32 if precision == "single" else np.float64
                ctl.state.psi = np.asarray(
                    0.03 * (1 + 0.1 * np.cos(2 * np.pi * x / cfg.grid.lx))
                    * np.exp(1j * 0.2 * np.sin(2 * np.pi * y / cfg.grid.ly)), dtype=dtype)
                fields = tuple(np.asarray(0.2 + 0.02 * np.cos(2 * np.pi * x / cfg.grid.lx)
                                          + index * 0.04, dtype=real)
                               for index in range(len(ctl.reservoir.get_state())))
                ctl.reservoir.set_state(tuple(f.reshape(1, 1, *f.shape) for f in fields))
                ctl.potential = np.asarray(
                    0.01 * np.cos(2 * np.pi * x / cfg.grid.lx)
                    - 0.003j * (1 + np.sin(2 * np.pi * y / cfg.grid.ly)), dtype=dtype)
                key = f"{precision}_{reservoir_type}_eta{eta:g}"
                result[key + "_psi0"] = np.array(ctl.state.field, copy=True)
                result[key + "_res0"] = np.stack([np.array(f, copy=True) for f in ctl.reservoir.get_state()])
                result[key + "_potential"] = np.asarray(ctl.model.potential)
                times = sorted({round(s * 0.007 + c * 0.007, 12)
                                for s in range(5) for c in (0.0, 0.5, 1.0)})
                result[key + "_pump_times"] = np.asarray(times)
                result[key + "_pumps"] = np.stack([np.asarray(ctl.pump_field(t)) for t in times])
                for _ in range(5):
                    ctl.solver.step(ctl.model, ctl.state, cfg.solver.dt)
                psi = np.asarray(ctl.state.psi)
                res = np.asarray(ctl.reservoir.get_state()[0][0, 0])
                tol = 1e-5 if precision == "single" else 1e-12
                np.testing.assert_allclose(psi, shipped[key + "_psi"], rtol=tol,
                                           atol=tol * max(1e-3, np.max(abs(shipped[key + "_psi"]))))
                result[key + "_psi"] = np.asarray(shipped[key + "_psi"])
                result[key + "_res"] = np.asarray(shipped[key + "_res0"])
                np.testing.assert_allclose(res, result[key + "_res"], rtol=tol, atol=tol)
                result[key + "_dx"] = np.float64(ctl.grid.dx)
                result[key + "_dy"] = np.float64(ctl.grid.dy)
                result[key + "_k_squared"] = np.asarray(ctl.grid.k_squared)
                result[key + "_physics"] = _physics_json(cfg)
    np.savez_compressed(out / "ifrk4.npz", **result)


def dp5_case(out, name="dp5", nx=12, ny=8):
    """A nonuniform adaptive DP5 run of the reference's generic Lawson path."""
    from polarism.config.simulation_parameters import ComputeEngineParameters
    from polarism.simulation_controller import SimulationController
    from tests.unit.conftest import small_config

    cfg = small_config(
        grid__nx=nx, grid__ny=ny, grid__lx=float(nx), grid__ly=float(ny),
        solver__method="ifrk-fft-cuda", solver__tableau="dp5", solver__adaptive=True,
        solver__dt=0.05, solver__total_time=0.4, solver__rtol=1e-6, solver__atol=1e-8,
        reservoir__reservoir_type="single", noise__enabled=True, laser__P0=0.3,
        laser__sigma_space=3.0, compute_engine=ComputeEngineParameters(use_gpu=False))
    ctl = SimulationController(cfg)
    x, y = ctl.grid.X, ctl.grid.Y
    ctl.state.psi = np.asarray(0.5 * np.exp(-0.5 * (x ** 2 + y ** 2) / 2.0 ** 2)
                               * np.exp(1j * 0.7 * x), dtype=np.complex128)
    psi0 = np.array(ctl.state.field, copy=True)
    res0 = np.stack([np.array(f, copy=True) for f in ctl.reservoir.get_state()])
    ctl.solver.advance(ctl.model, ctl.state, 8)
    stats = ctl.solver.step_controller.statistics
    np.savez_compressed(
        out / f"{name}.npz", psi0=psi0, res0=res0, envelope=np.asarray(ctl.lasers[0]._spatial_envelope),
        p0=np.float64(cfg.laser.P0), dt=np.float64(cfg.solver.dt), ticks=np.int64(8),
        rtol=np.float64(cfg.solver.rtol), atol=np.float64(cfg.solver.atol),
        dx=np.float64(ctl.grid.dx), dy=np.float64(ctl.grid.dy),
        k_squared=np.asarray(ctl.grid.k_squared), physics=_physics_json(cfg),
        psi=np.asarray(ctl.state.field), res=np.stack([np.asarray(f) for f in ctl.reservoir.get_state()]),
        accepted=np.int64(stats["accepted"]), rejected=np.int64(stats["rejected"]),
        t=np.float64(ctl.state.t))


def spinor_case(out, name, tableau="dp5", adaptive=True, reservoir="double", res_components=2,
                wigner=False, ticks=6, nx=16, ny=16, polarization=0.0):
    """Two-component (circular basis) field with TE-TM, Zeeman and cross-spin terms through the
    reference's generic Lawson path: ring pump, double (or single) reservoir per component or
    shared, adaptive DP5 or fixed-step RK4 with the Wigner hook."""
    from polarism.config.simulation_parameters import ComputeEngineParameters
    from polarism.simulation_controller import SimulationController
    from tests.unit.conftest import small_config

    cfg = small_config(
        grid__nx=nx, grid__ny=ny, grid__lx=2.0 * nx, grid__ly=2.0 * ny,
        solver__method="ifrk-fft-cuda", solver__tableau=tableau, solver__adaptive=adaptive,
        solver__dt=0.0625, solver__total_time=2.0, solver__rtol=1e-6, solver__atol=1e-8,
        reservoir__reservoir_type=reservoir, noise__enabled=True,
        compute_engine=ComputeEngineParameters(use_gpu=False))
    cfg.reservoir.components = res_components
    cfg.physics.spin = "spinor"
    cfg.physics.zeeman = 0.05
    cfg.physics.te_tm = 0.02
    cfg.physics.alpha_2 = -0.1 * cfg.physics.g_C
    cfg.physics.g_I = 0.0005
    cfg.laser.laser_type = "profile"
    cfg.laser.profile = {"type": "ring", "radius": 0.35 * nx, "width": 2.0}
    cfg.laser.P0 = 0.4
    cfg.laser.circular_polarization = polarization
    if wigner:
        cfg.noise.stochastic = "wigner"
        cfg.noise.seed = 7
    ctl = SimulationController(cfg)
    x, y = ctl.grid.X, ctl.grid.Y
    blob = np.exp(-0.5 * (x ** 2 + y ** 2) / (0.2 * nx) ** 2)
    field = np.stack((0.6 * blob * np.exp(1j * 0.5 * x), 0.4 * blob * np.exp(-1j * 0.3 * y)))
    ctl.state.psi = np.asarray(field, dtype=np.complex128)
    fields = ctl.reservoir.get_state()
    seeded = tuple(np.asarray(0.2 * (q + 1) * np.broadcast_to(blob, f.shape), dtype=f.dtype)
                   for q, f in enumerate(fields))
    ctl.reservoir.set_state(seeded)
    psi0 = np.array(ctl.state.field, copy=True)
    res0 = np.stack([np.array(f, copy=True) for f in ctl.reservoir.get_state()])
    ctl.solver.advance(ctl.model, ctl.state, ticks)
    stats = getattr(getattr(ctl.solver, "step_controller", None), "statistics", {"accepted": ticks, "rejected": 0})
    np.savez_compressed(
        out / f"{name}.npz", psi0=psi0, res0=res0, envelope=np.asarray(ctl.lasers[0]._spatial_envelope),
        p0=np.float64(cfg.laser.P0), dt=np.float64(cfg.solver.dt), ticks=np.int64(ticks),
        rtol=np.float64(cfg.solver.rtol), atol=np.float64(cfg.solver.atol),
        dx=np.float64(ctl.grid.dx), dy=np.float64(ctl.grid.dy), kx=np.asarray(ctl.grid.KX),
        ky=np.asarray(ctl.grid.KY), k_squared=np.asarray(ctl.grid.k_squared),
        weights=np.asarray(ctl.model.pump_weights).reshape(-1, 2), physics=_physics_json(cfg),
        reservoir=reservoir, tableau=tableau, adaptive=np.bool_(adaptive), wigner=np.bool_(wigner),
        seed=np.uint64(cfg.noise.seed or 0), psi=np.asarray(ctl.state.field),
        res=np.stack([np.asarray(f) for f in ctl.reservoir.get_state()]),
        accepted=np.int64(stats["accepted"]), rejected=np.int64(stats["rejected"]),
        t=np.float64(ctl.state.t))


def accumulator_case(out, name="accumulators", samples=6):
    """The reference's own ``MomentumDistribution`` and ``G2Accumulator``
    (``polarism/results/accumulators.py:95-172``) over a short noisy ``rk4-fdm`` run of two
    members with different Wigner strengths, sampled after every step.  Stores the sampled
    fields (so the sums can be formed again, on the host or the device) and the reference's
    finalised results: n(k) with the s/2 vacuum subtraction, g1, the corrected density moments
    and g2 (``polarism/analysis/correlations.py:11-29``)."""
    from polarism.config.simulation_parameters import Config
    from polarism.results.accumulators import available_accumulators
    from polarism.simulation_controller import SimulationController

    cfg = Config()
    cfg.grid.nx, cfg.grid.ny, cfg.grid.lx, cfg.grid.ly = 16, 8, 20.0, 6.0
    cfg.reservoir.reservoir_type = "single"
    cfg.potential.potential_type = "zero"
    cfg.laser.mode = "single"
    cfg.laser.laser_type = "continuous-gaussian"
    cfg.laser.P0, cfg.laser.sigma_space = 0.3, 4.0
    cfg.solver.method = "rk4-fdm"
    cfg.solver.dt = 2e-3
    cfg.solver.precision = "double"
    cfg.solver.total_time = 2e-3 * samples
    cfg.noise.seed = 5
    cfg.noise.stochastic = "wigner"
    ctl = SimulationController(cfg, members=[{"noise.seed": 5, "noise.stochastic_strength": 1.0},
                                             {"noise.seed": 6, "noise.stochastic_strength": 0.5}])
    # A condensate well above the Wigner vacuum (|psi|^2 of order 2 against s / 2dV <= 0.53),
    # so that the corrected moments and g2 are not dominated by the subtraction.
    rng = np.random.default_rng(11)
    g = ctl.grid
    blob = 1.4 * np.exp(-0.5 * (g.X ** 2 + g.Y ** 2) / 5.0 ** 2)
    shape = np.shape(ctl.state.field)
    ctl.state.field = (blob + 0.3 * (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)))
    mom = available_accumulators.lookup("momentum-distribution")(ctl)
    g2acc = available_accumulators.lookup("g2")(ctl)
    fields = []
    for k in range(samples):
        ctl.solver.advance(ctl.model, ctl.state, 1)
        fields.append(np.array(ctl.state.field, copy=True))
        mom.update(ctl.state, ctl.state.t)
        g2acc.update(ctl.state, ctl.state.t)
    results = {r.name: np.asarray(r.value) for r in mom.results() + g2acc.results()}
    np.savez_compressed(
        out / f"{name}.npz", fields=np.stack(fields), samples=np.int64(samples),
        cell=np.float64(mom.cell), cells=np.int64(mom.cells),
        strength=np.asarray(mom.strength).reshape(-1), delta=np.asarray(g2acc.delta).reshape(-1),
        sum_k=np.asarray(mom.sum_k), sum_density=np.asarray(g2acc.sum_density),
        sum_density_squared=np.asarray(g2acc.sum_density_squared), **results)


CASES = {"accumulators": accumulator_case}


def main(root, only=()):
    _import_reference(root)
    HERE.mkdir(exist_ok=True)
    if only:
        for name in only:
            CASES[name](HERE)
        print("golden fixtures written to", HERE, ":", ", ".join(only))
        return
    philox_cases(HERE)
    wigner_cases(HERE)
    common = dict(nx=32, ny=24, lx=40.0, ly=30.0, dt=2e-3, p0=0.05, sigma=8.0, seed=42, wigner=True)
    trajectory_case(HERE, "rk4_fdm", "rk4-fdm", 20, **common)
    trajectory_case(HERE, "split_cpu", "split-step-fft", 20, **common)
    trajectory_case(HERE, "rk4_fdm_quiet", "rk4-fdm", 20,
                    **dict(common, wigner=False, seed=0, p0=0.02, sigma=12.0))
    trajectory_case(HERE, "split_cpu_p2", "split-step-fft", 12,
                    **dict(common, nx=32, ny=16, lx=40.0, ly=20.0))
    for res in ("double", "quadratic-double"):
        trajectory_case(HERE, "rk4_fdm_" + res.replace("-", "_"), "rk4-fdm", 20,
                        **dict(common, reservoir=res, p0=0.3))
        trajectory_case(HERE, "split_cpu_p2_" + res.replace("-", "_"), "split-step-fft", 12,
                        **dict(common, nx=32, ny=16, lx=40.0, ly=20.0, reservoir=res, p0=0.3))
    two_laser_case(HERE, "rk4_fdm_two_lasers", "rk4-fdm", 20, **dict(common, nx=32, ny=16, ly=20.0))
    two_laser_case(HERE, "split_cpu_two_lasers", "split-step-fft", 20,
                   **dict(common, nx=32, ny=16, ly=20.0))
    kouter_case(HERE)
    ifrk4_cases(HERE, root)
    dp5_case(HERE)
    dp5_case(HERE, "dp5_p2", nx=16, ny=8)
    spinor_case(HERE, "spinor_dp5", ticks=16)
    spinor_case(HERE, "spinor_dp5_shared", reservoir="single", res_components=1, nx=16, ny=8, ticks=16,
                polarization=0.3)
    spinor_case(HERE, "spinor_rk4_wigner", tableau="rk4", adaptive=False, wigner=True, ticks=4)
    accumulator_case(HERE)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    # make_golden.py [PATH/TO/POLARISM] [case ...]: every fixture, or only the named cases
    # (of CASES); the path may come from POLARISM_REFERENCE instead.
    args = sys.argv[1:]
    root = args.pop(0) if args and args[0] not in CASES else reference_root()
    if root is None:
        sys.exit("usage: make_golden.py PATH/TO/POLARISM [case ...] (or set POLARISM_REFERENCE)")
    main(root, tuple(args))
