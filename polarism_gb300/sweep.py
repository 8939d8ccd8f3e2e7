"""Uneven-size sweeps: members of different grids advanced by one persistent launch per step.

Polarism's ``Sweep`` (``polarism/sweep.py:98-324``) groups members by their non-batchable
overrides -- ``grid.*`` among them (``polarism/sweep_config.py:17-60``) -- and runs each group
as its own batch through ``SimulationController``, one group after another.  Here every member,
whatever its (power-of-two) grid, lives in one ``pg_sweep`` (``include/polarism_gb300.h``):
one kernel launch per RK4 step advances all of them, chunks of 64 steps are replayed as CUDA
graphs, and the tile shape of the launch comes from :func:`autotune_tiling`, a measured search
in the manner of ``autotune_batch_size`` (``polarism/sweep.py:23-48``) with its choices cached
per device and member mix.

The steady-state stop follows ``SimulationController._check_steady_state``
(``polarism/simulation_controller.py:710-734``) and its run loop (``:1069-1123``): every
``stop.check_every`` ps the relative change of each member's density and norm since the
previous check is compared with ``stop.rtol``; a member's stop time is the first check at or
after ``stop.min_time`` where both are below it, and the run ends when every member has a stop
time or ``solver.total_time`` is reached.
"""
from __future__ import annotations

import copy
import ctypes as C
import json
import math
import os
import tempfile
import time
from dataclasses import dataclass, field
from itertools import product
from pathlib import Path

import numpy as np

from polarism_gb300 import _lib
from polarism_gb300.engine import MemberPhysics, _pointer


def _pack(arrays, offsets, dtype):
    out = np.empty(int(offsets[-1]), dtype=dtype)
    for m, a in enumerate(arrays):
        out[offsets[m]:offsets[m + 1]] = np.asarray(a, dtype=dtype).reshape(-1)
    return out


class SweepEngine:
    """Owner of one ``pg_sweep``: packed FP32 state of members with their own grids.

    ``grids`` is a list of ``(nx, ny, dx, dy)``; ``physics`` one :class:`MemberPhysics` (or a
    physics-like object) per member.  Per-member arrays cross the boundary as lists of
    ``(ny, nx)`` arrays and are packed member after member.
    """

    def __init__(self, grids, physics, dt: float):
        self._lib = _lib.load()
        self.members = len(grids)
        if self.members < 1:
            raise ValueError("a sweep needs at least one member")
        if len(physics) != self.members:
            raise ValueError("one physics entry per member is required")
        self.grids = [(int(nx), int(ny), float(dx), float(dy)) for nx, ny, dx, dy in grids]
        self.dt = float(dt)
        structs = (_lib.PgSweepGrid * self.members)(
            *[_lib.PgSweepGrid(nx, ny, dx, dy) for nx, ny, dx, dy in self.grids])
        phys = (_lib.PgPhysics * self.members)(
            *[(p if isinstance(p, MemberPhysics) else MemberPhysics.from_object(p)).as_struct()
              for p in physics])
        handle = C.c_void_p()
        _lib.check(self._lib.pg_sweep_create(self.members, structs, phys, self.dt, C.byref(handle)),
                   "pg_sweep_create")
        self._h = handle
        offsets = np.zeros(self.members + 1, dtype=np.int64)
        _lib.check(self._lib.pg_sweep_offsets(self._h, offsets.ctypes.data), "pg_sweep_offsets")
        self.offsets = offsets
        self.sites = int(offsets[-1])

    # ------------------------------------------------------------------ lifecycle
    def close(self):
        if getattr(self, "_h", None):
            self._lib.pg_sweep_destroy(self._h)
            self._h = None

    def __del__(self):  # pragma: no cover - interpreter shutdown order varies
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self):
        return self._lib.pg_sweep_stream(self._h)

    # ------------------------------------------------------------------ data
    def set_state(self, psi, n_res):
        """psi, n_res: lists of per-member (ny, nx) arrays, or packed device arrays."""
        if hasattr(psi, "__cuda_array_interface__"):
            p, _, keep_p = _pointer(psi)
            r, _, keep_r = _pointer(n_res)
            _lib.check(self._lib.pg_sweep_set_state(self._h, p, r, 1), "pg_sweep_set_state")
            return
        packed_psi = _pack(psi, self.offsets, np.complex64)
        packed_res = _pack(n_res, self.offsets, np.float32)
        _lib.check(self._lib.pg_sweep_set_state(self._h, packed_psi.ctypes.data,
                                                packed_res.ctypes.data, 0), "pg_sweep_set_state")

    def get_packed_state(self):
        psi = np.empty(self.sites, dtype=np.complex64)
        res = np.empty(self.sites, dtype=np.float32)
        _lib.check(self._lib.pg_sweep_get_state(self._h, psi.ctypes.data, res.ctypes.data, 0),
                   "pg_sweep_get_state")
        return psi, res

    def unpack(self, packed, m):
        nx, ny = self.grids[m][0], self.grids[m][1]
        return packed[self.offsets[m]:self.offsets[m + 1]].reshape(ny, nx)

    def get_state(self):
        """Per-member lists of (psi (ny, nx) complex64, n_R (ny, nx) float32)."""
        psi, res = self.get_packed_state()
        return ([self.unpack(psi, m) for m in range(self.members)],
                [self.unpack(res, m) for m in range(self.members)])

    def set_pump(self, envelopes):
        packed = _pack(envelopes, self.offsets, np.float32)
        _lib.check(self._lib.pg_sweep_set_pump(self._h, packed.ctypes.data, 0), "pg_sweep_set_pump")

    def set_noise(self, seeds=None, gamma=None, scattering=None, strength=None):
        if seeds is None:
            _lib.check(self._lib.pg_sweep_set_noise(self._h, None, None, None, None), "pg_sweep_set_noise")
            return
        arrays = [np.ascontiguousarray(np.asarray(seeds, dtype=np.uint64).reshape(-1))]
        arrays += [np.ascontiguousarray(np.asarray(v, dtype=np.float64).reshape(-1))
                   for v in (gamma, scattering, strength)]
        if any(a.size != self.members for a in arrays):
            raise ValueError("noise arrays need one entry per member")
        _lib.check(self._lib.pg_sweep_set_noise(self._h, *[a.ctypes.data for a in arrays]),
                   "pg_sweep_set_noise")

    # ------------------------------------------------------------------ launch shape
    def set_tiling(self, lanes: int, strip_rows: int):
        _lib.check(self._lib.pg_sweep_set_tiling(self._h, int(lanes), int(strip_rows)),
                   "pg_sweep_set_tiling")

    @property
    def tiling(self):
        vals = [C.c_int32() for _ in range(4)]
        _lib.check(self._lib.pg_sweep_get_tiling(self._h, *[C.byref(v) for v in vals]),
                   "pg_sweep_get_tiling")
        return {"lanes": vals[0].value, "strip_rows": vals[1].value, "items": vals[2].value,
                "blocks": vals[3].value}

    def set_active(self, active=None):
        if active is None:
            _lib.check(self._lib.pg_sweep_set_active(self._h, None), "pg_sweep_set_active")
            return
        mask = np.ascontiguousarray(np.asarray(active, dtype=np.uint8).reshape(-1))
        if mask.size != self.members:
            raise ValueError("one active flag per member is required")
        _lib.check(self._lib.pg_sweep_set_active(self._h, mask.ctypes.data), "pg_sweep_set_active")

    def set_wait_limit(self, polls: int):
        """100000 (the default: the polls each mbarrier wait of the sweep kernel makes before it
        gives up, about two seconds) or 0: the kernel withholds each block's first row copy, so
        that a wait runs out and the next synchronising call reports PG_ERR_TIMEOUT."""
        _lib.check(self._lib.pg_sweep_set_wait_limit(self._h, int(polls)), "pg_sweep_set_wait_limit")

    # ------------------------------------------------------------------ stepping
    def advance(self, start_step: int, n_steps: int, stage_scales, use_graphs: bool = True):
        scales = np.ascontiguousarray(stage_scales, dtype=np.float64)
        if scales.shape != (n_steps, 3, self.members):
            raise ValueError(f"stage_scales must have shape ({n_steps}, 3, {self.members})")
        _lib.check(self._lib.pg_sweep_advance(self._h, int(start_step), int(n_steps),
                                              scales.ctypes.data, 1 if use_graphs else 0),
                   "pg_sweep_advance")

    def last_time_ms(self) -> float:
        v = C.c_float()
        _lib.check(self._lib.pg_sweep_last_time_ms(self._h, C.byref(v)), "pg_sweep_last_time_ms")
        return float(v.value)

    @property
    def last_launch_count(self) -> int:
        return int(self._lib.pg_sweep_last_launch_count(self._h))

    def synchronize(self):
        _lib.check(self._lib.pg_sweep_synchronize(self._h), "pg_sweep_synchronize")

    def steady_check(self):
        out = [np.empty(self.members, dtype=np.float64) for _ in range(3)]
        _lib.check(self._lib.pg_sweep_steady_check(self._h, *[o.ctypes.data for o in out]),
                   "pg_sweep_steady_check")
        return tuple(out)

    # -- device-resident steady-state monitor (as RK4Engine's) ---------------------------
    def steady_reset(self):
        _lib.check(self._lib.pg_sweep_steady_reset(self._h), "pg_sweep_steady_reset")

    def steady_update(self, step, record=True, rtol=1e-6, halt=False):
        """Enqueue one steady-state check (no wait)."""
        _lib.check(self._lib.pg_sweep_steady_update(self._h, int(step), int(bool(record)),
                                                    float(rtol), int(bool(halt))),
                   "pg_sweep_steady_update")

    def steady_poll(self):
        """(members stopped, checks finished since the reset), read without waiting."""
        stopped, done = C.c_int32(), C.c_int64()
        _lib.check(self._lib.pg_sweep_steady_poll(self._h, C.byref(stopped), C.byref(done)),
                   "pg_sweep_steady_poll")
        return int(stopped.value), int(done.value)

    def steady_results(self):
        """Waits; returns (rel_density, rel_norm, norms, stop_steps, halt_step or None)."""
        out = [np.empty(self.members, dtype=np.float64) for _ in range(3)]
        stops = np.empty(self.members, dtype=np.int64)
        halt = C.c_int64()
        _lib.check(self._lib.pg_sweep_steady_results(self._h, *[o.ctypes.data for o in out],
                                                     stops.ctypes.data, C.byref(halt)),
                   "pg_sweep_steady_results")
        return (*out, stops, None if halt.value < 0 else int(halt.value))

    def sync_counts(self):
        """(host_syncs, throttle_waits) of the sweep handle (see RK4Engine.sync_counts)."""
        h, w = C.c_int64(), C.c_int64()
        _lib.check(self._lib.pg_sweep_sync_counts(self._h, C.byref(h), C.byref(w)),
                   "pg_sweep_sync_counts")
        return int(h.value), int(w.value)


# --------------------------------------------------------------------------- autotuner
def tiling_candidates(grids):
    """(lanes, strip_rows) pairs valid for the member widths: lanes must hold the widest
    member and be at most 8x the narrowest; strip heights are powers of two up to the
    tallest member."""
    widths = [g[0] for g in grids]
    heights = [g[1] for g in grids]
    out = []
    for lanes in (512, 1024):
        if max(widths) > lanes or min(widths) * 8 < lanes:
            continue
        h = 8
        while True:
            out.append((lanes, h))
            if h >= max(heights):
                break
            h *= 2
    return out


def _cache_file() -> Path:
    root = os.environ.get("XDG_CACHE_HOME")
    return (Path(root) if root else Path.home() / ".cache") / "polarism_gb300" / "sweep_tiling.json"


def _cache_key(engine: SweepEngine, noise: bool) -> str:
    try:
        import torch

        device = torch.cuda.get_device_name() if torch.cuda.is_available() else "cuda"
    except Exception:  # pragma: no cover - torch is optional for the library itself
        device = "cuda"
    sizes = {}
    for nx, ny, _, _ in engine.grids:
        sizes[f"{ny}x{nx}"] = sizes.get(f"{ny}x{nx}", 0) + 1
    return json.dumps([device, sorted(sizes.items()), bool(noise)])


def _write_cache(path: Path, cache: dict) -> None:
    path.parent.mkdir(parents=True, exist_ok=True)
    fd, tmp = tempfile.mkstemp(dir=path.parent, prefix=".sweep_tiling_", suffix=".tmp")
    try:
        with os.fdopen(fd, "w", encoding="utf-8") as handle:
            json.dump(cache, handle, indent=2, sort_keys=True)
        os.replace(tmp, path)
    finally:
        if os.path.exists(tmp):
            os.unlink(tmp)


def autotune_tiling(engine: SweepEngine, *, noise: bool = True, steps: int = 32, repeats: int = 2,
                    candidates=None, use_cache: bool = True, stage_scale: float = 1.0):
    """Time every candidate tile shape on the engine's own members and keep the fastest.

    Each candidate runs ``steps`` graph-captured steps ``repeats`` times after one warm-up
    call; the device time of the best repeat (CUDA events on the sweep's stream) ranks it.
    The members' state is saved before and restored after, so tuning leaves no trace.  The
    winner is cached per (device, member sizes, noise) in ``$XDG_CACHE_HOME/polarism_gb300``.
    Returns ``{"lanes", "strip_rows", "timings"}``.
    """
    candidates = list(candidates) if candidates is not None else tiling_candidates(engine.grids)
    if not candidates:
        raise ValueError("no valid tile shape for these member widths")
    key = _cache_key(engine, noise)
    cache_path = _cache_file()
    if use_cache:
        try:
            cached = json.loads(cache_path.read_text()).get(key)
        except (OSError, ValueError):
            cached = None
        if isinstance(cached, dict) and (cached.get("lanes"), cached.get("strip_rows")) in candidates:
            engine.set_tiling(cached["lanes"], cached["strip_rows"])
            return {"lanes": cached["lanes"], "strip_rows": cached["strip_rows"], "timings": None}
    psi, res = engine.get_packed_state()
    scales = np.full((steps, 3, engine.members), stage_scale, dtype=np.float64)
    timings = {}
    for lanes, rows in candidates:
        engine.set_tiling(lanes, rows)
        engine.advance(0, steps, scales)
        best = math.inf
        for _ in range(repeats):
            engine.advance(0, steps, scales)
            best = min(best, engine.last_time_ms())
        timings[(lanes, rows)] = best / steps
    choice = min(timings, key=timings.get)
    engine.set_tiling(*choice)
    _lib.check(engine._lib.pg_sweep_set_state(engine._h, psi.ctypes.data, res.ctypes.data, 0),
               "pg_sweep_set_state")
    if use_cache:
        try:
            try:
                cache = json.loads(cache_path.read_text())
            except (OSError, ValueError):
                cache = {}
            cache[key] = {"lanes": choice[0], "strip_rows": choice[1]}
            _write_cache(cache_path, cache)
        except OSError:
            pass
    return {"lanes": choice[0], "strip_rows": choice[1],
            "timings": {f"{k[0]}x{k[1]}": v for k, v in timings.items()}}


# --------------------------------------------------------------------------- sweep driver
@dataclass
class SweepResult:
    psi: list
    reservoir: list
    stop_times: np.ndarray
    steps: int
    t: float
    wall_time: float
    tiling: dict = field(default_factory=dict)
    # Host waits of the sweep handle from the first chunk until the run first waited for the
    # device monitor's decisions (or to the end of the loop): 0 with the device monitor.
    loop_syncs: int = -1


def _member_inputs(cfg):
    """Grid, envelope, pump coefficient, initial psi and noise parameters of one member from
    a host-mirror config (:mod:`polarism_gb300.host`)."""
    from polarism_gb300 import host

    grid = host.PeriodicGrid(cfg.grid)
    laser = host.make_laser(cfg.laser, grid.X, grid.Y, "single")
    seed = cfg.noise.seed if cfg.noise.seed is not None else 0
    psi0 = host.make_initial_psi(grid.shape, cfg.noise.initial_amplitude if cfg.noise.enabled else 0.0,
                                 seed, np.complex64, np.float32,
                                 cfg.noise.initial if cfg.noise.enabled else "none")
    wigner = bool(cfg.noise.enabled and cfg.noise.stochastic == "wigner"
                  and cfg.noise.stochastic_strength > 0.0)
    return grid, laser, psi0, seed, wigner


def run_sweep(member_cfgs, *, total_time=None, check_every=None, rtol=None, min_time=None,
              steady_state=None, autotune=True, freeze_stopped=False, use_graphs=True,
              chunk_steps=None, initial=None, device_monitor=True):
    """Advance every member config (host-mirror ``Config`` objects that may differ in grid,
    pump, physics and seed; one ``dt``) with one persistent launch per RK4 step.

    Stop parameters default to the first member's ``stop`` section and its
    ``solver.total_time``.  ``freeze_stopped`` leaves members out of the launch once they
    have a stop time (the reference keeps stepping them until every member has stopped);
    ``initial`` optionally gives per-member ``(psi, n_R)`` starting fields.

    With ``device_monitor`` (the default) the steady-state checks are queued on the device
    behind the chunks (``pg_sweep_steady_update``): the host reads the monitor's progress word
    without waiting, and the check that finds every member stopped halts the sweep, so the run
    ends on that check's step with no host wait per chunk.  With ``freeze_stopped`` the host
    freezes members when the progress word shows new stops (one wait each time); they keep
    stepping until then, so a frozen member's final state can be a few chunks past its stop
    step.  ``device_monitor=False`` reads every check back and decides on the host.
    """
    cfgs = list(member_cfgs)
    first = cfgs[0]
    dt = float(first.solver.dt)
    for c in cfgs:
        if not math.isclose(float(c.solver.dt), dt, rel_tol=1e-12):
            raise ValueError("all sweep members must share solver.dt")
        if getattr(c.reservoir, "reservoir_type", "single") != "single":
            raise ValueError("the uneven-size sweep steps the single reservoir")
    total_time = float(first.solver.total_time if total_time is None else total_time)
    stop = first.stop
    steady = bool(stop.steady_state if steady_state is None else steady_state)
    check_every = float(stop.check_every if check_every is None else check_every)
    rtol = float(stop.rtol if rtol is None else rtol)
    min_time = float(stop.min_time if min_time is None else min_time)

    inputs = [_member_inputs(c) for c in cfgs]
    grids = [(g.nx, g.ny, g.dx, g.dy) for g, *_ in inputs]
    physics = [MemberPhysics.from_object(c.physics) for c in cfgs]
    engine = SweepEngine(grids, physics, dt)
    try:
        engine.set_pump([laser._spatial_envelope for _, laser, *_ in inputs])
        wigner = [w for *_, w in inputs]
        if any(wigner):
            engine.set_noise([s for *_, s, _ in inputs], [c.physics.gamma_C for c in cfgs],
                             [c.physics.R for c in cfgs],
                             [c.noise.stochastic_strength if w else 0.0 for c, w in zip(cfgs, wigner)])
        if initial is not None:
            engine.set_state([p for p, _ in initial], [n for _, n in initial])
        else:
            engine.set_state([psi0 for _, _, psi0, _, _ in inputs],
                             [np.zeros((g.ny, g.nx), np.float32) for g, *_ in inputs])
        tiling = {}
        if autotune:
            tiling = autotune_tiling(engine, noise=any(wigner))
        coefficients = [laser.power_coefficient for _, laser, *_ in inputs]

        n_total = int(round(total_time / dt))
        interval = int(round(check_every / dt)) if steady else 0
        if steady and (interval <= 0 or not math.isclose(interval * dt, check_every, rel_tol=1e-9)):
            raise ValueError("stop.check_every must be a positive multiple of solver.dt")
        chunk = int(chunk_steps or (interval if interval else min(n_total, 4096)) or 1)
        stop_times = np.full(engine.members, np.nan)
        active = np.ones(engine.members, dtype=bool)
        monitor = bool(interval and device_monitor)
        frozen = 0
        step = 0
        wall0 = time.perf_counter()
        if monitor:
            engine.steady_reset()
        syncs0 = engine.sync_counts()[0]
        loop_syncs = []

        def settle():
            """Wait for the queued checks; record their stops; the step the state is at."""
            if not loop_syncs:
                loop_syncs.append(engine.sync_counts()[0] - syncs0)
            *_, stops, halt_step = engine.steady_results()
            new = (stops >= 0) & np.isnan(stop_times)
            stop_times[new] = stops[new] * dt
            return new, halt_step

        while step < n_total and not (steady and np.isfinite(stop_times).all()):
            end = min(n_total, step + chunk)
            if interval:
                end = min(end, (step // interval + 1) * interval)
            n = end - step
            scales = np.empty((n, 3, engine.members), dtype=np.float64)
            for k in range(n):
                t = (step + k) * dt
                for s, tt in enumerate((t, t + 0.5 * dt, t + dt)):
                    scales[k, s] = [coef(tt) for coef in coefficients]
            engine.advance(step, n, scales, use_graphs=use_graphs)
            step = end
            if monitor and step % interval == 0:
                engine.steady_update(step, record=step * dt >= min_time, rtol=rtol, halt=True)
                stopped, _ = engine.steady_poll()
                if stopped == engine.members or (freeze_stopped and stopped > frozen):
                    new, halt_step = settle()
                    if halt_step is not None:
                        step = halt_step
                    elif freeze_stopped and new.any():
                        active &= ~new
                        engine.set_active(active)
                    frozen = int(np.isfinite(stop_times).sum())
            elif interval and step % interval == 0:
                rel_d, rel_n, norms = engine.steady_check()
                reached = (norms < 1e-30) | ((rel_n < rtol) & (rel_d < rtol))
                if step * dt >= min_time:
                    newly = reached & np.isnan(stop_times)
                    stop_times[newly] = step * dt
                    if freeze_stopped and newly.any():
                        active &= ~newly
                        engine.set_active(active)
        if monitor and not np.isfinite(stop_times).all():
            # The run reached total_time: the stops of the checks still queued, and the step of
            # the state when one of them halted the sweep.
            _, halt_step = settle()
            if halt_step is not None:
                step = halt_step
        if not loop_syncs:
            loop_syncs.append(engine.sync_counts()[0] - syncs0)
        engine.synchronize()
        wall = time.perf_counter() - wall0
        psi, res = engine.get_state()
        return SweepResult(psi=[p.copy() for p in psi], reservoir=[r.copy() for r in res],
                           stop_times=stop_times, steps=step, t=step * dt, wall_time=wall,
                           tiling=tiling or engine.tiling, loop_syncs=loop_syncs[0])
    finally:
        engine.close()


def _apply_override(cfg, path: str, value):
    section, _, name = path.partition(".")
    if not name or not hasattr(cfg, section):
        raise ValueError(f"Unknown sweep path {path!r}")
    target = getattr(cfg, section)
    if not hasattr(target, name):
        raise ValueError(f"Unknown sweep path {path!r}")
    setattr(target, name, value)


class Sweep:
    """``Sweep(cfg, parameters, mode)`` over dotted-path overrides (``polarism/sweep.py:98-138``:
    ``"product"`` or ``"zip"`` of the value sequences, members in deterministic order).

    Unlike the reference, members that differ in non-batchable sections (``grid.nx``,
    ``grid.lx``, ...) are not split into sequential groups: :meth:`run` advances all of them
    together with :func:`run_sweep`.  Results follow the reference's in-memory form: one
    ``{"psi": (1, ny, nx), "reservoir": ((ny, nx),)}`` dictionary per member; the stop times are
    kept in ``stop_times``.
    """

    def __init__(self, cfg, parameters, mode="product"):
        if mode not in {"product", "zip"}:
            raise ValueError("mode must be 'product' or 'zip'")
        if not isinstance(parameters, dict):
            raise ValueError("parameters must map dotted paths to sequences")
        keys = list(parameters)
        values = [list(parameters[key]) for key in keys]
        if any(not v for v in values):
            raise ValueError("sweep parameter sequences must be nonempty")
        if mode == "zip" and len({len(v) for v in values}) > 1:
            raise ValueError("zip sweep parameter sequences must have equal lengths")
        rows = product(*values) if mode == "product" else zip(*values)
        self.cfg = cfg
        self.mode = mode
        self.members = [dict(zip(keys, row)) for row in rows]
        self.stop_times = None
        self.result = None

    def member_configs(self):
        out = []
        for overrides in self.members:
            c = copy.deepcopy(self.cfg)
            for path, value in overrides.items():
                _apply_override(c, path, value)
            if c.noise.seed is None:
                c.noise.seed = self.cfg.noise.seed if self.cfg.noise.seed is not None else 0
            out.append(c)
        return out

    def run(self, **kwargs):
        self.result = run_sweep(self.member_configs(), **kwargs)
        self.stop_times = self.result.stop_times
        return [{"psi": p[None].copy(), "reservoir": (r.copy(),)}
                for p, r in zip(self.result.psi, self.result.reservoir)]
