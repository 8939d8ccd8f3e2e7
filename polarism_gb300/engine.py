"""Thin Python owner of one ``pg_solver`` handle (device buffers, stream, graphs).

Arrays cross the C ABI as raw pointers: NumPy arrays as host memory, PyTorch CUDA
tensors (or anything exposing ``__cuda_array_interface__``) as device memory.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from polarism_gb300 import _lib


def _pointer(array, dtype=None, writable=False):
    """Return (address, on_device, keepalive) for a NumPy array or a CUDA tensor."""
    if hasattr(array, "__cuda_array_interface__"):
        iface = array.__cuda_array_interface__
        if iface.get("strides") not in (None,):
            # Require a dense C-contiguous device array.
            shape, strides = iface["shape"], iface["strides"]
            itemsize = np.dtype(iface["typestr"]).itemsize
            expect = itemsize
            for dim, stride in zip(reversed(shape), reversed(strides)):
                if dim > 1 and stride != expect:
                    raise ValueError("device arrays passed to polarism_gb300 must be contiguous")
                expect *= dim
        return int(iface["data"][0]), 1, array
    arr = np.asarray(array)
    if dtype is not None and arr.dtype != dtype:
        if writable:
            raise TypeError(f"expected a {np.dtype(dtype)} array, got {arr.dtype}")
        arr = arr.astype(dtype)
    if not arr.flags.c_contiguous:
        if writable:
            raise ValueError("output arrays must be C-contiguous")
        arr = np.ascontiguousarray(arr)
    return arr.ctypes.data, 0, arr


@dataclass
class MemberPhysics:
    hbar: float = 0.6582119514
    m_eff: float = 0.284
    g_C: float = 0.001
    g_R: float = 0.002
    g_I: float = 0.0
    R: float = 0.02
    gamma_C: float = 0.083
    gamma_R: float = 0.005
    kinetic_relaxation_eta: float = 0.0
    gamma_I: float = 0.001
    gamma_A: float = 0.005
    R_IA: float = 5e-2
    R_AI: float = 2.5e-3
    alpha_2: float = 0.0
    zeeman: float = 0.0
    te_tm: float = 0.0
    pump_weight_plus: float = 0.5
    pump_weight_minus: float = 0.5
    kappa: float = 0.05

    @classmethod
    def from_object(cls, physics, index=None):
        """Read the constants from a PhysicsConstants-like object or a BatchPhysics."""
        values = {}
        for name in cls.__dataclass_fields__:
            if hasattr(physics, "get") and not isinstance(physics, dict):
                value = physics.get(name)
            elif isinstance(physics, dict):
                value = physics.get(name, getattr(cls, name))
            else:
                value = getattr(physics, name, getattr(cls, name))
            value = np.asarray(value, dtype=np.float64)
            values[name] = float(value.reshape(-1)[index if (index is not None and value.size > 1) else 0])
        return cls(**values)

    def as_struct(self):
        return _lib.PgPhysics(**self.__dict__)


_TABLEAUS = {"rk4": (0, 4), "dp5": (1, 7)}

# Stage nodes c_i of the tableaus (for the pump coefficients at t + c_i h).
TABLEAU_NODES = {
    "rk4": (0.0, 0.5, 0.5, 1.0),
    "dp5": (0.0, 1 / 5, 3 / 10, 4 / 5, 8 / 9, 1.0, 1.0),
}


class RK4Engine:
    """One device solver handle: ``members`` same-shape fields stepped on the GPU by the
    fused RK4 kernels or the split-step Fourier passes."""

    def __init__(self, nx, ny, members, dx, dy, dt, physics, precision="single", reservoir=True,
                 potential=_lib.PG_POT_NONE, pump_per_member=False, potential_per_member=False,
                 components=1, reservoir_components=None, pump_terms=1):
        """``reservoir``: True/"single", False/"none", "double" or "quadratic-double";
        ``components``: 1, or 2 for a circular-basis spinor (IFRK only);
        ``reservoir_components``: reservoir planes per field, 1 (shared) or ``components``;
        ``pump_terms``: separable lasers L (envelopes (L, ...) and coefficients with a term
        axis before the member axis when L > 1)."""
        self.lib = _lib.load()
        self.nx, self.ny, self.members = int(nx), int(ny), int(members)
        self.precision = precision
        self.real = np.float32 if precision == "single" else np.float64
        self.complex = np.complex64 if precision == "single" else np.complex128
        kind = {True: "single", False: "none"}.get(reservoir, reservoir)
        if kind not in ("none", "single", "double", "quadratic-double"):
            raise ValueError(f"unknown reservoir {reservoir!r}")
        self.reservoir_kind = kind
        self.res_fields = {"none": 0, "single": 1, "double": 2, "quadratic-double": 2}[kind]
        self.reservoir = self.res_fields > 0
        self.components = int(components)
        self.res_components = int(reservoir_components or self.components)
        self.potential_kind = int(potential)
        cfg = _lib.PgConfig(nx=self.nx, ny=self.ny, members=self.members,
                            precision=_lib.PG_SINGLE if precision == "single" else _lib.PG_DOUBLE,
                            reservoir={"none": 0, "single": 1, "double": 2, "quadratic-double": 3}[kind],
                            potential=self.potential_kind, pump_per_member=int(pump_per_member),
                            potential_per_member=int(potential_per_member),
                            dx=float(dx), dy=float(dy), dt=float(dt),
                            components=self.components,
                            reservoir_components=self.res_components,
                            pump_terms=int(pump_terms))
        self.pump_terms = max(1, int(pump_terms))
        if isinstance(physics, (list, tuple)):
            plist = list(physics)
        else:
            plist = [physics] * self.members
        if len(plist) != self.members:
            raise ValueError("need one physics entry per member")
        arr = (_lib.PgPhysics * self.members)(*[p.as_struct() for p in plist])
        handle = C.c_void_p()
        _lib.check(self.lib.pg_create(C.byref(cfg), arr, C.byref(handle)), "pg_create")
        self.handle = handle
        self.dt = float(dt)
        self.noise_on = False

    # -- lifecycle ---------------------------------------------------------------
    def close(self):
        if getattr(self, "handle", None):
            self.lib.pg_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self) -> int:
        return int(self.lib.pg_stream(self.handle) or 0)

    def synchronize(self):
        _lib.check(self.lib.pg_synchronize(self.handle), "pg_synchronize")

    @property
    def shape(self):
        return (self.members, self.components, self.ny, self.nx)

    @property
    def res_shape(self):
        """Reservoir layout: (B, Cr, ny, nx) for one field, (2, B, Cr, ny, nx) for the
        active and inactive fields of the double reservoir."""
        plane = (self.members, self.res_components, self.ny, self.nx)
        return plane if self.res_fields <= 1 else (self.res_fields,) + plane

    # -- data --------------------------------------------------------------------
    def set_state(self, psi, res=None):
        p, dev, keep = _pointer(psi, self.complex)
        if self.reservoir:
            if res is None:
                raise ValueError("reservoir state required")
            r, rdev, keep_r = _pointer(res, self.real)
            if rdev != dev:
                raise ValueError("psi and reservoir must both be host or both be device arrays")
        else:
            r, keep_r = None, None
        _lib.check(self.lib.pg_set_state(self.handle, p, r, dev), "pg_set_state")
        del keep, keep_r

    def get_state(self, psi_out=None, res_out=None):
        psi = np.empty(self.shape, dtype=self.complex) if psi_out is None else psi_out
        res = (np.empty(self.res_shape, dtype=self.real) if res_out is None else res_out) if self.reservoir else None
        p, dev, _ = _pointer(psi, self.complex, writable=True)
        r = _pointer(res, self.real, writable=True)[0] if res is not None else None
        _lib.check(self.lib.pg_get_state(self.handle, p, r, dev), "pg_get_state")
        return psi, res

    def state_pointers(self):
        p, r = C.c_void_p(), C.c_void_p()
        _lib.check(self.lib.pg_state_pointers(self.handle, C.byref(p), C.byref(r)), "pg_state_pointers")
        return p.value, r.value

    def set_pump(self, envelope):
        p, dev, keep = _pointer(envelope, self.real)
        _lib.check(self.lib.pg_set_pump(self.handle, p, dev), "pg_set_pump")

    def set_potential(self, potential):
        dtype = self.complex if self.potential_kind == _lib.PG_POT_COMPLEX else self.real
        p, dev, keep = _pointer(potential, dtype)
        _lib.check(self.lib.pg_set_potential(self.handle, p, dev), "pg_set_potential")

    def set_noise(self, seeds=None, gamma=None, scattering=None, strength=None, dt_over_4dv=0.0):
        if seeds is None:
            _lib.check(self.lib.pg_set_noise(self.handle, None, None, None, None, 0.0), "pg_set_noise")
            self.noise_on = False
            return
        m = self.members
        s = np.ascontiguousarray(np.broadcast_to(np.asarray(seeds, dtype=np.uint64), (m,)))
        g = np.ascontiguousarray(np.broadcast_to(np.asarray(gamma, dtype=np.float64), (m,)))
        r = np.ascontiguousarray(np.broadcast_to(np.asarray(scattering, dtype=np.float64), (m,)))
        st = np.ascontiguousarray(np.broadcast_to(np.asarray(strength, dtype=np.float64), (m,)))
        _lib.check(self.lib.pg_set_noise(self.handle, s.ctypes.data, g.ctypes.data, r.ctypes.data,
                                         st.ctypes.data, float(dt_over_4dv)), "pg_set_noise")
        self.noise_on = True

    def set_geometry(self, tile_w, strip_h):
        _lib.check(self.lib.pg_rk4_set_geometry(self.handle, int(tile_w), int(strip_h)),
                   "pg_rk4_set_geometry")

    def set_kernel(self, kind):
        """0 automatic, 1 tiled streaming kernel, 2 full-width FP32 kernel, 3 full-width kernel
        with four sites a thread (rows of 512 or 1024 sites)."""
        _lib.check(self.lib.pg_rk4_set_kernel(self.handle, int(kind)), "pg_rk4_set_kernel")

    def fail_next_graph(self, what):
        """Test hook: the next CUDA graph fails at capture (1) or instantiation (2)."""
        _lib.check(self.lib.pg_test_fail_next_graph(self.handle, int(what)), "pg_test_fail_next_graph")

    @property
    def graph_fallbacks(self) -> int:
        """Chunks that ran as plain launches because their graph could not be built."""
        return int(self.lib.pg_graph_fallbacks(self.handle))

    def sync_counts(self):
        """(host_syncs, throttle_waits): the library's waits for this solver's stream to drain,
        and the advance calls that waited for a staging slot still in use."""
        h, w = C.c_int64(), C.c_int64()
        _lib.check(self.lib.pg_sync_counts(self.handle, C.byref(h), C.byref(w)), "pg_sync_counts")
        return int(h.value), int(w.value)

    def set_wait_limit(self, polls):
        """100000 (the default: the polls each mbarrier wait of the TMA-fed kernels makes before it
        gives up) or 0: the kernels withhold each block's first row copy, so that a wait runs
        out on a healthy GPU and the next synchronising call reports PG_ERR_TIMEOUT."""
        _lib.check(self.lib.pg_set_wait_limit(self.handle, int(polls)), "pg_set_wait_limit")

    def kernel(self) -> int:
        k = C.c_int32()
        _lib.check(self.lib.pg_rk4_get_kernel(self.handle, C.byref(k)), "pg_rk4_get_kernel")
        return k.value

    def geometry(self):
        t, h = C.c_int32(), C.c_int32()
        _lib.check(self.lib.pg_rk4_get_geometry(self.handle, C.byref(t), C.byref(h)),
                   "pg_rk4_get_geometry")
        return t.value, h.value

    # -- stepping ----------------------------------------------------------------
    def _coefficients(self, values, *lead):
        """Pump coefficients as a C-contiguous (*lead, [L,] members) FP64 array."""
        shape = tuple(int(v) for v in lead) + ((self.pump_terms,) if self.pump_terms > 1 else ()) \
            + (self.members,)
        return np.ascontiguousarray(np.broadcast_to(np.asarray(values, dtype=np.float64), shape))

    def prepare(self, n_steps):
        """Build the CUDA graphs an ``advance`` of ``n_steps`` uses, launching nothing."""
        _lib.check(self.lib.pg_rk4_prepare(self.handle, int(n_steps)), "pg_rk4_prepare")

    def split_prepare(self, ordering, n_steps):
        """Build the CUDA graphs a ``split_advance`` of ``n_steps`` uses, launching nothing."""
        _lib.check(self.lib.pg_split_prepare(self.handle, int(ordering), int(n_steps)),
                   "pg_split_prepare")

    def advance(self, start_step, n_steps, stage_scales, use_graphs=True):
        """``stage_scales``: array (n_steps, 3, [L,] members) of pump coefficients."""
        scales = self._coefficients(stage_scales, n_steps, 3)
        _lib.check(self.lib.pg_rk4_advance(self.handle, int(start_step), int(n_steps),
                                           scales.ctypes.data, int(bool(use_graphs))),
                   "pg_rk4_advance")

    def split_advance(self, ordering, start_step, n_steps, half_scales, use_graphs=True):
        """Split-step Fourier steps; ``half_scales`` is (n_steps, 2, members): the pump
        coefficients at t + dt/4 and t + 3 dt/4.  ordering 0 = R/2 K/2 N K/2 R/2 (real-space
        state), 1 = K/2 [R/2 N R/2] K/2 (leaves the unnormalised spectrum)."""
        scales = self._coefficients(half_scales, n_steps, 2)
        _lib.check(self.lib.pg_split_advance(self.handle, int(ordering), int(start_step),
                                             int(n_steps), scales.ctypes.data,
                                             int(bool(use_graphs))), "pg_split_advance")

    def ifrk_advance(self, tableau, start_step, n_steps, stage_scales):
        """Fixed-step Lawson IFRK steps; tableau "rk4" or "dp5"; ``stage_scales`` is
        (n_steps, stages, members): pump coefficients at t + c_i dt."""
        tab, stages = _TABLEAUS[tableau]
        scales = self._coefficients(stage_scales, n_steps, stages)
        _lib.check(self.lib.pg_ifrk_advance(self.handle, tab, int(start_step), int(n_steps),
                                            scales.ctypes.data), "pg_ifrk_advance")

    def ifrk_trial(self, h, stage_scales, rtol, atol):
        """One adaptive Dormand-Prince trial; returns (error, accepted).  Accepted trials
        become the state."""
        scales = self._coefficients(stage_scales, 7)
        err = C.c_double()
        acc = C.c_int32()
        _lib.check(self.lib.pg_ifrk_trial(self.handle, 1, float(h), scales.ctypes.data, float(rtol),
                                          float(atol), C.byref(err), C.byref(acc)), "pg_ifrk_trial")
        return err.value, bool(acc.value)

    # -- FP64 observables ----------------------------------------------------------
    def accumulate(self, density=True, momentum=False):
        kinds = (1 if density else 0) | (2 if momentum else 0)
        _lib.check(self.lib.pg_accumulate(self.handle, kinds), "pg_accumulate")

    def accumulator_sums(self, kind):
        """(sums, samples) for kind "rho", "rho2" or "k" (shape (B, 1, ny, nx), FP64)."""
        index = {"rho": 0, "rho2": 1, "k": 2}[kind]
        out = np.empty(self.shape, dtype=np.float64)
        samples = C.c_int64()
        _lib.check(self.lib.pg_accumulator_sums(self.handle, index, out.ctypes.data, C.byref(samples)),
                   "pg_accumulator_sums")
        return out, samples.value

    def accumulator_reset(self):
        _lib.check(self.lib.pg_accumulator_reset(self.handle), "pg_accumulator_reset")

    def accumulator_zero(self):
        """Zero the sums without a host wait and without touching the steady-state monitor."""
        _lib.check(self.lib.pg_accumulator_zero(self.handle), "pg_accumulator_zero")

    def accumulator_load(self, kind, sums, samples):
        """Restore one accumulator (kind "rho", "rho2" or "k") and its sample count."""
        index = {"rho": 0, "rho2": 1, "k": 2}[kind]
        arr = np.ascontiguousarray(np.broadcast_to(np.asarray(sums, dtype=np.float64), self.shape))
        _lib.check(self.lib.pg_accumulator_load(self.handle, index, arr.ctypes.data, int(samples)),
                   "pg_accumulator_load")

    def steady_export(self):
        """(density (B, ny, nx) or None, norms or None, stop_steps) of the steady monitor."""
        density = np.empty((self.members, self.ny, self.nx), dtype=self.real)
        norms = np.empty(self.members)
        stops = np.empty(self.members, dtype=np.int64)
        have = C.c_int32()
        _lib.check(self.lib.pg_steady_export(self.handle, density.ctypes.data, norms.ctypes.data,
                                             stops.ctypes.data, C.byref(have)), "pg_steady_export")
        if not have.value:
            return None, None, stops
        return density, norms, stops

    def steady_import(self, density, norms, stop_steps=None):
        """Restore the monitor from :meth:`steady_export`'s values (density None: no reference)."""
        have = density is not None
        d = n = None
        if have:
            d = np.ascontiguousarray(np.asarray(density, dtype=self.real).reshape(self.members, self.ny,
                                                                                   self.nx))
            n = np.ascontiguousarray(np.asarray(norms, dtype=np.float64).reshape(self.members))
        st = None if stop_steps is None else np.ascontiguousarray(np.asarray(stop_steps, dtype=np.int64))
        _lib.check(self.lib.pg_steady_import(self.handle, None if d is None else d.ctypes.data,
                                             None if n is None else n.ctypes.data,
                                             None if st is None else st.ctypes.data, int(have)),
                   "pg_steady_import")

    def norms(self):
        out = np.empty(self.members, dtype=np.float64)
        _lib.check(self.lib.pg_norms(self.handle, out.ctypes.data), "pg_norms")
        return out

    def steady_check(self):
        """(relative density change, relative norm change, norms) per member."""
        rd = np.empty(self.members)
        rn = np.empty(self.members)
        nm = np.empty(self.members)
        _lib.check(self.lib.pg_steady_check(self.handle, rd.ctypes.data, rn.ctypes.data,
                                            nm.ctypes.data), "pg_steady_check")
        return rd, rn, nm

    # -- device-resident steady-state monitor -----------------------------------------
    def steady_reset(self):
        _lib.check(self.lib.pg_steady_reset(self.handle), "pg_steady_reset")

    def steady_update(self, step, record=True, rtol=1e-6, halt=False):
        """Enqueue one steady-state check (no wait); see ``pg_steady_update``."""
        _lib.check(self.lib.pg_steady_update(self.handle, int(step), int(bool(record)), float(rtol),
                                             int(bool(halt))), "pg_steady_update")

    def steady_poll(self):
        """(members stopped, index of the newest finished check), read without waiting."""
        stopped = C.c_int32()
        done = C.c_int64()
        _lib.check(self.lib.pg_steady_poll(self.handle, C.byref(stopped), C.byref(done)),
                   "pg_steady_poll")
        return int(stopped.value), int(done.value)

    def steady_results(self):
        """Waits; returns (rel_density, rel_norm, norms, stop_steps, halt_step or None)."""
        rd = np.empty(self.members)
        rn = np.empty(self.members)
        nm = np.empty(self.members)
        stops = np.empty(self.members, dtype=np.int64)
        halt = C.c_int64()
        _lib.check(self.lib.pg_steady_results(self.handle, rd.ctypes.data, rn.ctypes.data,
                                              nm.ctypes.data, stops.ctypes.data, C.byref(halt)),
                   "pg_steady_results")
        return rd, rn, nm, stops, (None if halt.value < 0 else int(halt.value))

    def set_state_kind(self, spectral: bool):
        _lib.check(self.lib.pg_set_state_kind(self.handle, int(bool(spectral))), "pg_set_state_kind")

    def state_kind(self) -> bool:
        k = C.c_int32()
        _lib.check(self.lib.pg_get_state_kind(self.handle, C.byref(k)), "pg_get_state_kind")
        return bool(k.value)

    @property
    def last_launch_count(self) -> int:
        return int(self.lib.pg_last_launch_count(self.handle))


def philox_words(counters, key: int) -> np.ndarray:
    """Device Philox-4x32-10 words for host counters of shape (..., 4)."""
    lib = _lib.load()
    ctr = np.ascontiguousarray(np.asarray(counters, dtype=np.uint32))
    if ctr.shape[-1] != 4:
        raise ValueError("counters must have four words")
    out = np.empty_like(ctr)
    n = ctr.size // 4
    _lib.check(lib.pg_philox_words(ctr.ctypes.data, C.c_uint64(int(key)), out.ctypes.data, n),
               "pg_philox_words")
    return out



def wigner_normals(counters, key: int, precision: str = "single") -> np.ndarray:
    """The device Box-Muller normals (2, ...) drawn from each counter's Philox words."""
    lib = _lib.load()
    ctr = np.ascontiguousarray(np.asarray(counters, dtype=np.uint32))
    n = ctr.size // 4
    dtype = np.float32 if precision == "single" else np.float64
    out = np.empty((n, 2), dtype=dtype)
    _lib.check(lib.pg_wigner_normals(ctr.ctypes.data, C.c_uint64(int(key)),
                                     _lib.PG_SINGLE if precision == "single" else _lib.PG_DOUBLE,
                                     out.ctypes.data, n), "pg_wigner_normals")
    return out.T.reshape(2, *ctr.shape[:-1])


Engine = RK4Engine
