"""ctypes binding of libpolarism_gb300.so (the C ABI declared in include/polarism_gb300.h).

The library is built in-tree (``polarism_gb300/_build``).  There is no CPU
fallback: loading fails loudly when the library is missing, and every non-zero
status becomes a ``RuntimeError`` carrying ``pg_last_error()``.
"""
from __future__ import annotations

import ctypes as C
import os
import threading
from pathlib import Path

_PKG = Path(__file__).resolve().parent
LIBRARY_PATH = _PKG / "_build" / "libpolarism_gb300.so"

PG_OK, PG_ERR_INVALID, PG_ERR_CUDA, PG_ERR_UNSUPPORTED, PG_ERR_TIMEOUT = 0, 1, 2, 3, 4
PG_SINGLE, PG_DOUBLE = 0, 1
PG_RES_NONE, PG_RES_SINGLE, PG_RES_DOUBLE, PG_RES_QDOUBLE = 0, 1, 2, 3
PG_POT_NONE, PG_POT_REAL, PG_POT_COMPLEX = 0, 1, 2


class PgPhysics(C.Structure):
    """Mirror of ``pg_physics``."""

    _fields_ = [(name, C.c_double) for name in (
        "hbar", "m_eff", "g_C", "g_R", "g_I", "R", "gamma_C", "gamma_R",
        "kinetic_relaxation_eta", "gamma_I", "gamma_A", "R_IA", "R_AI", "alpha_2", "zeeman",
        "te_tm", "pump_weight_plus", "pump_weight_minus", "kappa")]


class PgConfig(C.Structure):
    """Mirror of ``pg_config``."""

    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("members", C.c_int32),
                ("precision", C.c_int32), ("reservoir", C.c_int32), ("potential", C.c_int32),
                ("pump_per_member", C.c_int32), ("potential_per_member", C.c_int32),
                ("dx", C.c_double), ("dy", C.c_double), ("dt", C.c_double),
                ("components", C.c_int32), ("reservoir_components", C.c_int32),
                ("pump_terms", C.c_int32), ("reserved_", C.c_int32)]


class PgSweepGrid(C.Structure):
    """Mirror of pg_sweep_grid (one sweep member's periodic grid)."""

    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("dx", C.c_double), ("dy", C.c_double)]


_vp = C.c_void_p
_i32, _i64, _u64, _f64 = C.c_int32, C.c_int64, C.c_uint64, C.c_double

# name -> (restype, argtypes); the exported surface of include/polarism_gb300.h.
SIGNATURES = {
    "pg_last_error": (C.c_char_p, []),
    "pg_device_count": (C.c_int, []),
    "pg_version": (C.c_int, []),
    "pg_create": (C.c_int, [C.POINTER(PgConfig), C.POINTER(PgPhysics), C.POINTER(_vp)]),
    "pg_destroy": (None, [_vp]),
    "pg_stream": (_vp, [_vp]),
    "pg_synchronize": (C.c_int, [_vp]),
    "pg_set_state": (C.c_int, [_vp, _vp, _vp, C.c_int]),
    "pg_get_state": (C.c_int, [_vp, _vp, _vp, C.c_int]),
    "pg_state_pointers": (C.c_int, [_vp, C.POINTER(_vp), C.POINTER(_vp)]),
    "pg_set_pump": (C.c_int, [_vp, _vp, C.c_int]),
    "pg_set_potential": (C.c_int, [_vp, _vp, C.c_int]),
    "pg_set_noise": (C.c_int, [_vp, _vp, _vp, _vp, _vp, _f64]),
    "pg_rk4_advance": (C.c_int, [_vp, _i64, _i32, _vp, C.c_int]),
    "pg_rk4_prepare": (C.c_int, [_vp, _i32]),
    "pg_rk4_set_geometry": (C.c_int, [_vp, _i32, _i32]),
    "pg_rk4_get_geometry": (C.c_int, [_vp, C.POINTER(_i32), C.POINTER(_i32)]),
    "pg_split_advance": (C.c_int, [_vp, _i32, _i64, _i32, _vp, C.c_int]),
    "pg_split_prepare": (C.c_int, [_vp, _i32, _i32]),
    "pg_set_state_kind": (C.c_int, [_vp, _i32]),
    "pg_get_state_kind": (C.c_int, [_vp, C.POINTER(_i32)]),
    "pg_ifrk_advance": (C.c_int, [_vp, _i32, _i64, _i32, _vp]),
    "pg_ifrk_trial": (C.c_int, [_vp, _i32, _f64, _vp, _f64, _f64, C.POINTER(_f64), C.POINTER(_i32)]),
    "pg_accumulate": (C.c_int, [_vp, _i32]),
    "pg_accumulator_sums": (C.c_int, [_vp, _i32, _vp, C.POINTER(_i64)]),
    "pg_accumulator_reset": (C.c_int, [_vp]),
    "pg_accumulator_zero": (C.c_int, [_vp]),
    "pg_norms": (C.c_int, [_vp, _vp]),
    "pg_steady_check": (C.c_int, [_vp, _vp, _vp, _vp]),
    "pg_steady_update": (C.c_int, [_vp, C.c_int64, C.c_int32, C.c_double, C.c_int32]),
    "pg_steady_poll": (C.c_int, [_vp, _vp, _vp]),
    "pg_steady_results": (C.c_int, [_vp, _vp, _vp, _vp, _vp, _vp]),
    "pg_steady_reset": (C.c_int, [_vp]),
    "pg_steady_export": (C.c_int, [_vp, _vp, _vp, _vp, _vp]),
    "pg_steady_import": (C.c_int, [_vp, _vp, _vp, _vp, C.c_int32]),
    "pg_accumulator_load": (C.c_int, [_vp, C.c_int32, _vp, C.c_int64]),
    "pg_field_norms": (C.c_int, [_vp, _i32, _i32, _i64, _f64, _vp, _vp]),
    "pg_field_norms_noalloc": (C.c_int, [_vp, _i32, _i32, _i64, _f64, _vp, _vp]),
    "pg_rk4_set_kernel": (C.c_int, [_vp, _i32]),
    "pg_rk4_get_kernel": (C.c_int, [_vp, C.POINTER(_i32)]),
    "pg_set_wait_limit": (C.c_int, [_vp, _i32]),
    "pg_test_fail_next_graph": (C.c_int, [_vp, _i32]),
    "pg_graph_fallbacks": (_i64, [_vp]),
    "pg_sync_counts": (C.c_int, [_vp, C.POINTER(_i64), C.POINTER(_i64)]),
    "pg_last_launch_count": (_i64, [_vp]),
    "pg_philox_words": (C.c_int, [_vp, _u64, _vp, _i64]),
    "pg_wigner_normals": (C.c_int, [_vp, _u64, _i32, _vp, _i64]),
    "pg_sweep_create": (C.c_int, [_i32, C.POINTER(PgSweepGrid), C.POINTER(PgPhysics), _f64,
                                  C.POINTER(_vp)]),
    "pg_sweep_destroy": (None, [_vp]),
    "pg_sweep_stream": (_vp, [_vp]),
    "pg_sweep_total_sites": (_i64, [_vp]),
    "pg_sweep_offsets": (C.c_int, [_vp, _vp]),
    "pg_sweep_set_state": (C.c_int, [_vp, _vp, _vp, C.c_int]),
    "pg_sweep_get_state": (C.c_int, [_vp, _vp, _vp, C.c_int]),
    "pg_sweep_state_pointers": (C.c_int, [_vp, C.POINTER(_vp), C.POINTER(_vp)]),
    "pg_sweep_set_pump": (C.c_int, [_vp, _vp, C.c_int]),
    "pg_sweep_set_noise": (C.c_int, [_vp, _vp, _vp, _vp, _vp]),
    "pg_sweep_set_tiling": (C.c_int, [_vp, _i32, _i32]),
    "pg_sweep_get_tiling": (C.c_int, [_vp, C.POINTER(_i32), C.POINTER(_i32), C.POINTER(_i32),
                                      C.POINTER(_i32)]),
    "pg_sweep_set_wait_limit": (C.c_int, [_vp, _i32]),
    "pg_sweep_set_active": (C.c_int, [_vp, _vp]),
    "pg_sweep_advance": (C.c_int, [_vp, _i64, _i32, _vp, C.c_int]),
    "pg_sweep_last_time_ms": (C.c_int, [_vp, C.POINTER(C.c_float)]),
    "pg_sweep_last_launch_count": (_i64, [_vp]),
    "pg_sweep_synchronize": (C.c_int, [_vp]),
    "pg_sweep_steady_check": (C.c_int, [_vp, _vp, _vp, _vp]),
    "pg_sweep_steady_reset": (C.c_int, [_vp]),
    "pg_sweep_steady_update": (C.c_int, [_vp, _i64, _i32, _f64, _i32]),
    "pg_sweep_steady_poll": (C.c_int, [_vp, C.POINTER(_i32), C.POINTER(_i64)]),
    "pg_sweep_steady_results": (C.c_int, [_vp, _vp, _vp, _vp, _vp, C.POINTER(_i64)]),
    "pg_sweep_sync_counts": (C.c_int, [_vp, C.POINTER(_i64), C.POINTER(_i64)]),
    "pg_gemm_bf16": (C.c_int, [_vp, _vp, _vp, _i32, _i32, _i32, _i32, _i32, _i32, _i32, _i32,
                               C.c_float, C.c_float, _i32, _i64, _i64, _i64, _vp]),
    "pg_gemm_bf16_2d": (C.c_int, [_vp, _vp, _vp, _i32, _i32, _i32, _i32, _i32, _i32, _i32, _i32,
                                  C.c_float, C.c_float, _i32, _i64, _i64, _i64, _i32, _i64, _i64,
                                  _i64, _vp]),
    "pg_fno_sum_slices": (C.c_int, [_vp, _vp, _i64, _i32, _i32, _vp]),
    "pg_gemm_set_engine": (C.c_int, [_i32]),
    "pg_gemm_timeouts": (C.c_int, [C.POINTER(_i32), _i32]),
    "pg_fno_to_bf16": (C.c_int, [_vp, _vp, _i64, _vp]),
    "pg_fno_bias_act": (C.c_int, [_vp, _vp, _vp, _vp, _i32, _i64, _i64, _i32, _vp]),
    "pg_fno_gelu_backward": (C.c_int, [_vp, _vp, _vp, _vp, _i64, _vp]),
    "pg_fno_channel_sum": (C.c_int, [_vp, _vp, _i32, _i32, _i64, _i32, _vp]),
    "pg_fno_mode_mix": (C.c_int, [_vp, _vp, _vp, _vp, _i32, _i32, _i32, _i32, _vp]),
    "pg_fno_mode_mix_backward": (C.c_int, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _i32, _i32, _i32,
                                           _i32, _vp]),
    "pg_fno_adam": (C.c_int, [_vp, _vp, _vp, _vp, _vp, _i64, C.c_float, C.c_float, C.c_float,
                              C.c_float, _i64, C.c_float, _vp]),
    "pg_fno_mse": (C.c_int, [_vp, _vp, _vp, _i32, _i64, _vp, _vp, _vp, _i32, _i64, C.c_float,
                             C.POINTER(_i32), _vp]),
}

_lock = threading.Lock()
_lib = None


def load(path: str | os.PathLike | None = None):
    """Load (once) and return the library with typed entry points."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        target = Path(path or os.environ.get("PG_LIBRARY", LIBRARY_PATH))
        if not target.exists():
            raise RuntimeError(
                f"libpolarism_gb300 is not built ({target} missing); run "
                "`python -m polarism_gb300.build` (or __graft_entry__.build()) first")
        lib = C.CDLL(str(target))
        for name, (restype, argtypes) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = restype
            fn.argtypes = argtypes
        _lib = lib
        return lib


def check(status: int, what: str = "") -> None:
    """Raise RuntimeError for a non-zero library status."""
    if status != PG_OK:
        message = (_lib.pg_last_error() or b"").decode(errors="replace") if _lib else ""
        kind = {PG_ERR_INVALID: "invalid argument", PG_ERR_CUDA: "CUDA error",
                PG_ERR_UNSUPPORTED: "unsupported", PG_ERR_TIMEOUT: "device wait timed out"}
        raise RuntimeError(f"{what or 'polarism_gb300'}: {kind.get(status, status)}: {message}")


def header_symbols() -> list[str]:
    """Function names declared in include/polarism_gb300.h (for the export test)."""
    import re

    text = (_PKG.parent / "include" / "polarism_gb300.h").read_text()
    body = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(pg_[a-z0-9_]+)\s*\(", body)))
