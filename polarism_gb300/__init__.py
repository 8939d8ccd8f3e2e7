"""GB300-native (sm_103a) time-stepping hot path for Polarism's driven-dissipative GPE.

Python host code mirrors the reference's solver interface and calls hand-written
CUDA kernels through the C ABI in ``include/polarism_gb300.h`` (ctypes).  Build the
library with ``python -m polarism_gb300.build``.

``register()`` installs the drop-in solvers into Polarism's solver registry when
Polarism is importable.
"""
from __future__ import annotations

__version__ = "0.1.0"

SOLVER_NAMES = {
    "rk4-cuda": "RK4CudaSolver",
    "split-step-fft": "SplitStepFFTSolver",
    "split-step-fft-cuda": "SplitStepFFTCudaSolver",
    "ifrk-fft-cuda": "IFRKFFTCudaSolver",
    "ifrk4-fft-cuda": "IFRK4FFTCudaSolver",
}


def register(names=None):
    """Register the GB300 solvers in ``polarism.solver.solver_registry``.

    Mirrors ``@register_solver(name)`` (``polarism/solver/solver_registry.py:12-16``);
    an existing registration is overridden with the registry's own warning.
    """
    from polarism.solver.solver_registry import available_solvers

    from polarism_gb300 import solvers

    registered = {}
    for name, cls_name in SOLVER_NAMES.items():
        if names is not None and name not in names:
            continue
        cls = getattr(solvers, cls_name)
        available_solvers.register(name)(cls)
        registered[name] = cls
    return registered
