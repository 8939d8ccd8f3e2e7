"""Solver contract used when the Polarism package is not installed.

Same names, fields and defaults as ``polarism/solver/abstract_solver.py:11-101``
(``StepReport``, ``SolverCapabilities``, ``AbstractSolver``) so the drop-in solvers
have one code path with or without the reference installed.
"""
from __future__ import annotations

from abc import ABC, abstractmethod
from dataclasses import dataclass
from typing import ClassVar


@dataclass(frozen=True)
class StepReport:
    accepted: bool = True
    error: float | None = None
    dt_next: float | None = None


ACCEPTED = StepReport()

_BUILTIN_RESERVOIRS = frozenset({"single", "double", "quadratic-double", "none"})


@dataclass(frozen=True)
class SolverCapabilities:
    components: frozenset = frozenset({1})
    ndim: frozenset = frozenset({2})
    grid_types: frozenset = frozenset({"periodic"})
    reservoirs: frozenset = _BUILTIN_RESERVOIRS
    custom_reservoirs: str = "quantitative"
    potential: bool = True
    kinetic_relaxation: bool = False
    dispersion: frozenset = frozenset({"parabolic"})
    terms: bool = True
    noise: frozenset = frozenset({"none", "wigner"})
    adaptive: bool = False
    coherent_drive: bool = False
    time_dependent_potential: bool = False
    quantitative_reservoirs: frozenset = _BUILTIN_RESERVOIRS
    description: str = ""

    def __post_init__(self):
        for name in ("components", "ndim", "grid_types", "reservoirs", "dispersion", "noise",
                     "quantitative_reservoirs"):
            object.__setattr__(self, name, frozenset(getattr(self, name)))


class AbstractSolver(ABC):
    capabilities: ClassVar[SolverCapabilities] = SolverCapabilities()
    injects_noise: ClassVar[bool] = False

    def __init__(self, config, grid, model):
        import numpy as np

        self.config = config
        self.physics = config.physics
        self.batch_physics = model.physics
        self.xp = np

    @abstractmethod
    def step(self, model, state, dt) -> StepReport:
        raise NotImplementedError

    def advance(self, model, state, n_steps: int) -> None:
        for _ in range(n_steps):
            completed = state.step
            report = self.step(model, state, self.config.solver.dt)
            if report.accepted and model.noise is not None and not self.injects_noise:
                model.noise.apply_to_state(state, model.reservoir, completed)
