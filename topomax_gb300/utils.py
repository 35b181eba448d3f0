"""Result records of the design loop (the pickle layouts of the reference's src/utils.py)."""
from __future__ import annotations

from dataclasses import dataclass


@dataclass
class IterationData:
    domain_size: tuple
    objective: float
    iteration: int
    rho_file: str
    penalty: float


@dataclass
class SolverResult:
    exit_condition: str
    min_objective: float
    objectives: list
    iterations: int
    min_index: int
    times: list
