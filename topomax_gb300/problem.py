"""Problem interface of the design loop (the reference's src/problem.py:7-23)."""
from __future__ import annotations

from abc import ABC, abstractmethod
from typing import Any


class Problem(ABC):
    """State equation plus objective/gradient evaluation of a design problem."""

    @abstractmethod
    def set_penalization(self, penalization: float): ...

    @abstractmethod
    def calculate_objective_gradient(self) -> Any: ...

    @abstractmethod
    def calculate_objective(self, rho: Any) -> float: ...

    @abstractmethod
    def forward(self, rho: Any) -> Any: ...
