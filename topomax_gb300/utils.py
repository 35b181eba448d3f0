"""Result records, timer and root-finder helper (the reference's src/utils.py)."""
from __future__ import annotations

import time
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


class Timer:
    def __init__(self, task: str | None = None):
        self.task = task.capitalize() if task else None
        self.start_time = time.time()

    def __enter__(self):
        return self

    def __exit__(self, *_):
        msg = self.get_time_string()
        print(msg if self.task is None else f"{self.task} took {msg}")

    def restart(self):
        self.start_time = time.time()

    def get_time_seconds(self):
        return time.time() - self.start_time

    def get_time_string(self):
        return prettify_seconds(self.get_time_seconds())


def prettify_seconds(seconds: float) -> str:
    whole = int(seconds)
    ms = (seconds - whole) * 1000
    if whole == 0:
        return f"{ms:.3g}ms"
    if whole < 60:
        return f"{whole:d}s {ms:.0f}ms"
    if seconds < 3600:
        return f"{whole // 60:d}m {whole % 60:d}s {ms:.0f}ms"
    return f"{whole // 3600:d}h {(whole % 3600) // 60:d}m {whole % 60:d}s {ms:.0f}ms"
