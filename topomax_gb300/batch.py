"""Many independent designs on one GPU (the ragged design batch).

Designs are independent (no data exchange), so a batch is a set of design
loops: ``run_batch`` gives each worker thread its own CUDA stream and its own
library contexts and hands it designs from a shared queue (largest first).  The
C ABI releases the Python interpreter lock during its calls, so the workers'
solves overlap on the GPU.  Every design's result is the same as a
single-design run.

``config4_designs`` builds the 64-design sweep: domain 2 x 1, N ~ U{100, 150,
200, 250, 300} (nx = 2N, ny = N), bottom corners clamped (points; the reference
can clamp whole sides only), circular body force r = 0.05, value (0, -1), centre
(1.0, U(0.3, 0.7)), p in {3, 4, 5}, vf ~ U(0.3, 0.5), step size log-uniform in
[1e-2, 1e2], seed 3.
"""
from __future__ import annotations

import queue
import threading
import time
from dataclasses import dataclass, field

import numpy as np
import torch

from .solver import FEMSolver


@dataclass
class BatchItem:
    N: int
    design: dict
    name: str = ""


@dataclass
class BatchResult:
    name: str
    N: int
    history: dict = field(default_factory=dict)
    rho: np.ndarray | None = None
    error: str = ""
    setup_s: float = 0.0   # wall time of the design's set-up (contexts, load vectors, filter)
    solve_s: float = 0.0   # wall time of its design loop


def config4_designs(count: int = 64, seed: int = 3) -> list[BatchItem]:
    rng = np.random.default_rng(seed)
    items = []
    for k in range(count):
        N = int(rng.choice([100, 150, 200, 250, 300]))
        p = float(rng.choice([3.0, 4.0, 5.0]))
        vf = float(rng.uniform(0.3, 0.5))
        alpha = float(10 ** rng.uniform(-2.0, 2.0))
        cy = float(rng.uniform(0.3, 0.7))
        design = {
            "name": f"batch{k:02d}",
            "Elasticity": {
                "domain_parameters": dict(width=2.0, height=1.0, fem_step_size=alpha, dem_step_size=alpha,
                                          penalties=[p], volume_fraction=vf),
                "problem_parameters": dict(fixed_sides=[], fixed_points=[[0.0, 0.0], [2.0, 0.0]],
                                           body_force=dict(region=dict(center=[1.0, cy], radius=0.05),
                                                           value=[0.0, -1.0]),
                                           tractions=None, filter_radius=0.05, young_modulus=1.0,
                                           poisson_ratio=0.3)}}
        items.append(BatchItem(N, design, design["name"]))
    return items


def _run_one(item: BatchItem, iterations: int, precision: str, rtol: float) -> BatchResult:
    res = BatchResult(item.name, item.N)
    try:
        t0 = time.perf_counter()
        solver = FEMSolver(item.N, dict(item.design, name=item.name), precision=precision, rtol=rtol,
                           verbose=False, save=False, max_iterations=iterations)
        t1 = time.perf_counter()
        res.history = solver.solve()
        torch.cuda.current_stream().synchronize()
        res.setup_s, res.solve_s = t1 - t0, time.perf_counter() - t1
        res.rho = solver.to_array(solver.rho)
    except (ValueError, RuntimeError) as e:
        res.error = str(e)
    return res


def run_batch(items: list[BatchItem], iterations: int, *, workers: int = 4, precision: str = "mixed",
              rtol: float = 1e-8) -> list[BatchResult]:
    """Runs every design's EMD loop (at most ``iterations`` steps per penalty) and returns
    the results in input order."""
    results: list[BatchResult | None] = [None] * len(items)
    order = sorted(range(len(items)), key=lambda i: -items[i].N)  # largest first: better packing
    work: queue.Queue = queue.Queue()
    for i in order:
        work.put(i)
    device = torch.cuda.current_device()

    def worker():
        torch.cuda.set_device(device)
        stream = torch.cuda.Stream()
        with torch.cuda.stream(stream):
            while True:
                try:
                    i = work.get_nowait()
                except queue.Empty:
                    break
                results[i] = _run_one(items[i], iterations, precision, rtol)
        stream.synchronize()

    threads = [threading.Thread(target=worker) for _ in range(max(1, min(workers, len(items))))]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    return [r for r in results if r is not None]
