"""Ragged design batch (needs a CUDA device).

A small batch built like the 64-design sweep (clamped bottom corners, circular
body force, p in {3, 4, 5}, random volume fraction and step size) runs through
concurrent workers; every design's history must equal its single-design run,
and one design is checked against the FP64 oracle's design loop.
"""
import threading
import time

import numpy as np
import pytest

from oracle.fem import Design, OracleSolver

pytestmark = pytest.mark.gpu


def _small_batch():
    from topomax_gb300.batch import BatchItem, config4_designs
    items = config4_designs(6, seed=3)
    sizes = [12, 20, 16, 24, 12, 20]  # small N: the oracle and the test stay fast
    return [BatchItem(n, it.design, it.name) for n, it in zip(sizes, items)]


def test_config4_generator():
    from topomax_gb300.batch import config4_designs
    items = config4_designs()
    assert len(items) == 64
    assert {it.N for it in items} <= {100, 150, 200, 250, 300}
    for it in items:
        pp = it.design["Elasticity"]["problem_parameters"]
        dp = it.design["Elasticity"]["domain_parameters"]
        assert pp["fixed_points"] == [[0.0, 0.0], [2.0, 0.0]] and pp["fixed_sides"] == []
        assert dp["penalties"][0] in (3.0, 4.0, 5.0)
        assert 0.3 <= dp["volume_fraction"] <= 0.5 and 1e-2 <= dp["fem_step_size"] <= 1e2


def test_batch_matches_single_runs_and_oracle():
    from topomax_gb300.batch import run_batch
    items = _small_batch()
    conc = run_batch(items, iterations=4, workers=3, rtol=1e-10)
    seq = run_batch(items, iterations=4, workers=1, rtol=1e-10)
    assert [r.name for r in conc] == [it.name for it in items]
    for a, b in zip(conc, seq):
        assert not a.error and not b.error
        for p in a.history:
            assert a.history[p]["objectives"] == b.history[p]["objectives"]
        assert np.array_equal(a.rho, b.rho)
    # one design against the FP64 oracle's loop
    it, res = items[0], conc[0]
    dp = it.design["Elasticity"]["domain_parameters"]
    pp = it.design["Elasticity"]["problem_parameters"]
    d = Design(dp["width"], dp["height"], dp["fem_step_size"], list(dp["penalties"]), dp["volume_fraction"],
               list(pp["fixed_sides"]), pp["body_force"], pp["tractions"], pp["filter_radius"],
               pp["young_modulus"], pp["poisson_ratio"], pp["fixed_points"])
    run = OracleSolver(it.N, d, max_iterations=4).solve()[0]
    got = res.history[dp["penalties"][0]]["objectives"]
    n = min(len(got), len(run.objectives))
    assert n >= 2
    rel = max(abs(a - b) / abs(b) for a, b in zip(got[:n], run.objectives[:n]))
    assert rel <= 1e-6


def test_contexts_created_while_the_default_stream_is_busy():
    """Context set-up writes device memory on the default stream (arena zeroing, host
    tables, the filter's stencils), and batch workers call on non-blocking streams that
    are not ordered after it.  The create call returns only when that work is done, so
    filters created and applied at once on a non-blocking stream, while another thread
    keeps the default stream busy with bounded sleep kernels, equal one made on a quiet
    device."""
    import torch
    import topomax_gb300 as tg
    mesh = tg.RectangleMesh(2.0, 1.0, 200, 100)
    V = tg.FunctionSpace(mesh, "CG", 1, dof_order="lattice")
    rho = np.random.default_rng(5).uniform(0, 1, V.dim())
    ref = tg.HelmholtzFilter(0.05, V, precision="mixed", rtol=1e-10).apply(rho).vector()[:]
    torch.cuda.synchronize()
    stop = threading.Event()

    def busy():
        # about 1 ms per sleep kernel at this GPU's clocks, at most two queued, for at most 5 s
        default = torch.cuda.default_stream()
        t0 = time.perf_counter()
        with torch.cuda.stream(default):
            while not stop.is_set() and time.perf_counter() - t0 < 5.0:
                torch.cuda._sleep(2_000_000)
                torch.cuda._sleep(2_000_000)
                default.synchronize()

    t = threading.Thread(target=busy)
    t.start()
    try:
        side = torch.cuda.Stream()
        got = []
        with torch.cuda.stream(side):
            for _ in range(4):
                f = tg.HelmholtzFilter(0.05, V, precision="mixed", rtol=1e-10)
                got.append(f.apply(rho).vector()[:])
                del f
    finally:
        stop.set()
        t.join()
    for g in got:
        assert np.max(np.abs(g - ref)) <= 1e-12 * np.max(np.abs(ref))
