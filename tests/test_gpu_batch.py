"""Ragged design batch (needs a CUDA device).

A small batch built like the 64-design sweep (clamped bottom corners, circular
body force, p in {3, 4, 5}, random volume fraction and step size) runs through
concurrent workers; every design's history must equal its single-design run,
and one design is checked against the FP64 oracle's design loop.
"""
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
