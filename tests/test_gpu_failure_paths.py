"""Failure paths of the design loop through the C ABI, on the GPU, against the oracle.

No GPU fault is involved: each case is an input for which the reference's own code
fails the same way (a volume that no shift of the design can reach, a Newton iteration
that breaks down) or a solve capped below what it needs.

* ``src/solver.py:149-186`` (project) and ``src/utils.py:138-157`` (smart_brentq): a
  volume that cannot be bracketed within radius 2000 raises ValueError with smart_brentq's
  message, and ``Solver.solve`` (``src/solver.py:239-244``) stops with that message as its
  exit condition;
* a Newton run that breaks down (zero derivative) falls back to the bracketing search
  and lands on the same root as the oracle's Brent fallback;
* a Krylov solve capped below its need returns TOPO_ERR_NOT_CONVERGED (ValueError).
"""
import os

import numpy as np
import pytest
from scipy import optimize

from oracle.fem import OracleSolver, expit, expit_diff
from tests.test_gpu_parity import _design, _gpu_problem, _write_design

pytestmark = pytest.mark.gpu

NO_BRACKET = "f(-max_radius) and f(max_radius) must have different signs!"


def _solvers(N=10):
    import topomax_gb300 as tg
    d = _design()
    so = OracleSolver(N, d)
    s = tg.FEMSolver(N, _write_design(d), verbose=False, save=False, rtol=1e-10)
    return so, s


def test_unreachable_volume_raises_the_reference_error():
    import torch
    from topomax_gb300 import _capi
    so, s = _solvers()
    half = np.zeros(so.lattice.n_vertices)
    volume = 1.5 * s.width * s.height              # more than the domain holds
    with pytest.raises(ValueError) as ref:
        so.project(half, volume)
    with pytest.raises(_capi.TopoError) as got:
        s.project(torch.as_tensor(half), volume)
    assert str(ref.value) == NO_BRACKET
    assert str(got.value) == str(ref.value)
    assert got.value.code == _capi.TOPO_ERR_PROJECTION
    assert isinstance(got.value, ValueError)


def test_solver_stops_with_the_projection_error():
    """The loop catches the projection's ValueError and reports it as the exit condition,
    after the initial objective and before any design update (as the oracle's loop)."""
    so, s = _solvers()
    so.volume = s.volume = 1.5 * s.width * s.height
    rho0 = s.rho.tensor.clone()
    h = s.solve()[3.0]
    ref = so.solve()[0]
    assert h["exit_condition"] == ref.exit_condition == NO_BRACKET
    assert h["iterations"] == ref.iterations == 1
    assert len(h["objectives"]) == len(ref.objectives) == 1
    assert abs(h["objectives"][0] - ref.objectives[0]) <= 1e-8 * abs(ref.objectives[0])
    assert bool((s.rho.tensor == rho0).all())


def test_newton_breakdown_falls_back_to_the_bracketing_root():
    """half ~ -40: f'(0) ~ 1e-17, the first Newton step lands where expit saturates and
    f' = 0, so Newton stops (scipy raises, the device iteration flags it); the root
    c ~ 40 is then bracketed at radius 64 and found by both to ~1e-12."""
    import torch
    so, s = _solvers()
    rng = np.random.default_rng(5)
    half = -40.0 + rng.uniform(-0.5, 0.5, so.lattice.n_vertices)

    def error(c):
        return so.integrate(expit(half + c)) - so.volume

    def error_derivative(c):
        return so.integrate(expit_diff(half + c))

    with pytest.raises(RuntimeError):                 # Newton breaks down on the CPU too
        optimize.newton(error, 0, error_derivative, tol=1e-12, full_output=True)
    ref = so.project(half, so.volume)
    psi = s.project(torch.as_tensor(half), s.volume).cpu().numpy()
    assert 32.0 < s.last_multiplier < 64.0
    assert np.max(np.abs(psi - ref)) <= 1e-10
    assert abs(s.integrate(torch.sigmoid(torch.as_tensor(psi))) - s.volume) <= 1e-11


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_iteration_cap_reports_not_converged(precision):
    from topomax_gb300 import _capi
    d = _design()
    prob, V = _gpu_problem(d, 80, 40, precision=precision, rtol=1e-10)
    prob.set_penalization(3.0)
    rho = np.random.default_rng(6).uniform(0.01, 1.0, V.dim())
    prob.set_iteration_limit(1)
    with pytest.raises(_capi.TopoError) as e:
        prob.calculate_objective(rho)
    assert e.value.code == _capi.TOPO_ERR_NOT_CONVERGED
    assert isinstance(e.value, ValueError)
    with pytest.raises(ValueError):
        prob.set_iteration_limit(-1)
    # the context stays usable: back to the default caps, the same answer as a fresh problem
    prob.set_iteration_limit(0)
    C = prob.calculate_objective(rho)
    fresh, _ = _gpu_problem(d, 80, 40, precision=precision, rtol=1e-10)
    fresh.set_penalization(3.0)
    C_ref = fresh.calculate_objective(rho)
    assert abs(C - C_ref) <= 1e-9 * abs(C_ref)
