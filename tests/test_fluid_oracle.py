"""The Stokes-Brinkman fluid oracle (oracle/fluid.py) against the reference's known answer
(tests/test_fluid_solver.py: diffuser, N = 20, penalty 0.1).

Parity is partial and the bars say so: the design loop must end exactly as the
reference's (iteration 20, convergence threshold), the final objective within 1e-3
(the least-squares closure of the singular, slightly inconsistent pressure system is
5.6e-4 off the reference's MUMPS answer), and the sorted final design within 1e-2.
"""
import json
import os

import numpy as np
import pytest

from oracle.fluid import FluidDesign, FluidOracle, FluidOracleSolver, rule_degree7

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def test_degree7_rule_is_exact_to_degree_7():
    pts, w = rule_degree7()
    assert abs(w.sum() - 1.0) < 1e-14
    from math import factorial
    for a in range(8):
        for b in range(8 - a):
            exact = 2.0 * factorial(a) * factorial(b) / factorial(a + b + 2)  # 2 x int over the unit triangle
            got = float(np.sum(w * pts[:, 1] ** a * pts[:, 2] ** b))
            assert abs(got - exact) < 1e-14


@pytest.mark.parametrize("pressure", ["lsq", "mean"])
def test_diffuser_known_answer(pressure):
    """Both closures (the full system's least-squares solution, and the reduced system's
    that the GPU solver computes) end the loop as the reference does."""
    ref = json.load(open(os.path.join(GOLDEN, "diffuser_N20.json")))
    d = FluidDesign.from_dict(json.load(open(os.path.join(GOLDEN, "designs", ref["design"]))))
    s = FluidOracleSolver(ref["N"], d, pressure=pressure)
    flux = s.oracle.boundary_flux()
    assert abs(flux) < 1e-3  # the interpolated outflow profile's mass defect (2/3 in, 2/3 out)
    run = s.solve()[0]
    assert run.iterations == ref["iteration"]
    assert run.exit_condition == "Convergence treshold reached"
    assert abs(run.objectives[-1] - ref["objective"]) <= 1e-3 * ref["objective"]
    assert np.max(np.abs(np.sort(run.rho) - np.asarray(ref["rho_sorted"]))) <= 1e-2
    assert abs(run.rho.sum() - ref["rho_sum"]) <= 1e-2 * ref["rho_sum"]


def test_state_solution_is_divergence_free_and_meets_the_boundary_data():
    ref = json.load(open(os.path.join(GOLDEN, "diffuser_N20.json")))
    d = FluidDesign.from_dict(json.load(open(os.path.join(GOLDEN, "designs", ref["design"]))))
    from oracle.fem import Lattice
    o = FluidOracle(Lattice(1.0, 1.0, 20, 20), d)
    o.set_penalization(0.1)
    rho = np.random.default_rng(7).uniform(0.0, 1.0, o.nv)
    u, p = o.state_solve(rho)
    assert np.max(np.abs(u[o.bc_dofs] - o.bc_vals)) < 1e-6  # least squares moves the data by ~flux/|y|
    K = o.assemble(rho).tocsr()
    cont = K[o.nuv:, :o.nuv] @ u
    assert np.max(np.abs(cont)) < 1e-5
    g = o.gradient(rho, u)
    assert g.shape == rho.shape and np.all(np.isfinite(g))
    # the L2 projection keeps the integral of 1/2 alpha'(rho) |u|^2 (negative: alpha' < 0)
    total = float(np.sum(o.M1 @ g))
    assert total < 0
    rhs = 0.0
    for t in o.tab:
        uq, _ = o._u_at(u, t, t["N7"])
        from oracle.fluid import fluid_penalty_derivative
        dr = fluid_penalty_derivative(o._rho_at(rho, t, t["lam7"]), 0.1)
        rhs += float(np.sum(0.5 * dr * np.sum(uq * uq, axis=2) * t["w7"][None] * t["area"]))
    assert abs(total - rhs) <= 1e-10 * abs(rhs)


def test_twin_pipe_gradient_matches_finite_differences():
    """tests/test_fluid_gradient.py of the reference, on the oracle: the twin pipe at N = 10,
    penalty 0.1, forward differences of the objective along the constant direction
    volume / volume_fraction against int 1/2 alpha'(rho) direction |u|^2 dx, at t = 1e-3 and
    1e-7.  The reference's check is kept as it is written: ``Polynomial.fit`` works in a
    scaled variable, so its ``coef[1] >= 4`` asks for a log-log slope of at least
    4 / 4.6 (4.6 = half the width of log t over the two steps), i.e. first order."""
    with open(os.path.join(GOLDEN, "designs", "twin_pipe.json")) as f:
        d = FluidDesign.from_dict(json.load(f))
    s = FluidOracleSolver(10, d)
    o = s.oracle
    s.problem.set_penalization(0.1)
    rho = s.rho.copy()
    J = s.problem.calculate_objective(rho)
    direction = np.full_like(rho, s.volume / d.volume_fraction)
    gradient = float(direction @ (o.M1 @ o.gradient(rho, s.problem.u)))
    ts = [1e-3, 1e-7]
    errors = [abs((s.problem.calculate_objective(rho + t * direction) - J) / t - gradient) for t in ts]
    poly = np.polynomial.Polynomial.fit(np.log(ts), np.log(errors), 1)
    assert poly.coef[1] >= 4
    assert poly.convert().coef[1] > 0.9  # the plain slope: first-order forward differences
