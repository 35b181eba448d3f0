"""The Stokes-Brinkman fluid problem on the GPU against the oracle (oracle/fluid.py).

The kernels' triangle phases and gathers, and the formulation of the state solve,
are also checked on the CPU in test_fluid_emulated.py.  The file name makes pytest
collect it after the elasticity tests.
"""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _design():
    from oracle.fluid import FluidDesign
    return FluidDesign.from_dict(json.load(open(os.path.join(GOLDEN, "designs", "diffuser.json"))))


def _problem(nx, ny, q=0.1):
    import topomax_gb300 as tg
    from topomax_gb300.fem import RectangleMesh
    domain, params = tg.parse_design(os.path.join(GOLDEN, "designs", "diffuser.json"))
    from topomax_gb300.fluid import FluidProblem
    prob = FluidProblem(RectangleMesh(domain.width, domain.height, nx, ny), params, domain, rtol=1e-12)
    prob.set_penalization(q)
    return prob


def _oracle(nx, ny, q=0.1):
    from oracle.fem import Lattice
    from oracle.fluid import FluidOracle
    d = _design()
    o = FluidOracle(Lattice(d.width, d.height, nx, ny), d, pressure="mean")
    o.set_penalization(q)
    return o


def test_fluid_operator_and_boundary_data_match_oracle():
    import torch
    nx, ny = 12, 10
    prob, o = _problem(nx, ny), _oracle(nx, ny)
    rng = np.random.default_rng(1)
    rho = rng.uniform(0.0, 1.0, o.nv)
    x = rng.standard_normal(o.n)
    y = prob.apply_operator(torch.as_tensor(rho).cuda(), torch.as_tensor(x).cuda()).cpu().numpy()
    s = np.ones(o.n)
    s[o.nuv:] = -1.0
    ref = s * (o.assemble(rho) @ x)
    assert np.max(np.abs(y - ref)) <= 1e-12 * np.max(np.abs(ref))
    ub = prob.boundary_values().cpu().numpy()
    want = np.zeros(o.nuv)
    want[o.bc_dofs] = o.bc_vals
    assert np.array_equal(ub, want)


@pytest.mark.parametrize("kind", ["random", "channel"])
def test_fluid_state_objective_gradient_match_oracle(kind):
    import torch
    nx = ny = 24
    prob, o = _problem(nx, ny), _oracle(nx, ny)
    if kind == "random":
        rho = np.random.default_rng(2).uniform(0.0, 1.0, o.nv)
    else:
        X, Y = np.meshgrid(np.linspace(0, 1, nx + 1), np.linspace(0, 1, ny + 1))
        rho = np.where(np.abs(Y - 0.5) < 0.5 - X / 3.0, 1.0, 0.0).ravel()
    J = prob.calculate_objective(torch.as_tensor(rho).cuda())
    u_ref, p_ref = o.state_solve(rho)
    u = prob.u.tensor.cpu().numpy()
    assert np.max(np.abs(u - u_ref)) <= 1e-8 * np.max(np.abs(u_ref))
    p = prob.p.tensor.cpu().numpy()
    assert np.max(np.abs(p - p_ref)) <= 1e-7 * np.max(np.abs(p_ref))
    J_ref = o.objective(rho, u_ref)
    assert abs(J - J_ref) <= 1e-9 * abs(J_ref)
    g = prob.calculate_objective_gradient().tensor.cpu().numpy()
    g_ref = o.gradient(rho, u_ref)
    assert np.max(np.abs(g - g_ref)) <= 1e-7 * np.max(np.abs(g_ref))


def test_fluid_design_loop_matches_oracle_and_known_answer(tmp_path):
    """Diffuser, N = 20 (tests/test_fluid_solver.py of the reference): the loop ends as the
    reference's (iteration 20, convergence threshold); the objective equals the oracle's
    closure to 1e-6 and the reference's MUMPS answer to 1e-3."""
    from oracle.fluid import FluidOracleSolver
    from topomax_gb300.solver import FEMSolver
    ref = json.load(open(os.path.join(GOLDEN, "diffuser_N20.json")))
    s = FEMSolver(ref["N"], os.path.join(GOLDEN, "designs", "diffuser.json"), data_path=str(tmp_path),
                  precision="fp64", rtol=1e-12, verbose=False, save=False)
    h = s.solve()[ref["penalty"]]
    orun = FluidOracleSolver(ref["N"], _design(), pressure="mean").solve()[0]
    assert h["iterations"] == ref["iteration"] == orun.iterations
    assert h["exit_condition"] == "Convergence treshold reached"
    assert abs(h["objectives"][-1] - orun.objectives[-1]) <= 1e-6 * abs(orun.objectives[-1])
    assert abs(h["objectives"][-1] - ref["objective"]) <= 1e-3 * ref["objective"]


def test_twin_pipe_gradient_matches_finite_differences(tmp_path):
    """tests/test_fluid_gradient.py of the reference, through FEMSolver on the GPU: forward
    differences of the objective along volume / volume_fraction against
    int 1/2 alpha'(rho) direction |u|^2 dx at t = 1e-3 and 1e-7, with the reference's
    own (scaled-variable) fit.  The objective is the energy the state minimises under the
    divergence constraint, so a solve error enters it at second order: rtol 1e-12 leaves
    the t = 1e-7 difference intact."""
    import torch
    from topomax_gb300.solver import FEMSolver
    s = FEMSolver(10, os.path.join(GOLDEN, "designs", "twin_pipe.json"), data_path=str(tmp_path),
                  precision="fp64", rtol=1e-12, verbose=False, save=False)
    s.problem.set_penalization(0.1)
    rho = s.rho.tensor.clone()
    J = s.problem.calculate_objective(rho)
    direction = torch.full_like(rho, s.volume / s.parameters.volume_fraction)
    gradient = float(torch.dot(s.problem.gradient_rhs(rho, s.problem.u), direction))
    ts = [1e-3, 1e-7]
    errors = [abs((s.problem.calculate_objective(rho + t * direction) - J) / t - gradient) for t in ts]
    poly = np.polynomial.Polynomial.fit(np.log(ts), np.log(errors), 1)
    assert poly.coef[1] >= 4
