"""Compliance autograd against central finite differences (needs a CUDA device).

The 400 x 200 workload: domain 2 x 1, left side clamped, traction (0, -1) on the
right side centred at 0.5 with length 0.2, rho ~ U(0.05, 1) (seed 1), FP32 inner
solves inside FP64 refinement.  Central differences with h = 1e-6 on 200 random
CG1 vertices (seed 2) are compared with the backward pass, which returns
M1 g (the Euclidean gradient; g is the reference's CG1 Riesz representative),
and the mixed-precision gradient with the plain-FP64 one.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _problem(precision, rtol):
    import topomax_gb300 as tg
    from topomax_gb300.designs import parse_design_dict
    dd = {"Elasticity": {
        "domain_parameters": dict(width=2.0, height=1.0, fem_step_size=0.002, dem_step_size=0.002,
                                  penalties=[3.0], volume_fraction=0.5),
        "problem_parameters": dict(fixed_sides=["Left"], body_force=None,
                                   tractions=[dict(side="Right", center=0.5, length=0.2, value=[0.0, -1.0])],
                                   filter_radius=0.05, young_modulus=1.0, poisson_ratio=0.3)}}
    dom, par = parse_design_dict(dd)
    mesh = tg.RectangleMesh(2.0, 1.0, 400, 200)
    V = tg.FunctionSpace(mesh, "CG", 1, dof_order="lattice")
    prob = tg.ElasticityProblem(mesh, V, dom, par, precision=precision, rtol=rtol)
    prob.set_penalization(3.0)
    return prob, V


def test_compliance_gradient_matches_central_differences():
    """C = f.u is linear in a solve's error, so differences with h = 1e-6 need solves
    accurate to ~1e-13: they are evaluated on the plain-FP64 path at rtol 1e-13; the
    gradients under test come from the mixed-precision problem (and from FP64)."""
    import torch
    from topomax_gb300.autograd import compliance
    from topomax_gb300.fem import Function
    prob, V = _problem("mixed", 1e-10)
    g1 = torch.Generator().manual_seed(1)
    rho0 = (torch.rand(V.dim(), generator=g1, dtype=torch.float64) * 0.95 + 0.05).cuda()
    rho = rho0.clone().requires_grad_(True)
    c = compliance(prob, rho)
    c.backward()
    grad = rho.grad.cpu().numpy()

    prob64, _ = _problem("fp64", 1e-13)
    rho64 = rho0.clone().requires_grad_(True)
    c64 = compliance(prob64, rho64)
    c64.backward()
    g64 = rho64.grad.cpu().numpy()
    assert abs(float(c) - float(c64)) <= 1e-9 * abs(float(c64))
    assert np.max(np.abs(grad - g64)) <= 1e-6 * np.max(np.abs(g64))

    idx = torch.randperm(V.dim(), generator=torch.Generator().manual_seed(2))[:200].numpy()
    h = 1e-6
    fd = np.empty(len(idx))
    for n, i in enumerate(idx):
        vals = []
        for s in (+1.0, -1.0):
            r = rho0.clone()
            r[int(i)] += s * h
            vals.append(prob64.calculate_objective(Function(V, r)))
        fd[n] = (vals[0] - vals[1]) / (2 * h)
    assert np.all(np.isfinite(fd))
    assert np.linalg.norm(fd - grad[idx]) <= 1e-3 * np.linalg.norm(grad[idx])


def test_compliance_gradient_matches_the_oracles_analytic_sensitivity():
    """The same 400 x 200 workload against the FP64 oracle's analytic sensitivity (the
    reference's FEM_src/elasisity_problem.py:134-150 restated: the filtered -r'(xi)(...)
    Riesz representative g, times the CG1 mass matrix M1 for the Euclidean gradient),
    and the compliance against the oracle's sparse-LU value."""
    import torch
    from oracle.fem import Design, FEMOracle, Lattice
    from topomax_gb300.autograd import compliance
    prob, V = _problem("mixed", 1e-10)
    g1 = torch.Generator().manual_seed(1)
    rho0 = (torch.rand(V.dim(), generator=g1, dtype=torch.float64) * 0.95 + 0.05).cuda()
    rho = rho0.clone().requires_grad_(True)
    c = compliance(prob, rho)
    c.backward()
    grad = rho.grad.cpu().numpy()
    d = Design(width=2.0, height=1.0, fem_step_size=0.002, penalties=[3.0], volume_fraction=0.5,
               fixed_sides=["Left"], body_force=None,
               tractions=[dict(side="Right", center=0.5, length=0.2, value=[0.0, -1.0])],
               filter_radius=0.05, young_modulus=1.0, poisson_ratio=0.3)
    o = FEMOracle(Lattice(2.0, 1.0, 400, 200), d)
    o.set_penalization(3.0)
    r = rho0.cpu().numpy()
    xi = o.filter_apply(r)
    u = o.state_solve(xi)
    assert abs(float(c.detach()) - o.compliance(u)) <= 1e-9 * abs(o.compliance(u))
    ref = o.M1 @ o.gradient(u, xi)
    assert np.max(np.abs(grad - ref)) <= 1e-6 * np.max(np.abs(ref))
