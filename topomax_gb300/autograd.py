"""The compliance as a differentiable torch function of the nodal design.

``compliance(problem, rho)`` returns C(rho) = f.u with u = K(xi(rho))^-1 f and
xi = the Helmholtz-filtered rho (``ElasticityProblem.calculate_objective``,
FEM_src/elasisity_problem.py:152-166).  Its backward returns the Euclidean
gradient dC/d rho = M1 g, where g is the CG1 Riesz representative the
reference's ``calculate_objective_gradient`` returns (FEM_src/elasisity_problem.py:
134-150) and M1 the consistent CG1 mass matrix: with A_f = eps^2 K1 + M1 and
xi = A_f^-1 M1 rho, dC/d rho = M1 A_f^-1 b = M1 g (A_f symmetric).
"""
from __future__ import annotations

import torch

from .fem import ElasticityProblem, Function


class _Compliance(torch.autograd.Function):
    @staticmethod
    def forward(ctx, rho: torch.Tensor, problem: ElasticityProblem):
        values = rho.detach().to(device="cuda", dtype=torch.float64).contiguous()
        c = problem.calculate_objective(Function(problem.control_space, values))
        ctx.problem = problem
        return torch.tensor(c, dtype=torch.float64, device=rho.device)

    @staticmethod
    def backward(ctx, grad):
        problem = ctx.problem
        g = problem.calculate_objective_gradient()
        euclid = problem.filter.mass_apply(g)
        return grad.to(euclid.device) * euclid, None


def compliance(problem: ElasticityProblem, rho: torch.Tensor) -> torch.Tensor:
    """C(rho) with torch autograd reaching rho (1-D, lattice order, V1 entries)."""
    return _Compliance.apply(rho, problem)
