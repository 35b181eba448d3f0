"""topomax_gb300: the topomax FEM design loops on one GB300 (sm_103a).

Reference-facing classes (same names and call surface as Emilinya/topomax):
``ElasticityProblem``, ``FluidProblem``, ``HelmholtzFilter``, ``FEMSolver``/``Solver``,
``parse_design``.  The arithmetic runs in hand-written CUDA kernels behind the
C ABI of ``include/topomax_gb300.h`` (``libtopomax_gb300.so``, built by
``topomax_gb300.build``).
"""
from .designs import (DomainParameters, ElasticityParameters, FluidParameters, Flow, Force, CircularRegion, Side,
                      Traction, parse_design, parse_design_dict)
from .penalizers import ElasticPenalizer, FluidPenalizer
from .problem import Problem

__all__ = [
    "DomainParameters", "ElasticityParameters", "FluidParameters", "Flow", "Force", "CircularRegion", "Side",
    "Traction", "parse_design",
    "parse_design_dict", "ElasticPenalizer", "FluidPenalizer", "Problem", "ElasticityProblem", "FluidProblem",
    "HelmholtzFilter", "FEMSolver", "Solver", "RectangleMesh", "FunctionSpace", "VectorFunctionSpace", "Function",
]


def __getattr__(name):
    # the device-backed classes import torch and load the C-ABI library lazily
    if name in ("ElasticityProblem", "HelmholtzFilter", "RectangleMesh", "FunctionSpace", "VectorFunctionSpace",
                "Function"):
        from . import fem
        return getattr(fem, name)
    if name == "FluidProblem":
        from . import fluid
        return fluid.FluidProblem
    if name in ("FEMSolver", "Solver"):
        from . import solver
        return getattr(solver, name)
    raise AttributeError(name)
