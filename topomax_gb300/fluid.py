"""Stokes-Brinkman fluid problem with the reference's call surface (FEM_src/fluid_problem.py:48-155).

``FluidProblem(mesh, fluid_parameters, domain_parameters)`` offers the reference's
``set_penalization``, ``calculate_objective``, ``calculate_objective_gradient`` and
``forward``; ``FEMSolver`` runs the design loop on it exactly as on the elasticity
problem.  The state (Taylor-Hood: vector P2 velocity, P1 pressure), the objective and
the CG1-projected gradient run in ``libtopomax_gb300.so`` in FP64.  The pressure comes
back with zero sum: the state system is singular in the pressure constant and, with the
interpolated flow profiles, slightly inconsistent; the continuity right-hand side is
projected to zero sum (the reduced system's least-squares closure).
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _capi
from .designs import DomainParameters, FluidParameters, Side
from .fem import (DEFAULT_RTOL, Function, FunctionSpace, RectangleMesh, VectorFunctionSpace, _Context, _device,
                  _grid, _ptr, _stream, as_cg1_tensor)
from .penalizers import FluidPenalizer
from .problem import Problem


class _FluidContext:
    """Owns a topo_fluid_ctx."""

    def __init__(self, ptr):
        self.ptr = ptr
        self._lib = _capi.load_library()

    def __del__(self):
        if getattr(self, "ptr", None):
            self._lib.topo_fluid_destroy(self.ptr)
            self.ptr = None

    def check(self, rc):
        if rc == _capi.TOPO_OK:
            return
        msg = self._lib.topo_fluid_last_error(self.ptr).decode()
        if rc == _capi.TOPO_ERR_CUDA:
            raise RuntimeError(f"topomax_gb300 CUDA error: {msg}")
        raise _capi.TopoError(rc, msg or f"topomax_gb300 error {rc}")


class FluidProblem(Problem):
    """Borrvall-Petersson Stokes-Brinkman flow (FEM_src/fluid_problem.py:48-155).

    Keyword-only extras: ``rtol`` (relative residual of the state solve and of the
    projection's mass-matrix solve).
    """

    def __init__(self, mesh: RectangleMesh, fluid_parameters: FluidParameters, domain_parameters: DomainParameters,
                 *, rtol: float = DEFAULT_RTOL):
        super().__init__()
        self.parameters = fluid_parameters
        self.domain_size = (domain_parameters.width, domain_parameters.height)
        if abs(mesh.width - self.domain_size[0]) > 1e-12 or abs(mesh.height - self.domain_size[1]) > 1e-12:
            raise ValueError("mesh does not span the design domain")
        self.mesh = mesh
        self.control_space = FunctionSpace(mesh, "CG", 1)
        self.solution_space = VectorFunctionSpace(mesh, "CG", 2)
        self.viscosity = self.parameters.viscosity
        self.penalizer = FluidPenalizer()
        self.rtol = float(rtol)
        self.u: Function | None = None
        self.p: Function | None = None
        self.rho: torch.Tensor | None = None
        self.stats = {"state_iterations": 0, "projection_iterations": 0}
        self._fctx = self._create_context()
        # the design loop's CG1 operations (integrate, EMD step and projection) run on a
        # design-space context: the filter of radius zero, i.e. the CG1 mass matrix
        lib = _capi.load_library()
        st = ctypes.c_int(0)
        ptr = lib.topo_create_filter(ctypes.byref(_grid(mesh)), 0.0, _capi.PREC_FP64, ctypes.byref(st))
        if not ptr:
            raise _capi.TopoError(st.value, f"could not create the design-space context (status {st.value})")
        self._ctx = _Context(ptr)
        self._scalar = torch.zeros(1, dtype=torch.float64, device=_device())

    def _create_context(self) -> _FluidContext:
        lib = _capi.load_library()
        _device()
        flows = self.parameters.flows
        arr = (_capi.Flow * max(1, len(flows)))()
        for k, f in enumerate(flows):
            side = f["side"] if isinstance(f, dict) else f.side
            center = f["center"] if isinstance(f, dict) else f.center
            length = f["length"] if isinstance(f, dict) else f.length
            rate = f["rate"] if isinstance(f, dict) else f.rate
            s = side if isinstance(side, Side) else Side.from_string(side)
            arr[k] = _capi.Flow(s.mask, float(center), float(length), float(rate))
        st = ctypes.c_int(0)
        ptr = lib.topo_fluid_create(ctypes.byref(_grid(self.mesh)), float(self.viscosity), arr, len(flows),
                                    ctypes.byref(st))
        if not ptr:
            raise _capi.TopoError(st.value, f"could not create the fluid problem (status {st.value})")
        return _FluidContext(ptr)

    # -- Problem interface -----------------------------------------------------
    def set_penalization(self, penalization: float):
        self.penalizer.set_penalization(penalization)
        self._fctx.check(self._fctx._lib.topo_fluid_set_penalization(self._fctx.ptr, float(penalization)))

    def calculate_objective_gradient(self) -> Function:
        """phi'(rho) = 1/2 alpha'(rho) |u|^2, L2-projected onto CG1."""
        if self.rho is None or self.u is None:
            raise ValueError("You must call calculate_objective before calling calculate_objective_gradient")
        self.penalizer.assert_has_penalization()
        g = Function(self.control_space)
        it = ctypes.c_int(0)
        self._fctx.check(self._fctx._lib.topo_fluid_gradient(self._fctx.ptr, _ptr(self.rho), _ptr(self.u.tensor),
                                                             _ptr(g.tensor), self.rtol, ctypes.byref(it),
                                                             _stream()))
        self.stats["projection_iterations"] += it.value
        return g

    def calculate_objective(self, rho) -> float:
        """phi(rho) = 1/2 int alpha(rho) |u|^2 + mu |grad u|^2 dx."""
        self.rho = as_cg1_tensor(rho, self.control_space).clone()
        self.u, self.p = self.forward(self.rho)
        self._fctx.check(self._fctx._lib.topo_fluid_objective(self._fctx.ptr, _ptr(self.rho), _ptr(self.u.tensor),
                                                              _ptr(self._scalar), _stream()))
        return float(self._scalar.item())

    def forward(self, rho):
        """(velocity, pressure) of the state equation for the design rho."""
        self.penalizer.assert_has_penalization()
        r = as_cg1_tensor(rho, self.control_space)
        u = Function(self.solution_space)
        p = Function(self.control_space)
        it = ctypes.c_int(0)
        self._fctx.check(self._fctx._lib.topo_fluid_state_solve(self._fctx.ptr, _ptr(r), _ptr(u.tensor),
                                                                _ptr(p.tensor), self.rtol, ctypes.byref(it),
                                                                _stream()))
        self.stats["state_iterations"] += it.value
        return u, p

    # -- extras -------------------------------------------------------------------
    def apply_operator(self, rho, x: torch.Tensor, clamp: bool = False) -> torch.Tensor:
        """y = A(rho) x for x = [velocity (2 n2) | pressure (n_vertices)], continuity rows negated."""
        y = torch.empty_like(x)
        r = as_cg1_tensor(rho, self.control_space)
        self._fctx.check(self._fctx._lib.topo_fluid_apply(self._fctx.ptr, _ptr(r), _ptr(x), _ptr(y), int(clamp),
                                                          _stream()))
        return y

    def boundary_values(self) -> torch.Tensor:
        u = torch.empty(self.solution_space.dim(), dtype=torch.float64, device=_device())
        self._fctx.check(self._fctx._lib.topo_fluid_boundary_values(self._fctx.ptr, _ptr(u), _stream()))
        return u

    def gradient_rhs(self, rho, u: Function) -> torch.Tensor:
        b = torch.empty(self.control_space.dim(), dtype=torch.float64, device=_device())
        r = as_cg1_tensor(rho, self.control_space)
        self._fctx.check(self._fctx._lib.topo_fluid_gradient_rhs(self._fctx.ptr, _ptr(r), _ptr(u.tensor), _ptr(b),
                                                                 _stream()))
        return b

    def launch_count(self) -> int:
        n = ctypes.c_int64(0)
        self._fctx.check(self._fctx._lib.topo_fluid_launch_count(self._fctx.ptr, ctypes.byref(n)))
        m = ctypes.c_int64(0)
        self._ctx.check(self._ctx._lib.topo_launch_count(self._ctx.ptr, ctypes.byref(m)))
        return int(n.value + m.value)
