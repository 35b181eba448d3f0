"""Entropic mirror descent design loop (the reference's src/solver.py:42-349, FEM_src/solver.py:15-89).

``FEMSolver(N, design_file).solve()`` runs the same loop as the reference --
step-size schedule, volume projection, stopping rules, penalty continuation,
per-iteration and result pickles -- with the design vectors psi, rho and the
gradient resident in HBM.  One device-to-host read per iteration (objective
and the design change) drives the stopping rules, as in the reference.
"""
from __future__ import annotations

import ctypes
import os
import pickle
import time
from abc import ABC, abstractmethod

import numpy as np
import torch

from . import _capi
from .designs import ElasticityParameters, FluidParameters, parse_design, parse_design_dict
from .fem import (DEFAULT_RTOL, ElasticityProblem, Function, FunctionSpace, RectangleMesh, _device, _ptr,
                  _stream, as_cg1_tensor, design_record)
from .utils import IterationData, SolverResult


def expit(x):
    return 1.0 / (1.0 + torch.exp(-x)) if isinstance(x, torch.Tensor) else 1.0 / (1.0 + np.exp(-x))


def expit_diff(x):
    e = expit(x)
    return e * (1 - e)


def logit(x):
    return torch.log(x / (1.0 - x)) if isinstance(x, torch.Tensor) else np.log(x / (1.0 - x))


class Solver(ABC):
    """EMD driver; subclasses supply the discretisation hooks (src/solver.py:80-128)."""

    def __init__(self, N: int, design_file, data_path="output", skip_multiple=1, verbose=True,
                 save=True):
        """design_file: a design JSON path as in the reference, or the parsed JSON dict itself
        (its optional top-level "name" names the output folder)."""
        self.full_N = N
        self.design_file = design_file
        if isinstance(design_file, dict):
            design_file = dict(design_file)
            self.design_str = str(design_file.pop("name", "design"))
            self._design_dict = design_file
        else:
            self.design_str = os.path.splitext(os.path.basename(design_file))[0]
            self._design_dict = None
        self.output_folder = f"{data_path}/{self.get_name()}/{self.design_str}/data"
        self.skip_multiple = skip_multiple
        self.verbose = verbose
        self.save = save
        if self._design_dict is not None:
            self.parameters, problem_parameters = parse_design_dict(self._design_dict)
        else:
            self.parameters, problem_parameters = parse_design(design_file)
        self.width = self.parameters.width
        self.height = self.parameters.height
        self.N = int(self.full_N / min(self.width, self.height))
        self.full_N = int(self.N * min(self.width, self.height))
        self.volume = self.width * self.height * self.parameters.volume_fraction
        self.step_size = self.get_step_size()
        self.prepare_domain()
        self.rho = self.create_rho(self.parameters.volume_fraction)
        self.problem = self.create_problem(problem_parameters)
        self.penalty_formatter = self.get_penalty_formatter(self.parameters.penalties)
        self.history: dict = {}

    @abstractmethod
    def get_name(self) -> str: ...

    @abstractmethod
    def get_step_size(self) -> float: ...

    @abstractmethod
    def prepare_domain(self) -> None: ...

    @abstractmethod
    def create_rho(self, volume_fraction: float): ...

    @abstractmethod
    def create_problem(self, problem_parameters): ...

    @abstractmethod
    def to_array(self, rho) -> np.ndarray: ...

    @abstractmethod
    def set_from_array(self, rho, values) -> None: ...

    @abstractmethod
    def integrate(self, values) -> float: ...

    @abstractmethod
    def save_rho(self, rho, file_root: str) -> str: ...

    def get_penalty_formatter(self, penalties):
        pads = np.array([[len(v) for v in str(p).split(".")] for p in penalties])
        left_pad, right_pad = np.max(pads[:, 0]), np.max(pads[:, 1])

        def penalty_formatter(penalty: float):
            left = len(str(penalty).split(".", maxsplit=1)[0])
            return f"{'0' * (left_pad - left)}{penalty:.{right_pad}f}"

        return penalty_formatter

    @staticmethod
    def tolerance(k: int):
        return min(25 * (k + 1) * 1e-5, 1e-2)

    def step_size_at_iter(self, k: int):
        if len(self.parameters.penalties) > 1:
            return self.step_size * min(k + 1, 10)
        return self.step_size * (k + 1)


class FEMSolver(Solver):
    """Structured-grid FEM design loop on the GPU (FEM_src/solver.py:15-89)."""

    def __init__(self, N: int, design_file, data_path: str = "output", skip_multiple: int = 1, *,
                 precision: str = "mixed", rtol: float = DEFAULT_RTOL, verbose: bool = True, save: bool = True,
                 max_iterations: int = 1000):
        self.precision = precision
        self.rtol = rtol
        self.max_iterations = max_iterations
        super().__init__(N, design_file, data_path, skip_multiple, verbose, save)

    def get_name(self):
        return "FEM"

    def get_step_size(self):
        return self.parameters.fem_step_size

    def prepare_domain(self):
        self.mesh = RectangleMesh(self.width, self.height, int(self.width * self.N), int(self.height * self.N))
        self.control_space = FunctionSpace(self.mesh, "CG", 1)

    def create_rho(self, volume_fraction: float):
        rho = Function(self.control_space)
        rho.tensor.fill_(volume_fraction)
        return rho

    def create_problem(self, problem_parameters):
        if isinstance(problem_parameters, ElasticityParameters):
            return ElasticityProblem(self.mesh, self.control_space, self.parameters, problem_parameters,
                                     precision=self.precision, rtol=self.rtol)
        if isinstance(problem_parameters, FluidParameters):
            from .fluid import FluidProblem
            return FluidProblem(self.mesh, problem_parameters, self.parameters, rtol=self.rtol)
        raise ValueError(f"Got unknown problem '{self.parameters.problem}'")

    def to_array(self, rho) -> np.ndarray:
        """The design's values in the control space's host dof order (dolfin's, as the
        reference's FEM_src/solver.py:75-76)."""
        return rho.vector()[:]

    def set_from_array(self, rho, values):
        rho.vector()[:] = values

    def integrate(self, values) -> float:
        t = as_cg1_tensor(values, self.control_space)
        out = torch.zeros(1, dtype=torch.float64, device=_device())
        ctx = self.problem._ctx
        ctx.check(ctx._lib.topo_integrate(ctx.ptr, _ptr(t), _ptr(out), _stream()))
        return float(out.item())

    def save_rho(self, rho, file_root: str):
        """FEM_src/solver.py:86-89: the design in the reference's pickle, dolfin's dof order."""
        rho_file = file_root + "_rho.dat"
        with open(rho_file, "wb") as f:
            pickle.dump(design_record(rho.tensor.cpu().numpy(), self.mesh), f)
        return os.path.basename(rho_file)

    # -- EMD ------------------------------------------------------------------
    def project(self, half_step, volume: float):
        """half_step + c with int expit(half_step + c) dx = volume (src/solver.py:149-186).

        A numpy array (in the control space's host dof order) gives a numpy array in the
        same order, as the reference's; a tensor or Function gives a lattice-order tensor."""
        h = as_cg1_tensor(half_step, self.control_space)
        zero = torch.zeros_like(h)
        psi = self._emd(h, zero, 0.0, volume)
        if isinstance(half_step, (torch.Tensor, Function)):
            return psi
        return self.control_space.to_host_order(psi.cpu().numpy())

    def _emd(self, psi_prev: torch.Tensor, g: torch.Tensor, alpha: float, volume: float) -> torch.Tensor:
        psi = torch.empty_like(psi_prev)
        c = ctypes.c_double(0.0)
        ctx = self.problem._ctx
        ctx.check(ctx._lib.topo_emd_step(ctx.ptr, _ptr(psi_prev), _ptr(g), float(alpha), float(volume), _ptr(psi),
                                         ctypes.byref(c), _stream()))
        self.last_multiplier = c.value
        return psi

    def step(self, previous_psi: torch.Tensor, step_size: float) -> torch.Tensor:
        """Entropic mirror descent step with volume correction (src/solver.py:188-194)."""
        g = self.problem.calculate_objective_gradient()
        return self._emd(previous_psi, g.tensor, step_size, self.volume)

    def _finish(self, psi: torch.Tensor, previous_psi: torch.Tensor | None) -> float:
        ctx = self.problem._ctx
        d = ctypes.c_double(0.0)
        ctx.check(ctx._lib.topo_emd_finish(ctx.ptr, _ptr(psi), _ptr(previous_psi) if previous_psi is not None else None,
                                           _ptr(self.rho.tensor), ctypes.byref(d), _stream()))
        return d.value

    def solve(self):
        """Solve the topology optimisation problem (src/solver.py:208-302)."""
        t_total = time.perf_counter()
        psi = logit(self.rho.tensor.clone())
        for penalty in self.parameters.penalties:
            self.problem.set_penalization(penalty)
            t_step = time.perf_counter()
            objectives = [self.problem.calculate_objective(self.rho)]
            times = [time.perf_counter() - t_step]
            deltas = []
            if self.verbose:
                print(f"penalty {penalty}: k=0 objective={objectives[0]:.6g}")
            k = 0
            exit_condition = ""
            for k in range(self.max_iterations):
                if self.save and k % self.skip_multiple == 0:
                    self.save_iteration(self.rho, objectives[-1], k, penalty)
                t_step = time.perf_counter()
                previous_psi = psi.clone()
                try:
                    psi = self.step(previous_psi, self.step_size_at_iter(k))
                except ValueError as e:
                    exit_condition = str(e)
                    if self.verbose:
                        print(f"EXIT: {exit_condition}!")
                    break
                difference = self._finish(psi, previous_psi)
                objectives.append(self.problem.calculate_objective(self.rho))
                times.append(time.perf_counter() - t_step)
                deltas.append(difference)
                if self.verbose:
                    print(f"k={k + 1} objective={objectives[-1]:.10g} delta_rho={difference:.3e} "
                          f"tol={self.tolerance(k):.1e} time={times[-1] * 1e3:.1f}ms")
                if np.isnan(objectives[-1]):
                    exit_condition = "Objective is NaN"
                    break
                min_index = int(np.argmin(objectives))
                if objectives[-1] > 2 * objectives[min_index]:
                    exit_condition = "Objective is increasing"
                    break
                if k >= min_index + 50:
                    exit_condition = "Objective is not decreasing"
                    break
                if difference < self.tolerance(k):
                    exit_condition = "Convergence treshold reached"
                    break
            else:
                exit_condition = "Iteration did not converge"
            if self.verbose:
                print(f"EXIT: {exit_condition}")
            self.history[penalty] = dict(objectives=objectives, times=times, deltas=deltas,
                                         exit_condition=exit_condition, iterations=k + 1)
            if self.save:
                self.save_iteration(self.rho, objectives[-1], k + 1, penalty)
                self.save_result(objectives, times, penalty, exit_condition)
        if self.verbose:
            print(f"design loop: {time.perf_counter() - t_total:.3f} s")
        return self.history

    def save_iteration(self, rho, objective: float, k: int, penalty: float):
        file_root = f"{self.output_folder}/N={self.full_N}_p={self.penalty_formatter(penalty)}_{k=}"
        os.makedirs(os.path.dirname(file_root), exist_ok=True)
        rho_basename = self.save_rho(rho, file_root)
        data = IterationData((self.width, self.height), objective, k, rho_basename, penalty)
        with open(f"{file_root}.dat", "wb") as f:
            pickle.dump(data, f)

    def save_result(self, objectives, times, penalty: float, exit_condition: str):
        file_root = f"{self.output_folder}/N={self.full_N}_p={self.penalty_formatter(penalty)}_result"
        min_index = int(np.argmin(objectives))
        data = SolverResult(exit_condition, objectives[min_index], objectives, len(objectives), min_index, times)
        with open(f"{file_root}.dat", "wb") as f:
            pickle.dump(data, f)
