"""Device-resident FEM objects with the reference's call surface.

Mirrors the pieces of FEniCS the reference's elasticity path touches:

* ``RectangleMesh`` -- the structured triangulation of FEM_src/solver.py:38-49
  (dolfin's "right" diagonal);
* ``FunctionSpace`` / ``Function`` -- CG1 design fields on the vertex lattice
  and vector-P2 displacements on the half-spacing node lattice, held in HBM
  as FP64 torch tensors (``.vector()[:]`` reads/writes like dolfin's);
* ``HelmholtzFilter`` -- FEM_src/filter.py:11-41;
* ``ElasticityProblem`` -- FEM_src/elasisity_problem.py:76-196.

All arithmetic runs in ``libtopomax_gb300.so`` on the GPU; this module only
marshals arguments.

Vector ordering.  On the device (``Function.tensor``, torch tensors passed
in): CG1 vertex (i, j) at j*(nx+1)+i, P2 node (a, b) at b*(2nx+1)+a with
components interleaved.  On the host side of a CG1 space -- ``.vector()``
views and numpy arrays or lists passed to the problem and filter methods --
the space's ``dof_order``: "dolfin" (the default) is the numbering the
reference's serial dolfin gives the CG1 dofs of its RectangleMesh, so arrays
from the reference (``to_array``, saved designs) are read as the reference
reads them; "lattice" is the device order.
"""
from __future__ import annotations

import ctypes
import os
import pickle

import numpy as np
import torch

from . import _capi
from .designs import DomainParameters, ElasticityParameters, Side
from .penalizers import ElasticPenalizer
from .problem import Problem

DEFAULT_RTOL = 1e-10
PRECISIONS = {"fp64": _capi.PREC_FP64, "mixed": _capi.PREC_MIXED}


def _device():
    if not torch.cuda.is_available():
        raise RuntimeError("topomax_gb300 needs a CUDA device (there is no CPU path)")
    return torch.device("cuda", torch.cuda.current_device())


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _ptr(t: torch.Tensor):
    return ctypes.c_void_p(t.data_ptr())


class RectangleMesh:
    """[0, width] x [0, height] split into nx x ny squares, two triangles each."""

    def __init__(self, width: float, height: float, nx: int, ny: int):
        if nx < 1 or ny < 1:
            raise ValueError("RectangleMesh needs at least one cell per direction")
        self.width = float(width)
        self.height = float(height)
        self.nx = int(nx)
        self.ny = int(ny)

    @property
    def hx(self):
        return self.width / self.nx

    @property
    def hy(self):
        return self.height / self.ny

    def num_vertices(self):
        return (self.nx + 1) * (self.ny + 1)

    def num_cells(self):
        return 2 * self.nx * self.ny

    def coordinates(self) -> np.ndarray:
        """(n_vertices, 2) vertex coordinates in lattice order (x_i = i * (W / nx))."""
        x = np.array([0.0 + i * (self.width / self.nx) for i in range(self.nx + 1)])
        y = np.array([0.0 + j * (self.height / self.ny) for j in range(self.ny + 1)])
        X, Y = np.meshgrid(x, y)
        return np.stack([X.ravel(), Y.ravel()], axis=1)

    def hmin(self):
        return float(np.hypot(self.hx, self.hy))


class FunctionSpace:
    """CG1 scalar space (degree 1) or vector CG2 space (``vector=True``, degree 2).

    ``dof_order`` (CG1 only) is the order of the space's host-side arrays: "dolfin"
    (default; the reference's CG1 dof numbering, FEM_src/solver.py:75-79 hands such
    arrays to the design loop) or "lattice" (the device order).  The vector CG2 space
    is always in lattice order."""

    def __init__(self, mesh: RectangleMesh, family: str = "CG", degree: int = 1, vector: bool = False,
                 dof_order: str = "dolfin"):
        if family not in ("CG", "Lagrange", "P"):
            raise ValueError(f"unsupported family {family}")
        if (degree, vector) not in ((1, False), (2, True)):
            raise ValueError("supported spaces: scalar CG1 and vector CG2")
        if dof_order not in ("dolfin", "lattice"):
            raise ValueError(f"dof_order must be 'dolfin' or 'lattice', got {dof_order!r}")
        self._mesh = mesh
        self.degree = degree
        self.vector = vector
        self.dof_order = "lattice" if vector else dof_order
        self._perm = None

    def dolfin_permutation(self):
        """Lattice index of each host-side dof (None when the host order is the lattice)."""
        if self.dof_order == "lattice":
            return None
        if self._perm is None:
            self._perm = dolfin_cg1_order(self._mesh.nx, self._mesh.ny)
        return self._perm

    def to_host_order(self, lattice_values: np.ndarray) -> np.ndarray:
        perm = self.dolfin_permutation()
        return lattice_values if perm is None else lattice_values[perm]

    def from_host_order(self, values: np.ndarray) -> np.ndarray:
        perm = self.dolfin_permutation()
        if perm is None:
            return values
        out = np.empty_like(values)
        out[perm] = values
        return out

    def mesh(self):
        return self._mesh

    def dim(self) -> int:
        m = self._mesh
        if self.vector:
            return 2 * (2 * m.nx + 1) * (2 * m.ny + 1)
        return m.num_vertices()


def VectorFunctionSpace(mesh: RectangleMesh, family: str = "CG", degree: int = 2):
    return FunctionSpace(mesh, family, degree, vector=True)


class _VectorView:
    """``Function.vector()``: the coefficients in the space's host-side dof order."""

    def __init__(self, f: "Function"):
        self._f = f

    def __len__(self):
        return self._f.tensor.numel()

    def __getitem__(self, idx):
        return self._f._V.to_host_order(self._f.tensor.detach().cpu().numpy())[idx]

    def __setitem__(self, idx, value):
        V, t = self._f._V, self._f.tensor
        if V.dolfin_permutation() is None:
            if isinstance(value, torch.Tensor):
                t[idx] = value.to(t)
            else:
                v = np.asarray(value, dtype=np.float64)
                t[idx] = torch.as_tensor(v, device=t.device) if v.ndim else float(v)
            return
        host = self[:]
        host[idx] = value.detach().cpu().numpy() if isinstance(value, torch.Tensor) else value
        t.copy_(torch.as_tensor(V.from_host_order(host), device=t.device))

    def get_local(self):
        return self[:]


class Function:
    """A finite-element function whose coefficient vector lives in HBM (FP64)."""

    def __init__(self, V: FunctionSpace, tensor: torch.Tensor | None = None):
        self._V = V
        if tensor is None:
            tensor = torch.zeros(V.dim(), dtype=torch.float64, device=_device())
        if tensor.numel() != V.dim() or tensor.dtype != torch.float64 or not tensor.is_cuda:
            raise ValueError("Function needs a contiguous FP64 CUDA tensor of the space's dimension")
        self.tensor = tensor.contiguous()

    def function_space(self):
        return self._V

    def vector(self):
        return _VectorView(self)

    def copy(self):
        return Function(self._V, self.tensor.clone())


def dolfin_cg1_order(nx: int, ny: int) -> np.ndarray:
    """Lattice index of every CG1 dof in the order the reference's (serial) dolfin numbers
    them on its RectangleMesh with the "right" diagonal: a level structure grown from the
    top-left vertex -- vertex (i, j) on level i + (ny - j) -- with x increasing inside a
    level.  It reproduces the design vectors the reference saves
    (tests/test_data/FEM/{triangle,diffuser}/data/correct_rho.dat, 1 x 1 at N = 10 and 20);
    on other rectangles the same two corners are the mesh graph's only pair at maximal
    distance, and the same rule is assumed."""
    I, J = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1))
    I, J = I.ravel(), J.ravel()
    return (J * (nx + 1) + I)[np.lexsort((I, I + (ny - J)))]


def to_dolfin_order(values, nx: int, ny: int) -> np.ndarray:
    """CG1 values in lattice order -> dolfin's dof order."""
    return np.asarray(values)[dolfin_cg1_order(nx, ny)]


def from_dolfin_order(values, nx: int, ny: int) -> np.ndarray:
    """CG1 values in dolfin's dof order -> lattice order."""
    v = np.asarray(values)
    out = np.empty_like(v)
    out[dolfin_cg1_order(nx, ny)] = v
    return out


def mesh_to_N(mesh: RectangleMesh) -> int:
    """Cells per unit length (FEM_src/utils.py:29-37: 1 / (hmin / sqrt 2))."""
    N = 1 / (mesh.hmin() / np.sqrt(2))
    if abs(N - int(round(N))) / N > 1e-10:
        print(f"save_function: got non-integer N: {N}, this could result in wrong data getting saved")
    return int(round(N))


def mesh_to_domain_size(mesh: RectangleMesh) -> tuple:
    """Largest vertex coordinates (FEM_src/utils.py:40-44), as the mesh computes them."""
    return (0.0 + mesh.nx * (mesh.width / mesh.nx), 0.0 + mesh.ny * (mesh.height / mesh.ny))


def design_record(values, mesh: RectangleMesh, N: int | None = None, domain_size=None) -> dict:
    """The pickled record of a CG1 design (FEM_src/utils.py:47-69 ``save_function``) from
    lattice-order values: N, domain size, problem "design" and the vector in dolfin's dof order."""
    return {"N": mesh_to_N(mesh) if N is None else N,
            "domain_size": mesh_to_domain_size(mesh) if domain_size is None else domain_size,
            "problem": "design", "vector": to_dolfin_order(values, mesh.nx, mesh.ny)}


def save_function(f: "Function", filename: str, problem: str = "design", N: int | None = None,
                  domain_size=None):
    """``save_function`` (FEM_src/utils.py:47-69) for CG1 designs: the reference's pickle,
    the vector in dolfin's dof order, readable by the reference's ``load_function``."""
    V = f.function_space()
    if V.vector or V.degree != 1 or problem != "design":
        raise ValueError("save_function writes CG1 designs (problem 'design')")
    with open(filename, "wb") as datafile:
        pickle.dump(design_record(f.tensor.cpu().numpy(), V.mesh(), N, domain_size), datafile)


def load_function(filename: str, mesh: RectangleMesh | None = None, function_space: FunctionSpace | None = None):
    """``load_function`` (FEM_src/utils.py:72-109) for design files -- the reference's own
    or this package's: returns (Function, mesh, function space)."""
    with open(filename, "rb") as datafile:
        data = pickle.load(datafile)
    if data["problem"] != "design":
        raise ValueError(f"load_function reads CG1 designs; got problem '{data['problem']}'")
    if mesh is None:
        w, h = data["domain_size"]
        mesh = RectangleMesh(w, h, int(w * data["N"]), int(h * data["N"]))
    if function_space is None:
        function_space = FunctionSpace(mesh, "CG", 1)
    m = function_space.mesh()
    values = np.asarray(data["vector"], dtype=np.float64)
    if values.size != function_space.dim():
        raise ValueError(f"design vector of {values.size} values does not fit {function_space.dim()} vertices")
    f = Function(function_space, torch.as_tensor(from_dolfin_order(values, m.nx, m.ny)).to(_device()))
    return f, mesh, function_space


def as_cg1_tensor(value, V: FunctionSpace) -> torch.Tensor:
    """CG1 coefficients in device (lattice) order of a Function, a torch tensor (taken to be
    in lattice order) or a numpy array / list (in the space's host-side dof order), copied
    to HBM where needed."""
    if isinstance(value, Function):
        return value.tensor
    if isinstance(value, torch.Tensor):
        t = value.to(device=_device(), dtype=torch.float64).contiguous()
    else:
        v = np.ascontiguousarray(value, dtype=np.float64).reshape(-1)
        if v.size == V.dim():
            v = np.ascontiguousarray(V.from_host_order(v))
        t = torch.as_tensor(v).to(_device())
    if t.numel() != V.dim():
        raise ValueError(f"expected {V.dim()} CG1 values, got {t.numel()}")
    return t.reshape(-1)


class _Context:
    """Owns a topo_ctx."""

    def __init__(self, ptr):
        self.ptr = ptr
        self._lib = _capi.load_library()

    def __del__(self):
        # topo_destroy frees with cudaFree, which waits for the device's pending work
        if getattr(self, "ptr", None):
            self._lib.topo_destroy(self.ptr)
            self.ptr = None

    def check(self, rc):
        _capi.check(rc, self.ptr)


def _grid(mesh: RectangleMesh) -> _capi.GridDesc:
    return _capi.GridDesc(mesh.width, mesh.height, mesh.nx, mesh.ny)


class HelmholtzFilter:
    """-eps^2 Lap(xi) + xi = rho with natural boundary conditions (FEM_src/filter.py:11-41).

    ``apply(f)`` accepts a CG1 ``Function`` (or CG1 coefficients) and returns
    the filtered CG1 ``Function``.  The operator is set up once, as the
    reference pre-assembles it.
    """

    def __init__(self, epsilon: float, function_space: FunctionSpace, *, precision: str = "mixed",
                 rtol: float = DEFAULT_RTOL, _ctx: _Context | None = None):
        if function_space.vector or function_space.degree != 1:
            raise ValueError("HelmholtzFilter acts on the CG1 design space")
        self.epsilon = float(epsilon)
        self.function_space = function_space
        self.rtol = float(rtol)
        self.last_iterations = 0
        if _ctx is None:
            lib = _capi.load_library()
            _device()
            st = ctypes.c_int(0)
            ptr = lib.topo_create_filter(ctypes.byref(_grid(function_space.mesh())), self.epsilon,
                                         PRECISIONS[precision], ctypes.byref(st))
            if not ptr:
                raise _capi.TopoError(st.value, f"could not create the filter (status {st.value})")
            _ctx = _Context(ptr)
        self._ctx = _ctx

    def mass_apply(self, values) -> torch.Tensor:
        """M1 x: the consistent CG1 mass matrix times nodal values (FP64, lattice order)."""
        x = as_cg1_tensor(values, self.function_space)
        y = torch.empty_like(x)
        self._ctx.check(self._ctx._lib.topo_mass_apply(self._ctx.ptr, _ptr(x), _ptr(y), _stream()))
        return y

    def apply(self, input_function) -> Function:
        f = as_cg1_tensor(input_function, self.function_space)
        out = Function(self.function_space)
        it = ctypes.c_int(0)
        self._ctx.check(self._ctx._lib.topo_filter_apply(self._ctx.ptr, _ptr(f), _ptr(out.tensor), self.rtol,
                                                         ctypes.byref(it), _stream()))
        self.last_iterations = it.value
        return out

    def solve_rhs(self, rhs: torch.Tensor) -> Function:
        """Filter of an already assembled CG1 right-hand side (integral against phi_i)."""
        out = Function(self.function_space)
        it = ctypes.c_int(0)
        self._ctx.check(self._ctx._lib.topo_filter_solve(self._ctx.ptr, _ptr(rhs), _ptr(out.tensor), self.rtol,
                                                         ctypes.byref(it), _stream()))
        self.last_iterations = it.value
        return out


class ElasticityProblem(Problem):
    """Elastic compliance topology optimisation problem (FEM_src/elasisity_problem.py:76-196).

    Same constructor and methods as the reference.  Keyword-only extras:
    ``precision`` ("mixed": FP32 multigrid CG inside FP64 refinement, or
    "fp64"), ``rtol`` (relative residual of every linear solve) and
    ``warm_start`` (start the state solve from the previous displacement, and the
    design and sensitivity filter solves from their previous solutions).
    """

    def __init__(self, mesh: RectangleMesh, control_space: FunctionSpace, domain_parameters: DomainParameters,
                 elasticity_parameters: ElasticityParameters, *, precision: str = "mixed",
                 rtol: float = DEFAULT_RTOL, warm_start: bool = True):
        super().__init__()
        self.parameters = elasticity_parameters
        self.domain_size = (domain_parameters.width, domain_parameters.height)
        if abs(mesh.width - self.domain_size[0]) > 1e-12 or abs(mesh.height - self.domain_size[1]) > 1e-12:
            raise ValueError("mesh does not span the design domain")
        self.mesh = mesh
        self.control_space = control_space
        self.solution_space = VectorFunctionSpace(mesh, "CG", 2)
        self.precision = precision
        self.rtol = float(rtol)
        self.warm_start = warm_start
        self._ctx = self._create_context()
        self._ctx.check(self._ctx._lib.topo_set_filter_warm_start(self._ctx.ptr, int(bool(warm_start))))
        self.filter = HelmholtzFilter(self.parameters.filter_radius, control_space, rtol=self.rtol,
                                      _ctx=self._ctx)
        self.Young_modulus = self.parameters.young_modulus
        self.Poisson_ratio = self.parameters.poisson_ratio
        self.penalizer = ElasticPenalizer()
        self.lamé_mu = self.Young_modulus / (2 * (1 + self.Poisson_ratio))
        self.lamé_lda = self.lamé_mu * self.Poisson_ratio / (0.5 - self.Poisson_ratio)
        self.u: Function | None = None
        # the state's solution history, newest first (warm-start extrapolation)
        self._u_hist: list = []
        # warm-start guess from the last solutions: 0 the last one, else the polynomial
        # extrapolation of that order (1 linear .. 4) over the design iterations
        # (TOPO_EXTRAPOLATE; the default is 3, cubic)
        self.extrapolate_order = max(0, min(4, int(os.environ.get("TOPO_EXTRAPOLATE", "3"))))
        self.extrapolate = self.extrapolate_order > 0
        self.filtered_rho: Function | None = None
        self.stats = {"state_iterations": 0, "filter_iterations": 0}
        self._scalar = torch.zeros(1, dtype=torch.float64, device=_device())

    # -- set-up -------------------------------------------------------------
    def _create_context(self) -> _Context:
        lib = _capi.load_library()
        _device()
        p = self.parameters
        mat = _capi.Material(p.young_modulus, p.poisson_ratio, p.filter_radius, 1e-6)
        mask = 0
        for s in p.fixed_sides:
            mask |= (s if isinstance(s, Side) else Side.from_string(s)).mask
        pts = np.array([c for xy in (p.fixed_points or []) for c in xy], dtype=np.float64)
        bc = _capi.BCDesc(mask, len(pts) // 2,
                          pts.ctypes.data_as(ctypes.POINTER(ctypes.c_double)) if len(pts) else None)
        trs = p.tractions or []
        tarr = (_capi.Traction * max(1, len(trs)))()
        for k, t in enumerate(trs):
            tarr[k] = _capi.Traction(t.side.mask, t.center, t.length, t.value[0], t.value[1])
        if p.body_force is not None:
            bf = p.body_force
            load = _capi.LoadDesc(1, bf.region.center[0], bf.region.center[1], bf.region.radius, bf.value[0],
                                  bf.value[1], len(trs), tarr)
        else:
            load = _capi.LoadDesc(0, 0.0, 0.0, 0.0, 0.0, 0.0, len(trs), tarr)
        st = ctypes.c_int(0)
        ptr = lib.topo_create(ctypes.byref(_grid(self.mesh)), ctypes.byref(mat), ctypes.byref(bc),
                              ctypes.byref(load), PRECISIONS[self.precision], ctypes.byref(st))
        if not ptr:
            raise _capi.TopoError(st.value, f"could not create the elasticity problem (status {st.value})")
        return _Context(ptr)

    def set_iteration_limit(self, max_iterations: int = 0):
        """Cap the Krylov iterations of every filter and state solve of this problem (0: the
        defaults).  A solve that reaches the cap without meeting rtol raises ValueError
        (``TopoError`` with code TOPO_ERR_NOT_CONVERGED)."""
        self._ctx.check(self._ctx._lib.topo_set_iteration_limit(self._ctx.ptr, int(max_iterations)))

    # -- Problem interface -------------------------------------------------
    def set_penalization(self, penalization: float):
        self.penalizer.set_penalization(penalization)
        self._ctx.check(self._ctx._lib.topo_set_penalization(self._ctx.ptr, float(penalization)))

    def calculate_objective_gradient(self) -> Function:
        """Filter of -r'(xi)(lambda |div u|^2 + 2 mu |eps(u)|^2) (CG1 Riesz representative)."""
        if self.filtered_rho is None or self.u is None:
            raise ValueError("You must call calculate_objective before calling calculate_objective_gradient")
        self.penalizer.assert_has_penalization()
        g = Function(self.control_space)
        it = ctypes.c_int(0)
        self._ctx.check(self._ctx._lib.topo_sensitivity(self._ctx.ptr, _ptr(self.u.tensor),
                                                        _ptr(self.filtered_rho.tensor), _ptr(g.tensor), self.rtol,
                                                        ctypes.byref(it), _stream()))
        self.stats["filter_iterations"] += it.value
        return g

    def calculate_objective(self, rho) -> float:
        """phi(rho) = int u.f dx + int u.t ds with u the state of the filtered rho."""
        try:
            self.filtered_rho = self.filter.apply(rho)
            self.stats["filter_iterations"] += self.filter.last_iterations
            self.u = self.forward(self.filtered_rho)
        except _capi.TopoError as e:
            if e.code == _capi.TOPO_ERR_NAN:   # the reference's solve returns NaN, Solver stops on it
                return float("nan")
            raise
        return self.compliance(self.u)

    def forward(self, rho) -> Function:
        """Displacement u solving the state equation for the (filtered) density rho."""
        self.penalizer.assert_has_penalization()
        xi = as_cg1_tensor(rho, self.control_space)
        flags = 0
        warm = self.warm_start and self.u is not None
        # a warm start writes every entry of u before the solve reads it: no zero fill
        u = Function(self.solution_space,
                     torch.empty(self.solution_space.dim(), dtype=torch.float64, device=_device()) if warm else None)
        if warm:
            order = min(self.extrapolate_order, len(self._u_hist) - 1) if self.extrapolate else 0
            if order > 0:
                # the design moves a little each iteration: the solve starts from the polynomial
                # extrapolation of the last order + 1 solutions, in one pass on the device,
                #   sum_i (-1)^i binom(order + 1, i + 1) u_(k-i)   (2 u_k - u_(k-1) for order 1)
                hist = (ctypes.c_void_p * (order + 1))(*[h.tensor.data_ptr() for h in self._u_hist[:order + 1]])
                self._ctx.check(self._ctx._lib.topo_state_warm_start(self._ctx.ptr, hist, order + 1, _ptr(u.tensor),
                                                                     _stream()))
            else:
                u.tensor.copy_(self.u.tensor)
            flags = _capi.SOLVE_WARM
        it = ctypes.c_int(0)
        self._ctx.check(self._ctx._lib.topo_state_solve(self._ctx.ptr, _ptr(xi), _ptr(u.tensor), self.rtol, flags,
                                                        ctypes.byref(it), _stream()))
        self.stats["state_iterations"] += it.value
        self._u_hist = ([u] + self._u_hist)[:self.extrapolate_order + 1]
        return u

    # -- extras ---------------------------------------------------------------
    def compliance(self, u: Function) -> float:
        self._ctx.check(self._ctx._lib.topo_compliance(self._ctx.ptr, _ptr(u.tensor), _ptr(self._scalar),
                                                       _stream()))
        return float(self._scalar.item())

    def sensitivity_rhs(self, u: Function, xi) -> torch.Tensor:
        """Assembled b_i = int -r'(xi)(...) phi_i (the gradient before filtering)."""
        b = torch.zeros(self.control_space.dim(), dtype=torch.float64, device=_device())
        x = as_cg1_tensor(xi, self.control_space)
        self._ctx.check(self._ctx._lib.topo_sensitivity_rhs(self._ctx.ptr, _ptr(u.tensor), _ptr(x), _ptr(b),
                                                            _stream()))
        return b

    def apply_operator(self, xi, u: torch.Tensor) -> torch.Tensor:
        """y = K(xi) u (clamped rows and columns replaced by identity), FP64."""
        y = torch.empty_like(u)
        x = as_cg1_tensor(xi, self.control_space)
        self._ctx.check(self._ctx._lib.topo_apply_state(self._ctx.ptr, _ptr(x), _ptr(u), _ptr(y), _stream()))
        return y

    def load_vector(self) -> torch.Tensor:
        b = torch.empty(self.solution_space.dim(), dtype=torch.float64, device=_device())
        self._ctx.check(self._ctx._lib.topo_load_vector(self._ctx.ptr, _ptr(b), _stream()))
        return b
