"""FP64 CPU restatement of the Stokes-Brinkman fluid problem (test infrastructure only).

The checker of the product's fluid path (csrc/topo_fluid.cu), pinned against the
reference's own known answer (``tests/test_fluid_solver.py``: the diffuser at
N = 20, penalty 0.1, objective 33.4987342021016 after 20 design steps).

Follows ``FEM_src/fluid_problem.py:12-155`` and ``src/penalizers.py:49-67``:

* state (Taylor-Hood, vector P2 velocity and P1 pressure on the right-diagonal
  lattice): a((u,p),(v,q)) = (alpha(rho) u, v) + (grad u, grad v) + (grad p, v)
  + (div u, q) = 0, Dirichlet velocity on every side (the parabolic flow profiles
  of ``BoundaryFlows`` on the flow sides, no slip elsewhere, the no-slip rows last);
* alpha(rho) = a_max + (a_min - a_max) rho (1 + q) / (rho + q), a_min = 2.5/100^2,
  a_max = 2.5/0.01^2;
* objective 1/2 int alpha(rho) |u|^2 + mu |grad u|^2 dx;
* gradient: the L2 projection onto CG1 of 1/2 alpha'(rho) |u|^2.

Quadrature follows the form compiler's degree estimates: degree 6 for the state
form and the objective (Strang-Fix 12-point rule), degree 7 for the projection's
right-hand side (the collapsed Gauss-Jacobi rule with 4 x 4 points that FIAT uses
above degree 6).  The pressure is determined up to a constant and the discrete
boundary flux of the diffuser's interpolated outflow profile is not exactly zero
(-1.7e-4 of 2/3): the reference hands that singular, slightly inconsistent system to
MUMPS, whose answer depends on its pivoting.  ``pressure = "lsq"`` (default) takes the
least-squares solution of the whole system, ``"mean"`` that of the reduced system (the
Dirichlet rows eliminated, the continuity right-hand side projected to zero sum, zero-sum
pressure: the closure the GPU solver computes), ``"pin"`` drops the continuity row of
vertex 0.  Parity is partial: the known answer's iteration count and exit condition are
reproduced, its objective to 5.6e-4 (``lsq`` and ``mean``; 1.4e-3 with ``pin``; no
single dropped continuity row comes closer than 1.9e-4).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla
from scipy.special import roots_jacobi

from oracle.fem import Lattice, OracleSolver, p2_basis, rule_degree6

A_MIN = 2.5 / 100 ** 2
A_MAX = 2.5 / 0.01 ** 2
SIDES = {"Left": 1, "Right": 2, "Top": 3, "Bottom": 4}


def fluid_penalty(rho, q):
    return A_MAX + (A_MIN - A_MAX) * rho * (1 + q) / (rho + q)


def fluid_penalty_derivative(rho, q):
    return (A_MIN - A_MAX) * q * (1 + q) / (rho + q) ** 2


def rule_degree7():
    """Collapsed Gauss-Jacobi rule, 4 x 4 points (exact to degree 7): Gauss-Legendre in
    one direction, Gauss-Jacobi with weight (1 - eta) in the collapsed one.  Barycentric
    points (1 - s - t, s, t) of the reference triangle, weights summing to 1."""
    x, wx = roots_jacobi(4, 0.0, 0.0)
    y, wy = roots_jacobi(4, 1.0, 0.0)
    pts, wts = [], []
    for xi, w1 in zip(x, wx):
        for eta, w2 in zip(y, wy):
            s = 0.25 * (1.0 + xi) * (1.0 - eta)
            t = 0.5 * (1.0 + eta)
            pts.append((1.0 - s - t, s, t))
            wts.append(0.25 * w1 * w2)
    return np.array(pts), np.array(wts)


@dataclass
class FluidDesign:
    width: float
    height: float
    fem_step_size: float
    penalties: list
    volume_fraction: float
    flows: list = field(default_factory=list)  # (side, center, length, rate)
    viscosity: float = 1.0

    @classmethod
    def from_dict(cls, d: dict) -> "FluidDesign":
        dp = d["Fluid"]["domain_parameters"]
        pp = d["Fluid"]["problem_parameters"]
        flows = [(f["side"], f["center"], f["length"], f["rate"]) for f in pp["flows"]]
        return cls(dp["width"], dp["height"], dp["fem_step_size"], list(dp["penalties"]),
                   dp["volume_fraction"], flows, pp["viscosity"])


def _flow(pos: float, center: float, length: float, rate: float) -> float:
    t = pos - center
    if -length / 2 < t < length / 2:
        return rate * (1 - (2 * t / length) ** 2)
    return 0.0


class FluidOracle:
    """Assembles and solves the Stokes-Brinkman state and its objective and gradient."""

    def __init__(self, lattice: Lattice, design: FluidDesign, pressure: str = "lsq"):
        self.L = L = lattice
        self.d = design
        self.pressure = pressure
        self.n2 = L.n_p2
        self.nv = L.n_vertices
        self.nuv = 2 * self.n2
        self.n = self.nuv + self.nv
        self.q = None
        self.r6 = rule_degree6()
        self.r7 = rule_degree7()
        self.tab = []
        for o in (0, 1):
            area, G = L.triangle_geometry(o)
            lam6, w6 = self.r6
            N6, dN6 = p2_basis(lam6, G)
            lam7, w7 = self.r7
            N7, dN7 = p2_basis(lam7, G)
            lap = area * np.einsum("q,qik,qjk->ij", w6, dN6, dN6)
            grad = area * np.einsum("q,qi,kc->ick", w6, N6, G)      # int N_i d_c(lambda_k)
            div = area * np.einsum("q,qk,qjc->kjc", w6, lam6, dN6)   # int lambda_k d_c(N_j)
            nn = np.einsum("qi,qj->qij", N6, N6)
            self.tab.append(dict(area=area, G=G, lam6=lam6, w6=w6, N6=N6, dN6=dN6, lam7=lam7, w7=w7, N7=N7,
                                 lap=lap, grad=grad, div=div, nn=nn,
                                 p2=L.triangle_p2_nodes(o), v=L.triangle_vertices(o)))
        self._bc()
        self._cg1()

    # -- boundary conditions (FEM_src/fluid_problem.py:12-45, 126-150) -------
    def _bc(self):
        L = self.L
        X, Y = L.p2_coords()
        n2x, n2y = 2 * L.nx + 1, 2 * L.ny + 1
        a = np.tile(np.arange(n2x), n2y)
        b = np.repeat(np.arange(n2y), n2x)
        on = {"Left": a == 0, "Right": a == n2x - 1, "Bottom": b == 0, "Top": b == n2y - 1}
        flow_sides = [f[0] for f in self.d.flows]
        vals = np.zeros((self.n2, 2))
        for node in np.nonzero(np.any([on[s] for s in flow_sides], axis=0))[0]:
            x, y = X[node], Y[node]
            v = [0.0, 0.0]
            for side, center, length, rate in self.d.flows:
                if side == "Left" and x == 0.0:
                    v[0] += _flow(y, center, length, rate)
                elif side == "Right" and x == self.d.width:
                    v[0] -= _flow(y, center, length, rate)
                elif side == "Top" and y == self.d.height:
                    v[1] -= _flow(x, center, length, rate)
                elif side == "Bottom" and y == 0:
                    v[1] += _flow(x, center, length, rate)
            vals[node] = v
        no_slip = [s for s in SIDES if s not in flow_sides]
        if no_slip:
            vals[np.any([on[s] for s in no_slip], axis=0)] = 0.0
        nodes = np.nonzero(np.any(list(on.values()), axis=0))[0]
        self.bc_dofs = np.concatenate([2 * nodes, 2 * nodes + 1])
        self.bc_vals = np.concatenate([vals[nodes, 0], vals[nodes, 1]])

    def _cg1(self):
        L = self.L
        rows, cols, vals = [], [], []
        self.vertex_weights = np.zeros(self.nv)
        for t in self.tab:
            Me = t["area"] / 12.0 * (np.ones((3, 3)) + np.eye(3))
            tv = t["v"]
            rows.append(np.repeat(tv, 3, axis=1).ravel())
            cols.append(np.tile(tv, (1, 3)).ravel())
            vals.append(np.broadcast_to(Me.ravel(), (tv.shape[0], 9)).ravel())
            np.add.at(self.vertex_weights, tv.ravel(), t["area"] / 3.0)
        self.M1 = sp.csc_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                                shape=(self.nv, self.nv))
        self._m1_lu = spla.splu(self.M1)

    # -- state -------------------------------------------------------------------
    def set_penalization(self, q: float):
        self.q = float(q)

    def _rho_at(self, rho, t, lam):
        return rho[t["v"]] @ lam.T

    def assemble(self, rho) -> sp.csr_matrix:
        rows, cols, vals = [], [], []
        for t in self.tab:
            T = t["p2"].shape[0]
            alpha = fluid_penalty(self._rho_at(rho, t, t["lam6"]), self.q)          # (T, nq)
            mass = t["area"] * np.einsum("tq,q,qij->tij", alpha, t["w6"], t["nn"])  # (T, 6, 6)
            blk = mass + t["lap"][None]
            vdof = np.empty((T, 12), dtype=np.int64)
            vdof[:, 0::2] = 2 * t["p2"]
            vdof[:, 1::2] = 2 * t["p2"] + 1
            Ae = np.zeros((T, 12, 12))
            Ae[:, 0::2, 0::2] = blk
            Ae[:, 1::2, 1::2] = blk
            rows.append(np.repeat(vdof, 12, axis=1).ravel())
            cols.append(np.tile(vdof, (1, 12)).ravel())
            vals.append(Ae.ravel())
            pdof = self.nuv + t["v"]                                               # (T, 3)
            Ge = np.zeros((12, 3))
            Ge[0::2] = t["grad"][:, 0, :]
            Ge[1::2] = t["grad"][:, 1, :]
            rows.append(np.repeat(vdof, 3, axis=1).ravel())
            cols.append(np.tile(pdof, (1, 12)).ravel())
            vals.append(np.broadcast_to(Ge.ravel(), (T, 36)).ravel())
            De = np.zeros((3, 12))
            De[:, 0::2] = t["div"][:, :, 0]
            De[:, 1::2] = t["div"][:, :, 1]
            rows.append(np.repeat(pdof, 12, axis=1).ravel())
            cols.append(np.tile(vdof, (1, 3)).ravel())
            vals.append(np.broadcast_to(De.ravel(), (T, 36)).ravel())
        return sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                             shape=(self.n, self.n))

    def state_solve(self, rho):
        """Velocity (2*n2, interleaved) and pressure (n_vertices)."""
        if self.pressure == "mean":
            return self._state_solve_mean(rho)
        K = self.assemble(rho)
        b = np.zeros(self.n)
        keep = np.ones(self.n)
        keep[self.bc_dofs] = 0.0
        b[self.bc_dofs] = self.bc_vals
        ident = np.zeros(self.n)
        ident[self.bc_dofs] = 1.0
        K0 = (sp.diags(keep) @ K + sp.diags(ident)).tocsr()
        if self.pressure == "lsq":
            # the system is singular (pressure constant) and, with the interpolated
            # boundary data, slightly inconsistent: remove the right-hand side's
            # component along the left null vector y (1 on the pressure rows, minus
            # the boundary fluxes of the Dirichlet dofs) -- the least-squares
            # solution -- then close it by one pressure row
            y = np.zeros(self.n)
            y[self.nuv:] = 1.0
            fb = np.asarray(K0[self.nuv:, :self.nuv].sum(axis=0)).ravel()
            y[self.bc_dofs] = -fb[self.bc_dofs]
            b = b - (y @ b) / (y @ y) * y
        keep1 = np.ones(self.n)
        keep1[self.nuv] = 0.0
        id1 = np.zeros(self.n)
        id1[self.nuv] = 1.0
        b[self.nuv] = 0.0
        x = spla.spsolve((sp.diags(keep1) @ K0 + sp.diags(id1)).tocsc(), b)
        return x[:self.nuv], x[self.nuv:]

    def _state_solve_mean(self, rho):
        """The closure of the reduced system: the Dirichlet velocity dofs eliminated, the
        continuity right-hand side projected to zero sum (its Euclidean least-squares
        part), the pressure fixed by sum(p) = 0 through a bordering row."""
        K = self.assemble(rho).tocsr()
        nuv = self.nuv
        bc = np.zeros(nuv, bool)
        bc[self.bc_dofs] = True
        I = np.nonzero(~bc)[0]
        uB = np.zeros(nuv)
        uB[self.bc_dofs] = self.bc_vals
        A, G, D = K[:nuv, :nuv], K[:nuv, nuv:], K[nuv:, :nuv]
        f = -(A[I] @ uB)
        g = -(D @ uB)
        g = g - g.mean()
        ones = sp.csr_matrix(np.ones((self.nv, 1)))
        S = sp.bmat([[A[I][:, I], G[I], None], [D[:, I], None, ones], [None, ones.T, None]]).tocsc()
        x = spla.spsolve(S, np.concatenate([f, g, [0.0]]))
        u = uB.copy()
        u[I] = x[:I.size]
        return u, x[I.size:I.size + self.nv]

    def boundary_flux(self, rho=None) -> float:
        """int div u_h dx of the interpolated boundary data (zero for a compatible one)."""
        u = np.zeros(self.nuv)
        u[self.bc_dofs] = self.bc_vals
        s = 0.0
        for t in self.tab:
            ue = np.stack([u[2 * t["p2"]], u[2 * t["p2"] + 1]], axis=2)   # (T, 6, 2)
            s += float(np.einsum("kjc,tjc->", t["div"], ue))
        return s

    def _u_at(self, u, t, N, dN=None):
        ue = np.stack([u[2 * t["p2"]], u[2 * t["p2"] + 1]], axis=2)       # (T, 6, 2)
        uq = np.einsum("qi,tic->tqc", N, ue)
        gq = None if dN is None else np.einsum("qik,tic->tqck", dN, ue)
        return uq, gq

    def objective(self, rho, u) -> float:
        s = 0.0
        for t in self.tab:
            uq, gq = self._u_at(u, t, t["N6"], t["dN6"])
            alpha = fluid_penalty(self._rho_at(rho, t, t["lam6"]), self.q)
            f = alpha * np.sum(uq * uq, axis=2) + self.d.viscosity * np.sum(gq * gq, axis=(2, 3))
            s += t["area"] * float(np.sum(f * t["w6"][None]))
        return 0.5 * s

    def gradient(self, rho, u) -> np.ndarray:
        rhs = np.zeros(self.nv)
        for t in self.tab:
            uq, _ = self._u_at(u, t, t["N7"])
            dr = fluid_penalty_derivative(self._rho_at(rho, t, t["lam7"]), self.q)
            f = 0.5 * dr * np.sum(uq * uq, axis=2) * t["w7"][None] * t["area"]  # (T, nq)
            np.add.at(rhs, t["v"], f @ t["lam7"])
        return self._m1_lu.solve(rhs)

    def integrate(self, values) -> float:
        return float(self.vertex_weights @ values)


class OracleFluidProblem:
    """Problem interface (set_penalization, calculate_objective, calculate_objective_gradient)."""

    def __init__(self, oracle: FluidOracle):
        self.o = oracle
        self.rho = None
        self.u = None

    def set_penalization(self, p):
        self.o.set_penalization(p)

    def calculate_objective(self, rho):
        self.rho = np.asarray(rho, dtype=np.float64).copy()
        self.u, _ = self.o.state_solve(self.rho)
        return self.o.objective(self.rho, self.u)

    def calculate_objective_gradient(self):
        if self.rho is None or self.u is None:
            raise ValueError("You must call calculate_objective before calling calculate_objective_gradient")
        return self.o.gradient(self.rho, self.u)


class FluidOracleSolver(OracleSolver):
    """``Solver.solve`` (src/solver.py:208-302) on the fluid problem."""

    def __init__(self, N: int, design: FluidDesign, max_iterations: int = 1000, pressure: str = "lsq"):
        self.design = design
        self.width, self.height = design.width, design.height
        self.N = int(N / min(self.width, self.height))
        self.lattice = Lattice(self.width, self.height, int(self.width * self.N), int(self.height * self.N))
        self.oracle = FluidOracle(self.lattice, design, pressure)
        self.problem = OracleFluidProblem(self.oracle)
        self.volume = self.width * self.height * design.volume_fraction
        self.step_size = design.fem_step_size
        self.rho = np.full(self.lattice.n_vertices, float(design.volume_fraction))
        self.max_iterations = max_iterations
        self.keep_history = False
