"""FP64 CPU restatement of the topomax FEM elasticity design loop (the oracle).

TEST INFRASTRUCTURE ONLY -- imported by ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline leg of ``bench.py``; never by the product package.

What it restates (reference file:line, paths inside the topomax project):

* mesh: ``FEM_src/solver.py:38-49`` -- dolfin ``RectangleMesh`` with the default
  "right" diagonal: square (i, j) is split into the triangles (v0, v1, v3)
  and (v0, v2, v3), v0 = bottom-left, v3 = top-right.  Vertex coordinates are
  ``x_i = i * (W / nx)`` as dolfin's mesh generator computes them.
* spaces: CG1 design space (``FEM_src/solver.py:49``) and vector P2
  displacement space (``FEM_src/elasisity_problem.py:194-196``).  P2 nodes
  are the (2nx+1) x (2ny+1) half-spacing lattice; edge-node coordinates are
  ``0.5*a + 0.5*b`` of the edge's end points (how the P2 dof points of an
  interpolated expression are placed).
* material: ``src/penalizers.py:29-46`` r(x) = m + x^p (1-m), m = 1e-6;
  Lame parameters ``FEM_src/elasisity_problem.py:97-99``.
* state operator ``FEM_src/elasisity_problem.py:104-132``:
  a(u, v) = (r(xi) sigma(u), eps(v)) integrated with the 7-point degree-5
  rule (the degree UFL estimates for that form), Dirichlet rows eliminated
  (``FEM_src/pde_solver.py:125``), direct sparse LU solve (MUMPS there,
  SuperLU here).
* loads ``FEM_src/elasisity_problem.py:20-73``: body-force indicator
  ``dist < radius`` and the traction side test (exact coordinate equality
  plus ``df.between`` with DOLFIN_EPS), both evaluated at P2 nodes and
  integrated exactly (P2 mass matrices on cells / boundary facets).
* filter ``FEM_src/filter.py:15-41``: (eps^2 K1 + M1) xi = b.
* objective ``FEM_src/elasisity_problem.py:152-166`` (= b . u) and gradient
  ``FEM_src/elasisity_problem.py:134-150`` (filter of
  -r'(xi)(lambda div(u)^2 + 2 mu eps:eps), RHS integrated with the 12-point
  degree-6 rule).
* design loop ``src/solver.py:149-302`` (EMD step, Newton/Brent projection,
  stopping rules) and ``FEM_src/solver.py:81-84`` (integrate).

Vectors are in lattice order: CG1 vertex ``v = j*(nx+1) + i``; P2 node
``n = b*(2nx+1) + a``; displacement dof ``2*n + c``.
"""
from __future__ import annotations

import json
import math
from dataclasses import dataclass, field

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla
from scipy import optimize

DOLFIN_EPS = 3e-16
PENAL_MIN = 1e-6

# ----------------------------------------------------------------------------
# quadrature rules on triangles, barycentric points, weights summing to 1
# ----------------------------------------------------------------------------


def _orbit3(a: float):
    b = 1.0 - 2.0 * a
    return [(b, a, a), (a, b, a), (a, a, b)]


def _orbit6(a: float, b: float):
    c = 1.0 - a - b
    return [(a, b, c), (a, c, b), (b, a, c), (b, c, a), (c, a, b), (c, b, a)]


def rule_degree5():
    """Radon's 7-point rule (exact to degree 5)."""
    s15 = math.sqrt(15.0)
    a1 = (6.0 - s15) / 21.0
    a2 = (6.0 + s15) / 21.0
    w1 = (155.0 - s15) / 1200.0
    w2 = (155.0 + s15) / 1200.0
    pts = [(1.0 / 3.0, 1.0 / 3.0, 1.0 / 3.0)] + _orbit3(a1) + _orbit3(a2)
    wts = [9.0 / 40.0] + [w1] * 3 + [w2] * 3
    return np.array(pts), np.array(wts)


def rule_degree6():
    """Strang & Fix / Dunavant 12-point rule (exact to degree 6)."""
    pts = (_orbit3(0.063089014491502) + _orbit3(0.249286745170910)
           + _orbit6(0.053145049844816, 0.310352451033785))
    wts = [0.050844906370207] * 3 + [0.116786275726379] * 3 + [0.082851075618374] * 6
    return np.array(pts), np.array(wts)


# ----------------------------------------------------------------------------
# mesh
# ----------------------------------------------------------------------------

# lattice offsets (da, db) of the 6 P2 nodes [A, B, C, mid(BC), mid(AC), mid(AB)]
# of the two triangles of a square: orientation 0 = (v0, v1, v3), 1 = (v0, v2, v3)
P2_OFFSETS = (
    ((0, 0), (2, 0), (2, 2), (2, 1), (1, 1), (1, 0)),
    ((0, 0), (0, 2), (2, 2), (1, 2), (1, 1), (0, 1)),
)
P1_OFFSETS = (((0, 0), (1, 0), (1, 1)), ((0, 0), (0, 1), (1, 1)))


@dataclass
class Lattice:
    width: float
    height: float
    nx: int
    ny: int
    xv: np.ndarray = field(init=False)
    yv: np.ndarray = field(init=False)
    X2: np.ndarray = field(init=False)
    Y2: np.ndarray = field(init=False)

    def __post_init__(self):
        ab = self.width / self.nx
        cd = self.height / self.ny
        self.xv = np.array([0.0 + i * ab for i in range(self.nx + 1)])
        self.yv = np.array([0.0 + j * cd for j in range(self.ny + 1)])
        self.X2 = np.empty(2 * self.nx + 1)
        self.Y2 = np.empty(2 * self.ny + 1)
        self.X2[0::2] = self.xv
        self.X2[1::2] = 0.5 * self.xv[:-1] + 0.5 * self.xv[1:]
        self.Y2[0::2] = self.yv
        self.Y2[1::2] = 0.5 * self.yv[:-1] + 0.5 * self.yv[1:]

    @property
    def hx(self):
        return self.width / self.nx

    @property
    def hy(self):
        return self.height / self.ny

    @property
    def n_vertices(self):
        return (self.nx + 1) * (self.ny + 1)

    @property
    def n_p2(self):
        return (2 * self.nx + 1) * (2 * self.ny + 1)

    def vertex_coords(self):
        X, Y = np.meshgrid(self.xv, self.yv)
        return X.ravel(), Y.ravel()

    def p2_coords(self):
        X, Y = np.meshgrid(self.X2, self.Y2)
        return X.ravel(), Y.ravel()

    def triangle_vertices(self, o: int) -> np.ndarray:
        """(T, 3) CG1 vertex indices of orientation-o triangles, cell-major."""
        j, i = np.meshgrid(np.arange(self.ny), np.arange(self.nx), indexing="ij")
        i = i.ravel()
        j = j.ravel()
        cols = [(j + db) * (self.nx + 1) + (i + da) for da, db in P1_OFFSETS[o]]
        return np.stack(cols, axis=1)

    def triangle_p2_nodes(self, o: int) -> np.ndarray:
        """(T, 6) P2 node indices of orientation-o triangles, cell-major."""
        j, i = np.meshgrid(np.arange(self.ny), np.arange(self.nx), indexing="ij")
        i = i.ravel()
        j = j.ravel()
        n2x = 2 * self.nx + 1
        cols = [(2 * j + db) * n2x + (2 * i + da) for da, db in P2_OFFSETS[o]]
        return np.stack(cols, axis=1)

    def triangle_geometry(self, o: int):
        """(area, grad_lambda (3,2)) shared by every triangle of orientation o."""
        hx, hy = self.hx, self.hy
        if o == 0:
            P = np.array([[0.0, 0.0], [hx, 0.0], [hx, hy]])
        else:
            P = np.array([[0.0, 0.0], [0.0, hy], [hx, hy]])
        x0, y0 = P[0]
        x1, y1 = P[1]
        x2, y2 = P[2]
        a2 = (x1 - x0) * (y2 - y0) - (x2 - x0) * (y1 - y0)
        G = np.array([[y1 - y2, x2 - x1], [y2 - y0, x0 - x2], [y0 - y1, x1 - x0]]) / a2
        return 0.5 * abs(a2), G


def p2_basis(lam: np.ndarray, G: np.ndarray):
    """Values (nq,6) and physical gradients (nq,6,2) of the P2 basis."""
    l0, l1, l2 = lam[:, 0], lam[:, 1], lam[:, 2]
    N = np.stack([l0 * (2 * l0 - 1), l1 * (2 * l1 - 1), l2 * (2 * l2 - 1),
                  4 * l1 * l2, 4 * l0 * l2, 4 * l0 * l1], axis=1)
    g0, g1, g2 = G
    dN = np.stack([
        (4 * l0 - 1)[:, None] * g0, (4 * l1 - 1)[:, None] * g1,
        (4 * l2 - 1)[:, None] * g2,
        4 * (l1[:, None] * g2 + l2[:, None] * g1),
        4 * (l0[:, None] * g2 + l2[:, None] * g0),
        4 * (l0[:, None] * g1 + l1[:, None] * g0),
    ], axis=1)
    return N, dN


def elasticity_qp_matrices(dN: np.ndarray, lmbda: float, mu: float) -> np.ndarray:
    """(nq,12,12): integrand of (sigma(u), eps(v)) at each point, dof 2k+c."""
    nq = dN.shape[0]
    K = np.zeros((nq, 12, 12))
    for c in range(2):
        for d in range(2):
            # K[(m,c),(n,d)] = lam dc(Nm) dd(Nn) + mu dcd grad Nm.grad Nn + mu dc(Nn) dd(Nm)
            blk = lmbda * np.einsum("qm,qn->qmn", dN[:, :, c], dN[:, :, d])
            blk += mu * np.einsum("qn,qm->qmn", dN[:, :, c], dN[:, :, d])
            if c == d:
                blk += mu * np.einsum("qmk,qnk->qmn", dN, dN)
            K[:, c::2, d::2] = blk
    return K


def lame(young: float, poisson: float):
    mu = young / (2 * (1 + poisson))
    lmbda = mu * poisson / (0.5 - poisson)
    return lmbda, mu


def penalize(x, p):
    return PENAL_MIN + x ** p * (1 - PENAL_MIN)


def penalize_derivative(x, p):
    return p * x ** (p - 1) * (1 - PENAL_MIN)


# ----------------------------------------------------------------------------
# design description (the JSON format of designs/*.json)
# ----------------------------------------------------------------------------

SIDES = ("Left", "Right", "Top", "Bottom")


@dataclass
class Design:
    width: float
    height: float
    fem_step_size: float
    penalties: list
    volume_fraction: float
    fixed_sides: list
    body_force: dict | None
    tractions: list | None
    filter_radius: float
    young_modulus: float
    poisson_ratio: float
    fixed_points: list | None = None   # extension: clamped lattice vertices (x, y)

    @classmethod
    def from_file(cls, path: str) -> "Design":
        with open(path, "rb") as f:
            d = json.load(f)
        (key,) = d.keys()
        if key != "Elasticity":
            raise ValueError("oracle handles elasticity designs only")
        dp = d[key]["domain_parameters"]
        pp = d[key]["problem_parameters"]
        return cls(dp["width"], dp["height"], dp["fem_step_size"], list(dp["penalties"]),
                   dp["volume_fraction"], list(pp["fixed_sides"]), pp.get("body_force"),
                   pp.get("tractions"), pp["filter_radius"], pp["young_modulus"],
                   pp["poisson_ratio"], pp.get("fixed_points"))


# ----------------------------------------------------------------------------
# the FEM problem
# ----------------------------------------------------------------------------


class FEMOracle:
    """Assembles and solves every operator of the elasticity design loop."""

    def __init__(self, lattice: Lattice, design: Design):
        self.L = lattice
        self.d = design
        self.lmbda, self.mu = lame(design.young_modulus, design.poisson_ratio)
        self.p = None
        self.rule5 = rule_degree5()
        self.rule6 = rule_degree6()
        self._build_static()

    # -- static pieces -------------------------------------------------------
    def _build_static(self):
        L = self.L
        nv = L.n_vertices
        rows, cols, kv, mv = [], [], [], []
        self.vertex_weights = np.zeros(nv)
        for o in (0, 1):
            area, G = L.triangle_geometry(o)
            tv = L.triangle_vertices(o)
            Ke = area * G @ G.T
            Me = area / 12.0 * (np.ones((3, 3)) + np.eye(3))
            r = np.repeat(tv, 3, axis=1)
            c = np.tile(tv, (1, 3))
            rows.append(r.ravel())
            cols.append(c.ravel())
            kv.append(np.broadcast_to(Ke.ravel(), r.shape).ravel())
            mv.append(np.broadcast_to(Me.ravel(), r.shape).ravel())
            np.add.at(self.vertex_weights, tv.ravel(), area / 3.0)
        rows = np.concatenate(rows)
        cols = np.concatenate(cols)
        self.K1 = sp.csr_matrix((np.concatenate(kv), (rows, cols)), shape=(nv, nv))
        self.M1 = sp.csr_matrix((np.concatenate(mv), (rows, cols)), shape=(nv, nv))
        eps = self.d.filter_radius
        self.A_filter = (eps ** 2 * self.K1 + self.M1).tocsc()
        self._filter_lu = spla.splu(self.A_filter)

        # per-orientation QP tables
        self.tab5 = []
        self.tab6 = []
        for o in (0, 1):
            area, G = L.triangle_geometry(o)
            lam5, w5 = self.rule5
            N5, dN5 = p2_basis(lam5, G)
            Kq = elasticity_qp_matrices(dN5, self.lmbda, self.mu)
            self.tab5.append(dict(area=area, lam=lam5, w=w5, N=N5, dN=dN5, Kq=Kq))
            lam6, w6 = self.rule6
            N6, dN6 = p2_basis(lam6, G)
            self.tab6.append(dict(area=area, lam=lam6, w=w6, N=N6, dN=dN6))

        self.dirichlet_nodes = self._dirichlet_nodes()
        self.load = self._load_vector()
        nd = 2 * L.n_p2
        mask = np.ones(nd, dtype=bool)
        mask[2 * self.dirichlet_nodes] = False
        mask[2 * self.dirichlet_nodes + 1] = False
        self.free = np.nonzero(mask)[0]

    def _dirichlet_nodes(self) -> np.ndarray:
        L = self.L
        n2x, n2y = 2 * L.nx + 1, 2 * L.ny + 1
        a, b = np.meshgrid(np.arange(n2x), np.arange(n2y))
        a = a.ravel()
        b = b.ravel()
        m = np.zeros(L.n_p2, dtype=bool)
        for s in self.d.fixed_sides:
            if s == "Left":
                m |= a == 0
            elif s == "Right":
                m |= a == n2x - 1
            elif s == "Top":
                m |= b == n2y - 1
            elif s == "Bottom":
                m |= b == 0
            else:
                raise ValueError(f"Malformed side: {s}")
        for (px, py) in (self.d.fixed_points or []):
            i = int(round(px / L.hx))
            j = int(round(py / L.hy))
            m |= (a == 2 * i) & (b == 2 * j)
        return np.nonzero(m)[0]

    def traction_at(self, x: float, y: float):
        vx = vy = 0.0
        W, H = self.d.width, self.d.height
        for t in self.d.tractions or []:
            lo = t["center"] - t["length"] / 2
            hi = t["center"] + t["length"] / 2
            side = t["side"]
            if side == "Left":
                hit = x == 0.0 and lo - DOLFIN_EPS <= y <= hi + DOLFIN_EPS
            elif side == "Right":
                hit = x == W and lo - DOLFIN_EPS <= y <= hi + DOLFIN_EPS
            elif side == "Top":
                hit = y == H and lo - DOLFIN_EPS <= x <= hi + DOLFIN_EPS
            elif side == "Bottom":
                hit = y == 0 and lo - DOLFIN_EPS <= x <= hi + DOLFIN_EPS
            else:
                raise ValueError(f"Malformed side: {side}")
            if hit:
                vx += t["value"][0]
                vy += t["value"][1]
        return vx, vy

    def body_force_nodal(self) -> np.ndarray:
        """(n_p2, 2) P2 interpolant of the body-force indicator."""
        L = self.L
        f = np.zeros((L.n_p2, 2))
        bf = self.d.body_force
        if bf is None:
            return f
        X, Y = L.p2_coords()
        cx, cy = bf["region"]["center"]
        dist = np.sqrt((X - cx) ** 2 + (Y - cy) ** 2)
        inside = dist < bf["region"]["radius"]
        f[inside, 0] = bf["value"][0]
        f[inside, 1] = bf["value"][1]
        return f

    def _load_vector(self) -> np.ndarray:
        L = self.L
        b = np.zeros(2 * L.n_p2)
        fn = self.body_force_nodal()
        if np.any(fn):
            for o in (0, 1):
                t = self.tab5[o]
                Me = t["area"] * np.einsum("q,qm,qn->mn", t["w"], t["N"], t["N"])
                nodes = L.triangle_p2_nodes(o)
                for c in range(2):
                    fe = fn[nodes, c]            # (T, 6)
                    np.add.at(b, 2 * nodes + c, fe @ Me.T)
        # boundary facets: 1D quadratic mass matrix, nodes (end0, mid, end1)
        n2x = 2 * L.nx + 1
        X, Y = L.p2_coords()
        if self.d.tractions:
            facets = []
            for i in range(L.nx):          # bottom / top
                for bb in (0, 2 * L.ny):
                    facets.append(([bb * n2x + 2 * i, bb * n2x + 2 * i + 1,
                                    bb * n2x + 2 * i + 2], L.hx))
            for j in range(L.ny):          # left / right
                for aa in (0, 2 * L.nx):
                    facets.append(([(2 * j) * n2x + aa, (2 * j + 1) * n2x + aa,
                                    (2 * j + 2) * n2x + aa], L.hy))
            Mf = np.array([[4.0, 2.0, -1.0], [2.0, 16.0, 2.0], [-1.0, 2.0, 4.0]]) / 30.0
            for nodes, h in facets:
                tv = np.array([self.traction_at(X[n], Y[n]) for n in nodes])
                if not np.any(tv):
                    continue
                contrib = h * Mf @ tv        # (3, 2)
                for k, n in enumerate(nodes):
                    b[2 * n] += contrib[k, 0]
                    b[2 * n + 1] += contrib[k, 1]
        return b

    # -- penalisation ---------------------------------------------------------
    def set_penalization(self, p: float):
        self.p = float(p)

    def _need_p(self):
        if self.p is None:
            raise ValueError("You must set penalization before calling penalizer")
        return self.p

    # -- filter ---------------------------------------------------------------
    def filter_rhs_cg1(self, f: np.ndarray) -> np.ndarray:
        return self.M1 @ f

    def filter_solve(self, rhs: np.ndarray) -> np.ndarray:
        return self._filter_lu.solve(rhs)

    def filter_apply(self, f: np.ndarray) -> np.ndarray:
        return self.filter_solve(self.filter_rhs_cg1(f))

    # -- state ----------------------------------------------------------------
    def element_coefficients(self, xi: np.ndarray, o: int) -> np.ndarray:
        """(T, 7) w_q |T| r(xi_q) for the 7-point rule."""
        t = self.tab5[o]
        xq = xi[self.L.triangle_vertices(o)] @ t["lam"].T
        return penalize(xq, self._need_p()) * t["w"][None, :] * t["area"]

    def stiffness(self, xi: np.ndarray) -> sp.csr_matrix:
        L = self.L
        nd = 2 * L.n_p2
        rows, cols, vals = [], [], []
        for o in (0, 1):
            coef = self.element_coefficients(xi, o)
            Ke = np.einsum("tq,qab->tab", coef, self.tab5[o]["Kq"])
            nodes = L.triangle_p2_nodes(o)
            dofs = np.empty((nodes.shape[0], 12), dtype=np.int64)
            dofs[:, 0::2] = 2 * nodes
            dofs[:, 1::2] = 2 * nodes + 1
            rows.append(np.repeat(dofs, 12, axis=1).ravel())
            cols.append(np.tile(dofs, (1, 12)).ravel())
            vals.append(Ke.ravel())
        return sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                             shape=(nd, nd))

    def state_solve(self, xi: np.ndarray) -> np.ndarray:
        K = self.stiffness(xi)
        f = self.free
        Kff = K[f][:, f].tocsc()
        u = np.zeros(2 * self.L.n_p2)
        # symmetric fill-reducing ordering (minimum degree on A^T + A), as a symmetric
        # multifrontal LU such as MUMPS orders the matrix; SuperLU's default column
        # ordering fills in about 2.5x more work on this matrix
        u[f] = spla.spsolve(Kff, self.load[f], permc_spec="MMD_AT_PLUS_A")
        return u

    def apply_state(self, xi: np.ndarray, u: np.ndarray) -> np.ndarray:
        """y = K(xi) u with Dirichlet dofs treated as identity rows/cols."""
        K = self.stiffness(xi)
        uu = u.copy()
        dd = np.concatenate([2 * self.dirichlet_nodes, 2 * self.dirichlet_nodes + 1])
        uu[dd] = 0.0
        y = K @ uu
        y[dd] = u[dd]
        return y

    def compliance(self, u: np.ndarray) -> float:
        return float(self.load @ u)

    # -- sensitivity ----------------------------------------------------------
    def sensitivity_rhs(self, u: np.ndarray, xi: np.ndarray) -> np.ndarray:
        """b_i = int -r'(xi)(lambda div(u)^2 + 2 mu eps:eps) phi_i (12-point rule)."""
        p = self._need_p()
        L = self.L
        b = np.zeros(L.n_vertices)
        U = u.reshape(-1, 2)
        for o in (0, 1):
            t = self.tab6[o]
            nodes = L.triangle_p2_nodes(o)
            tv = L.triangle_vertices(o)
            ux = U[nodes, 0]                        # (T, 6)
            uy = U[nodes, 1]
            dN = t["dN"]                            # (q, 6, 2)
            uxx = ux @ dN[:, :, 0].T                # (T, q)
            uxy = ux @ dN[:, :, 1].T
            uyx = uy @ dN[:, :, 0].T
            uyy = uy @ dN[:, :, 1].T
            div = uxx + uyy
            exy = 0.5 * (uxy + uyx)
            ee = uxx ** 2 + uyy ** 2 + 2 * exy ** 2
            xq = xi[tv] @ t["lam"].T
            s = -penalize_derivative(xq, p) * (self.lmbda * div ** 2 + 2 * self.mu * ee)
            contrib = (s * t["w"][None, :] * t["area"]) @ t["lam"]     # (T, 3)
            np.add.at(b, tv.ravel(), contrib.ravel())
        return b

    def gradient(self, u: np.ndarray, xi: np.ndarray) -> np.ndarray:
        return self.filter_solve(self.sensitivity_rhs(u, xi))

    # -- integral of a CG1 function ------------------------------------------
    def integrate(self, values: np.ndarray) -> float:
        return float(self.vertex_weights @ values)


# ----------------------------------------------------------------------------
# the problem object with the reference's call surface
# ----------------------------------------------------------------------------


class OracleElasticityProblem:
    """``ElasticityProblem`` semantics (FEM_src/elasisity_problem.py:76-196)."""

    def __init__(self, oracle: FEMOracle):
        self.o = oracle
        self.u = None
        self.filtered_rho = None

    def set_penalization(self, p):
        self.o.set_penalization(p)

    def calculate_objective(self, rho):
        self.filtered_rho = self.o.filter_apply(rho)
        self.u = self.o.state_solve(self.filtered_rho)
        return self.o.compliance(self.u)

    def calculate_objective_gradient(self):
        if self.filtered_rho is None or self.u is None:
            raise ValueError("You must call calculate_objective "
                             "before calling calculate_objective_gradient")
        return self.o.gradient(self.u, self.filtered_rho)

    def forward(self, rho):
        return self.o.state_solve(rho)


def expit(x):
    return 1.0 / (1.0 + np.exp(-x))


def expit_diff(x):
    e = expit(x)
    return e * (1 - e)


def logit(x):
    return np.log(x / (1.0 - x))


def smart_brentq(f, initial_radius: float, max_radius: float):
    """``src/utils.py:138-157``: grow [-r, r] until f changes sign."""
    r = initial_radius
    while True:
        if r > max_radius:
            raise ValueError("f(-max_radius) and f(max_radius) must have different signs!")
        try:
            return optimize.brentq(f, -r, r, full_output=True)
        except ValueError:
            r *= 2


@dataclass
class OracleRun:
    objectives: list
    rho: np.ndarray
    psi: np.ndarray
    exit_condition: str
    iterations: int
    penalty: float
    rho_history: list


class OracleSolver:
    """``Solver.solve`` (src/solver.py:208-302) on the oracle problem."""

    def __init__(self, N: int, design: Design, max_iterations: int = 1000,
                 keep_history: bool = False):
        self.design = design
        self.width, self.height = design.width, design.height
        self.N = int(N / min(self.width, self.height))
        self.lattice = Lattice(self.width, self.height, int(self.width * self.N),
                               int(self.height * self.N))
        self.oracle = FEMOracle(self.lattice, design)
        self.problem = OracleElasticityProblem(self.oracle)
        self.volume = self.width * self.height * design.volume_fraction
        self.step_size = design.fem_step_size
        self.rho = np.full(self.lattice.n_vertices, float(design.volume_fraction))
        self.max_iterations = max_iterations
        self.keep_history = keep_history

    def integrate(self, v):
        return self.oracle.integrate(v)

    def project(self, half_step, volume):
        def error(c):
            return self.integrate(expit(half_step + c)) - volume

        def error_derivative(c):
            return self.integrate(expit_diff(half_step + c))

        try:
            c, result = optimize.newton(error, 0, error_derivative, tol=1e-12,
                                        full_output=True)
            if result.converged:
                return half_step + c
        except RuntimeError:
            pass
        c, result = smart_brentq(error, 2, 2000)
        if not result.converged:
            raise ValueError("Projection failed to converge")
        return half_step + c

    def step(self, previous_psi, step_size):
        g = self.problem.calculate_objective_gradient()
        return self.project(previous_psi - step_size * g, self.volume)

    @staticmethod
    def tolerance(k):
        return min(25 * (k + 1) * 1e-5, 1e-2)

    def step_size_at_iter(self, k):
        if len(self.design.penalties) > 1:
            return self.step_size * min(k + 1, 10)
        return self.step_size * (k + 1)

    def solve(self) -> list[OracleRun]:
        runs = []
        psi = logit(self.rho)
        for penalty in self.design.penalties:
            self.problem.set_penalization(penalty)
            objectives = [self.problem.calculate_objective(self.rho)]
            hist = [self.rho.copy()] if self.keep_history else []
            exit_condition = ""
            k = 0
            for k in range(self.max_iterations):
                previous_psi = psi.copy()
                try:
                    psi = self.step(previous_psi, self.step_size_at_iter(k))
                except ValueError as e:
                    exit_condition = str(e)
                    break
                self.rho = expit(psi)
                objectives.append(self.problem.calculate_objective(self.rho))
                if self.keep_history:
                    hist.append(self.rho.copy())
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
                diff = np.sqrt(self.integrate((self.rho - expit(previous_psi)) ** 2))
                if diff < self.tolerance(k):
                    exit_condition = "Convergence treshold reached"
                    break
            else:
                exit_condition = "Iteration did not converge"
            runs.append(OracleRun(objectives, self.rho.copy(), psi.copy(), exit_condition,
                                  k + 1, penalty, hist))
        return runs
