"""The fluid kernels' triangle phases and gathers (run on the CPU through the emulator)
against the Stokes-Brinkman oracle (oracle/fluid.py).

Covers the element tables and quadrature rules, the Dirichlet data of the flow
profiles, the operator (with the continuity rows negated), its symmetry on
interior velocities, the objective, the gradient's right-hand side, the
reduced-system closure the GPU solve computes (the oracle's ``pressure="mean"``),
and the block-preconditioned flexible GMRES of the state solve run with the
emulated multigrid phases.
"""
import json
import os

import numpy as np
import pytest
import scipy.linalg

from oracle.fem import Lattice, rule_degree6
from oracle.fluid import (A_MAX, A_MIN, FluidDesign, FluidOracle, fluid_penalty, fluid_penalty_derivative,
                          rule_degree7)
from tests import emu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")

# four flows on three sides (two on one side, one on the top): exercises every branch of
# the flow profiles and the no-slip override at the corners
MIXED = dict(Fluid=dict(domain_parameters=dict(width=1.5, height=1.0, fem_step_size=0.001, dem_step_size=0.001,
                                               penalties=[0.01], volume_fraction=1 / 3),
                        problem_parameters=dict(flows=[
                            dict(side="Left", center=0.25, length=0.2, rate=1.0),
                            dict(side="Left", center=0.75, length=0.2, rate=1.0),
                            dict(side="Right", center=0.25, length=0.2, rate=-1.0),
                            dict(side="Top", center=0.75, length=0.3, rate=-1.0)], viscosity=1.0)))


def design(name):
    if name == "mixed":
        return FluidDesign.from_dict(MIXED)
    with open(os.path.join(GOLDEN, "designs", f"{name}.json")) as f:
        return FluidDesign.from_dict(json.load(f))


def diffuser():
    return design("diffuser")


def setup(design, nx, ny, q=0.1, seed=0):
    L = Lattice(design.width, design.height, nx, ny)
    o = FluidOracle(L, design)
    o.set_penalization(q)
    rng = np.random.default_rng(seed)
    rho = rng.uniform(0.0, 1.0, L.n_vertices)
    return L, o, rho


def test_quadrature_rules_and_tables_match_the_oracle():
    L, o, _ = setup(diffuser(), 5, 4)
    T = emu.fluid_tables(L.hx, L.hy)
    lam6, w6 = rule_degree6()
    lam7, w7 = rule_degree7()
    assert np.array_equal(T["lam6"], lam6) and np.array_equal(T["w6"], w6)
    assert np.max(np.abs(T["lam7"] - lam7)) < 4e-16 and np.max(np.abs(T["w7"] - w7)) < 4e-16
    for k in (0, 1):
        t = o.tab[k]
        assert abs(T["area"] - t["area"]) < 1e-17
        assert np.max(np.abs(T["dN6"][k] - t["dN6"])) < 1e-12
        assert np.max(np.abs(T["lap"][k] - t["lap"])) < 1e-14
        # grad[i][c][k] = int N_i d_c lambda_k ; the oracle stores (i, c, k) the same way
        assert np.max(np.abs(T["grad"][k] - t["grad"])) < 1e-16
        assert np.max(np.abs(T["div"][k] - t["div"])) < 1e-16


def test_penalty_matches_the_reference_formula():
    assert A_MIN == 2.5 / 100 ** 2 and A_MAX == 2.5 / 0.01 ** 2
    for q in (0.01, 0.1, 1.0):
        for r in (0.0, 0.3, 1.0, 0.999):
            assert emu.fluid_alpha(q, r) == fluid_penalty(r, q)
            assert emu.fluid_alpha(q, r, True) == fluid_penalty_derivative(r, q)


@pytest.mark.parametrize("name,nx,ny", [("diffuser", 6, 6), ("mixed", 9, 6), ("diffuser", 20, 20),
                                         ("twin_pipe", 15, 10), ("pipe_bend", 10, 10)])
def test_boundary_data_match_the_oracle(name, nx, ny):
    d = design(name)
    L, o, _ = setup(d, nx, ny)
    ub = emu.fluid_bc(nx, ny, d.width, d.height, d.flows)
    ref = np.zeros(o.nuv)
    ref[o.bc_dofs] = o.bc_vals
    assert np.array_equal(ub, ref)


def test_node_incidence_covers_every_triangle_node_once():
    nx, ny = 4, 3
    L = Lattice(1.0, 1.0, nx, ny)
    seen = {}
    for b in range(2 * ny + 1):
        for a in range(2 * nx + 1):
            for t, loc in emu.p2_node_incidence(a, b, nx, ny):
                nodes = L.triangle_p2_nodes(t & 1)[t >> 1]
                assert nodes[loc] == b * (2 * nx + 1) + a
                seen[(t, loc)] = seen.get((t, loc), 0) + 1
    assert len(seen) == 2 * nx * ny * 6 and set(seen.values()) == {1}


def _oracle_operator(o, rho):
    K = o.assemble(rho).tocsr().astype(np.float64)
    S = np.ones(o.n)
    S[o.nuv:] = -1.0  # the kernels negate the continuity rows
    return K, S


@pytest.mark.parametrize("name,nx,ny,q", [("diffuser", 6, 5, 0.1), ("mixed", 9, 6, 0.01), ("pipe_bend", 7, 7, 0.1)])
def test_operator_matches_the_assembled_oracle(name, nx, ny, q):
    d = design(name)
    L, o, rho = setup(d, nx, ny, q)
    K, S = _oracle_operator(o, rho)
    x = np.random.default_rng(3).standard_normal(o.n)
    y = emu.fluid_apply(nx, ny, d.width, d.height, q, rho, x)
    ref = S * (K @ x)
    assert np.max(np.abs(y - ref)) <= 1e-13 * np.max(np.abs(ref))
    # clamped: identity rows on the boundary velocity dofs, the rest unchanged
    yc = emu.fluid_apply(nx, ny, d.width, d.height, q, rho, x, clamp=True)
    bc = np.zeros(o.n, bool)
    bc[o.bc_dofs] = True
    assert np.array_equal(yc[bc], x[bc])
    assert np.array_equal(yc[~bc], y[~bc])


def test_clamped_operator_is_symmetric_on_interior_velocities():
    d = diffuser()
    nx = ny = 6
    L, o, rho = setup(d, nx, ny)
    rng = np.random.default_rng(4)
    bc = np.zeros(o.n, bool)
    bc[o.bc_dofs] = True
    x, z = rng.standard_normal(o.n), rng.standard_normal(o.n)
    x[bc] = 0.0
    z[bc] = 0.0
    a = z @ emu.fluid_apply(nx, ny, d.width, d.height, 0.1, rho, x, clamp=True)
    b = x @ emu.fluid_apply(nx, ny, d.width, d.height, 0.1, rho, z, clamp=True)
    assert abs(a - b) <= 1e-12 * abs(a)


def test_objective_and_gradient_rhs_match_the_oracle():
    d = diffuser()
    nx, ny = 8, 8
    L, o, rho = setup(d, nx, ny, q=0.1)
    u, _ = o.state_solve(rho)
    J = emu.fluid_objective(nx, ny, d.width, d.height, 0.1, d.viscosity, rho, u)
    assert abs(J - o.objective(rho, u)) <= 1e-13 * abs(J)
    b = emu.fluid_gradient_rhs(nx, ny, d.width, d.height, 0.1, rho, u)
    ref = o.M1 @ o.gradient(rho, u)
    assert np.max(np.abs(b - ref)) <= 1e-11 * np.max(np.abs(ref))


def test_reduced_closure_reproduces_the_mean_oracle():
    """The state solve's formulation on the CPU: right-hand side = minus the unclamped
    operator on the lifted boundary data, boundary rows zero, continuity part centred;
    the clamped operator solved on the zero-sum pressure subspace.  Equals the oracle's
    ``pressure="mean"`` closure."""
    d = diffuser()
    nx = ny = 6
    L = Lattice(d.width, d.height, nx, ny)
    o = FluidOracle(L, d, pressure="mean")
    o.set_penalization(0.1)
    rho = np.random.default_rng(5).uniform(0.0, 1.0, L.n_vertices)
    ub = emu.fluid_bc(nx, ny, d.width, d.height, d.flows)
    lift = np.zeros(o.n)
    lift[:o.nuv] = ub
    rhs = -emu.fluid_apply(nx, ny, d.width, d.height, 0.1, rho, lift)
    bc = np.zeros(o.n, bool)
    bc[o.bc_dofs] = True
    rhs[bc] = 0.0
    rhs[o.nuv:] -= rhs[o.nuv:].mean()
    A = np.stack([emu.fluid_apply(nx, ny, d.width, d.height, 0.1, rho, e, clamp=True) for e in np.eye(o.n)], axis=1)
    # the zero-sum pressure closure: border with the constant pressure vector
    c = np.zeros(o.n)
    c[o.nuv:] = 1.0
    Ab = np.block([[A, c[:, None]], [c[None, :], np.zeros((1, 1))]])
    x = np.linalg.solve(Ab, np.concatenate([rhs, [0.0]]))[:o.n]
    u = x[:o.nuv] + ub
    uo, po = o.state_solve(rho)
    assert np.max(np.abs(u - uo)) <= 1e-10 * np.max(np.abs(uo))
    assert np.max(np.abs(x[o.nuv:] - po)) <= 1e-9 * np.max(np.abs(po))


def _cheb(lmax, lo_frac=0.1):
    """Degree-2 Chebyshev coefficients of the smoothing steps on [lo_frac, 1.1] * lmax."""
    hi, lo = 1.1 * lmax, lo_frac * lmax
    th, de = 0.5 * (hi + lo), 0.5 * (hi - lo)
    sg = th / de
    r0 = 1 / sg
    r1 = 1 / (2 * sg - r0)
    return 1 / th, r1 * r0, 2 * r1 / de


class _VCycle:
    """One V-cycle of the scalar P1 hierarchy as the multigrid runs it (Chebyshev degree 2
    pre/post smoothing on coefficients coarsened level by level, the kernels' transfers,
    an exact coarsest solve), built from the emulated kernel phases."""

    def __init__(self, nx, ny, hx, hy, dirv, kK, kM):
        self.lv = emu.build_levels(False, nx, ny, hx, hy, dirv, 1)
        self.ops = []
        for l, L in enumerate(self.lv):
            if l > 0:
                F = self.lv[l - 1]
                kK = emu.coarsen_kappa(kK, F["nx"], F["ny"], L["nx"], L["ny"])
                kM = emu.coarsen_kappa(kM, F["nx"], F["ny"], L["nx"], L["ny"])
            n = L["NX"] * L["NY"]
            hl = (hx * nx / L["nx"], hy * ny / L["ny"])
            A = np.stack([emu.p1_apply(1, L["nx"], L["ny"], *hl, 0, 0, L["dir"], kK, kM, e) for e in np.eye(n)], 1)
            dinv = 1 / np.diag(A)
            v = np.random.default_rng(0).standard_normal(n)
            for _ in range(30):
                w = dinv * (A @ v)
                lm = np.linalg.norm(w) / np.linalg.norm(v)
                v = w / np.linalg.norm(w)
            last = l == len(self.lv) - 1
            self.ops.append(dict(A=A, dinv=dinv, c=_cheb(lm), lu=scipy.linalg.lu_factor(A) if last else None))

    def __call__(self, b, l=0):
        o = self.ops[l]
        if o["lu"] is not None:
            return scipy.linalg.lu_solve(o["lu"], b)
        A, Di, (c0, c1, c2) = o["A"], o["dinv"], o["c"]
        d0 = c0 * Di * b
        x = d0 + c1 * d0 + c2 * Di * (b - A @ d0)
        f, c = self.lv[l], self.lv[l + 1]
        rc = emu.restrict(1, f["NX"], f["NY"], f["dir"], c["NX"], c["NY"], c["dir"], b - A @ x)
        u = x + emu.prolong(1, f["NX"], f["NY"], f["dir"], c["NX"], c["NY"], c["dir"], self(rc, l + 1))
        r0 = b - A @ u
        dd = c0 * Di * r0
        return u + dd + c1 * dd + c2 * Di * (r0 - A @ dd)


def _fgmres(A, P, b, m=30, tol=1e-12, maxit=1000):
    """Flexible GMRES(m), right preconditioned, stopping on the true residual."""
    x = np.zeros_like(b)
    bn = np.linalg.norm(b)
    its = 0
    while True:
        r = b - A(x)
        beta = np.linalg.norm(r)
        if beta <= tol * bn or its >= maxit:
            return x, its, beta / bn
        V, Z = [r / beta], []
        H = np.zeros((m + 1, m))
        for j in range(m):
            Z.append(P(V[j]))
            w = A(Z[j])
            its += 1
            for _ in range(2):
                for i in range(j + 1):
                    h = V[i] @ w
                    H[i, j] += h
                    w = w - h * V[i]
            H[j + 1, j] = np.linalg.norm(w)
            V.append(w / H[j + 1, j])
            e1 = np.zeros(j + 2)
            e1[0] = beta
            y = np.linalg.lstsq(H[:j + 2, :j + 1], e1, rcond=None)[0]
            if np.linalg.norm(H[:j + 2, :j + 1] @ y - e1) <= 0.5 * tol * bn or its >= maxit:
                break
        x = x + np.stack(Z, 1) @ y


def test_block_preconditioned_solve_reaches_the_oracle_closure():
    """The state solve's algorithm run with the emulated kernel phases: right-hand side and
    clamped operator as the kernels compute them, the block-diagonal preconditioner (one
    V-cycle of K + alpha M per velocity component on the (2nx)x(2ny) lattice, lumped mass +
    one V-cycle of the 1/alpha-weighted Laplacian with a 1e-3 mass shift for the pressure),
    flexible GMRES(30).  Converges to the oracle's reduced-system closure on a 0/1 design
    (alpha from 2.5e-4 to 2.5e4) in a few hundred iterations at most."""
    d = diffuser()
    N, q = 8, 0.1
    L = Lattice(1.0, 1.0, N, N)
    o = FluidOracle(L, d, pressure="mean")
    o.set_penalization(q)
    X, Y = L.vertex_coords()
    rho = np.where(np.abs(Y - 0.5) < 0.5 - X / 3.0, 1.0, 0.0)
    nuv = o.nuv
    ub = emu.fluid_bc(N, N, 1.0, 1.0, d.flows)
    lift = np.zeros(o.n)
    lift[:nuv] = ub
    rhs = -emu.fluid_apply(N, N, 1.0, 1.0, q, rho, lift)
    bc = np.zeros(o.n, bool)
    bc[o.bc_dofs] = True
    rhs[bc] = 0.0
    rhs[nuv:] -= rhs[nuv:].mean()
    # preconditioner coefficients as the set-up kernels compute them
    R = rho.reshape(N + 1, N + 1)
    Rf = np.zeros((2 * N + 1, 2 * N + 1))
    Rf[0::2, 0::2] = R
    Rf[0::2, 1::2] = 0.5 * (R[:, :-1] + R[:, 1:])
    Rf[1::2, 0::2] = 0.5 * (R[:-1, :] + R[1:, :])
    Rf[1::2, 1::2] = 0.5 * (R[:-1, :-1] + R[1:, 1:])
    L2 = Lattice(1.0, 1.0, 2 * N, 2 * N)
    km = np.zeros(2 * (2 * N) ** 2)
    kk = np.zeros(2 * N * N)
    for t in (0, 1):
        km[t::2] = fluid_penalty(Rf.ravel()[L2.triangle_vertices(t)].mean(axis=1), q)
        kk[t::2] = 1.0 / fluid_penalty(rho[L.triangle_vertices(t)].mean(axis=1), q)
    vel = _VCycle(2 * N, 2 * N, 0.5 / N, 0.5 / N, emu.make_dir(2 * N, 2 * N, 0.5 / N, 0.5 / N,
                                                               ["Left", "Right", "Top", "Bottom"]), np.ones_like(km), km)
    pre = _VCycle(N, N, 1.0 / N, 1.0 / N, emu.no_dir(N + 1, N + 1), kk, np.full_like(kk, 1e-3))
    ml = emu.vertex_weights(N, N, 1.0 / N, 1.0 / N)
    nb = bc[0:nuv:2]

    def P(r):
        z = np.zeros_like(r)
        for c in (0, 1):
            z[c:nuv:2] = np.where(nb, 0.0, vel(np.where(nb, 0.0, r[c:nuv:2])))
        rp = r[nuv:]
        zp = rp / ml + pre(rp - rp.mean())
        z[nuv:] = zp - zp.mean()
        return z

    x, its, rel = _fgmres(lambda v: emu.fluid_apply(N, N, 1.0, 1.0, q, rho, v, clamp=True), P, rhs)
    assert rel <= 1e-12 and its <= 400
    u_ref, p_ref = o.state_solve(rho)
    assert np.max(np.abs(x[:nuv] + ub - u_ref)) <= 1e-10 * np.max(np.abs(u_ref))
    assert np.max(np.abs(x[nuv:] - p_ref)) <= 1e-9 * np.max(np.abs(p_ref))
