"""GPU path against the FP64 oracle through the C ABI (needs a CUDA device).

Tolerances: FP64-residual solves run to rtol 1e-12 here, so the displacement
matches the oracle's direct solve to ~1e-9 relative and the compliance to
~1e-10; mixed precision (FP32 CG inside FP64 refinement) reaches the same
refinement target.  The design-loop tests use the parity bar rel <= 1e-6 on
the compliance history.
"""
import numpy as np
import pytest

from oracle.fem import Design, FEMOracle, Lattice, OracleSolver

pytestmark = pytest.mark.gpu

GOLDEN = __import__("os").path.join(__import__("os").path.dirname(__file__), "golden")


def _design(**kw):
    base = dict(width=2.0, height=1.0, fem_step_size=0.002, penalties=[3.0], volume_fraction=0.5,
                fixed_sides=["Left"], body_force=None,
                tractions=[dict(side="Right", center=0.5, length=0.5, value=[0.0, -1.0])],
                filter_radius=0.05, young_modulus=1.0, poisson_ratio=0.3)
    base.update(kw)
    return Design(**base)


def _gpu_problem(d: Design, nx, ny, precision="mixed", rtol=1e-12):
    import topomax_gb300 as tg
    from topomax_gb300.designs import parse_design_dict
    dd = {"Elasticity": {"domain_parameters": dict(width=d.width, height=d.height, fem_step_size=d.fem_step_size,
                                                   dem_step_size=1.0, penalties=d.penalties,
                                                   volume_fraction=d.volume_fraction),
                         "problem_parameters": dict(fixed_sides=d.fixed_sides, body_force=d.body_force,
                                                    tractions=d.tractions, filter_radius=d.filter_radius,
                                                    young_modulus=d.young_modulus, poisson_ratio=d.poisson_ratio,
                                                    fixed_points=d.fixed_points)}}
    dom, par = parse_design_dict(dd)
    mesh = tg.RectangleMesh(d.width, d.height, nx, ny)
    V = tg.FunctionSpace(mesh, "CG", 1, dof_order="lattice")   # the oracle's vertex order
    return tg.ElasticityProblem(mesh, V, dom, par, precision=precision, rtol=rtol), V


@pytest.mark.parametrize("nx,ny,sides", [(10, 10, ["Bottom"]), (80, 40, ["Left"]), (33, 9, ["Left", "Right", "Top"])])
def test_operator_and_load_match_oracle(nx, ny, sides):
    import torch
    d = _design(fixed_sides=sides)
    prob, V = _gpu_problem(d, nx, ny)
    o = FEMOracle(Lattice(d.width, d.height, nx, ny), d)
    o.set_penalization(3.0)
    prob.set_penalization(3.0)
    rng = np.random.default_rng(0)
    xi = rng.uniform(0.01, 1.0, o.L.n_vertices)
    u = rng.standard_normal(2 * o.L.n_p2)
    y = prob.apply_operator(xi, torch.tensor(u, device="cuda")).cpu().numpy()
    ref = o.apply_state(xi, u)
    assert np.max(np.abs(y - ref)) <= 1e-12 * np.max(np.abs(ref))
    b = prob.load_vector().cpu().numpy()
    bref = o.load.copy()
    bref[np.concatenate([2 * o.dirichlet_nodes, 2 * o.dirichlet_nodes + 1])] = 0
    assert np.max(np.abs(b - bref)) <= 1e-14 * np.max(np.abs(bref))


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_filter_matches_oracle(precision):
    import topomax_gb300 as tg
    d = _design()
    nx, ny = 80, 40
    mesh = tg.RectangleMesh(2.0, 1.0, nx, ny)
    V = tg.FunctionSpace(mesh, "CG", 1, dof_order="lattice")
    f = tg.HelmholtzFilter(0.05, V, precision=precision, rtol=1e-12)
    o = FEMOracle(Lattice(2.0, 1.0, nx, ny), d)
    rho = np.random.default_rng(1).uniform(0, 1, o.L.n_vertices)
    xi = f.apply(rho).vector()[:]
    ref = o.filter_apply(rho)
    assert np.max(np.abs(xi - ref)) <= 1e-10 * np.max(np.abs(ref))


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_filter_identity_at_zero_radius(precision):
    """tests/test_filter.py:25-34: epsilon = 0 leaves rho unchanged."""
    import topomax_gb300 as tg
    mesh = tg.RectangleMesh(1.0, 1.0, 10, 10)
    V = tg.FunctionSpace(mesh, "CG", 1)
    f = tg.HelmholtzFilter(0.0, V, precision=precision, rtol=1e-14)
    np.random.seed(198)
    rho = np.random.random(V.dim())
    xi = f.apply(rho).vector()[:]
    assert np.max(np.abs(xi - rho)) < 1e-13


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
@pytest.mark.parametrize("case", ["cantilever", "triangle"])
def test_state_compliance_gradient_match_oracle(precision, case):
    if case == "cantilever":
        d, nx, ny = _design(), 80, 40
    else:
        d = _design(width=1.0, height=1.0, fixed_sides=["Bottom"], tractions=None, filter_radius=0.02,
                    young_modulus=2.5, poisson_ratio=0.25,
                    body_force=dict(region=dict(center=[0.5, 0.5], radius=0.05), value=[0.0, -10.0]))
        nx, ny = 40, 40
    prob, V = _gpu_problem(d, nx, ny, precision=precision, rtol=1e-11)
    o = FEMOracle(Lattice(d.width, d.height, nx, ny), d)
    prob.set_penalization(3.0)
    o.set_penalization(3.0)
    rho = np.random.default_rng(2).uniform(0.01, 1.0, o.L.n_vertices)
    C = prob.calculate_objective(rho)
    xi_ref = o.filter_apply(rho)
    u_ref = o.state_solve(xi_ref)
    C_ref = o.compliance(u_ref)
    assert abs(C - C_ref) <= 1e-9 * abs(C_ref)
    u = prob.u.vector()[:]
    assert np.max(np.abs(u - u_ref)) <= 1e-8 * np.max(np.abs(u_ref))
    g = prob.calculate_objective_gradient().vector()[:]
    g_ref = o.gradient(u_ref, xi_ref)
    tol = 1e-9 if precision == "fp64" else 2e-6
    assert np.max(np.abs(g - g_ref)) <= tol * np.max(np.abs(g_ref))


def test_projection_matches_oracle():
    import torch
    import topomax_gb300 as tg
    d = _design()
    solver_o = OracleSolver(40, d)
    rng = np.random.default_rng(4)
    half = rng.normal(0.0, 3.0, solver_o.lattice.n_vertices)
    ref = solver_o.project(half, solver_o.volume)
    from tests.test_gpu_parity import _write_design
    path = _write_design(d)
    s = tg.FEMSolver(40, path, verbose=False, save=False)
    psi = s.project(torch.as_tensor(half), s.volume).cpu().numpy()    # tensors: lattice order
    assert np.max(np.abs(psi - ref)) <= 1e-10
    assert abs(s.integrate(torch.sigmoid(torch.as_tensor(psi))) - s.volume) <= 1e-11
    # host arrays in the solver's (dolfin) dof order, as the reference's project takes them
    V = s.control_space
    psi_host = s.project(V.to_host_order(half), s.volume)
    assert isinstance(psi_host, np.ndarray)
    assert np.max(np.abs(V.from_host_order(psi_host) - ref)) <= 1e-10


def _write_design(d: Design, name="design.json"):
    import json
    import tempfile
    import os
    dd = {"Elasticity": {"domain_parameters": dict(width=d.width, height=d.height, fem_step_size=d.fem_step_size,
                                                   dem_step_size=1.0, penalties=d.penalties,
                                                   volume_fraction=d.volume_fraction),
                         "problem_parameters": dict(fixed_sides=d.fixed_sides, body_force=d.body_force,
                                                    tractions=d.tractions, filter_radius=d.filter_radius,
                                                    young_modulus=d.young_modulus, poisson_ratio=d.poisson_ratio)}}
    p = os.path.join(tempfile.mkdtemp(), name)
    with open(p, "w") as f:
        json.dump(dd, f)
    return p


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_triangle_known_answer(precision, tmp_path):
    """tests/test_elasticity_solver.py:30-55: triangle, N=10, objective at k=24."""
    import json
    import os
    import topomax_gb300 as tg
    gold = json.load(open(os.path.join(GOLDEN, "triangle_N10.json")))
    s = tg.FEMSolver(10, os.path.join(GOLDEN, "designs", "triangle.json"), data_path=str(tmp_path),
                     skip_multiple=999, precision=precision, rtol=1e-10, verbose=False)
    hist = s.solve()[3.0]
    assert hist["exit_condition"] == "Convergence treshold reached"
    assert hist["iterations"] == gold["iteration"]
    obj = hist["objectives"][-1]
    assert abs(obj - gold["objective"]) <= 1e-6 * abs(gold["objective"])
    rho = np.sort(s.to_array(s.rho))
    assert np.max(np.abs(rho - np.array(gold["rho_sorted"]))) <= 1e-5
    assert os.path.isfile(os.path.join(tmp_path, "FEM", "triangle", "data", "N=10_p=3.0_k=24.dat"))
    # the saved design is the reference's own file (FEM_src/utils.py:47-69): same keys, the
    # vector in dolfin's dof order, matching the reference's saved correct_rho.dat
    import pickle
    from topomax_gb300.fem import load_function
    path = os.path.join(tmp_path, "FEM", "triangle", "data", "N=10_p=3.0_k=24_rho.dat")
    with open(path, "rb") as f:
        rec = pickle.load(f)
    assert set(rec) == {"N", "domain_size", "problem", "vector"} and rec["N"] == 10
    assert np.max(np.abs(np.asarray(rec["vector"]) - np.array(gold["rho_dolfin"]))) <= 1e-5
    f, mesh, V = load_function(path)
    assert np.array_equal(f.vector()[:], s.to_array(s.rho))


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_cantilever_design_loop_parity(precision):
    """80x40 cantilever, 20 EMD iterations: compliance history rel <= 1e-6 vs the oracle."""
    import topomax_gb300 as tg
    d = _design()
    so = OracleSolver(40, d, max_iterations=20)
    ref = so.solve()[0]
    path = _write_design(d)
    s = tg.FEMSolver(40, path, precision=precision, rtol=1e-10, verbose=False, save=False, max_iterations=20)
    hist = s.solve()[3.0]
    objs = np.array(hist["objectives"])
    robjs = np.array(ref.objectives)
    assert len(objs) == len(robjs)
    assert np.max(np.abs(objs - robjs) / np.abs(robjs)) <= 1e-6
    assert np.max(np.abs(s.rho.tensor.cpu().numpy() - ref.rho)) <= 1e-5
    assert np.max(np.abs(s.to_array(s.rho) - s.control_space.to_host_order(ref.rho))) <= 1e-5


def test_call_order_errors():
    import topomax_gb300 as tg
    d = _design()
    prob, V = _gpu_problem(d, 8, 4)
    with pytest.raises(ValueError):
        prob.calculate_objective(np.full(V.dim(), 0.5))        # no penalisation set
    prob.set_penalization(3.0)
    with pytest.raises(ValueError):
        prob.calculate_objective_gradient()                    # before calculate_objective
    assert np.isnan(prob.calculate_objective(np.full(V.dim(), np.nan)))


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_large_grid_properties(precision):
    """1000x500 (4,006,002 dofs): residual, symmetry and energy identities."""
    import torch
    d = _design()
    prob, V = _gpu_problem(d, 1000, 500, precision=precision, rtol=1e-8)
    prob.set_penalization(3.0)
    g = torch.Generator().manual_seed(0)
    rho = torch.rand(V.dim(), generator=g, dtype=torch.float64) * 0.99 + 0.01
    C = prob.calculate_objective(rho.numpy())
    u = prob.u.tensor
    xi = prob.filtered_rho.tensor
    b = prob.load_vector()
    r = b - prob.apply_operator(xi, u)
    assert (r.norm() / b.norm()).item() <= 1e-8
    assert abs(C - torch.dot(b, u).item()) <= 1e-12 * abs(C)
    Ku = prob.apply_operator(xi, u)
    assert abs(torch.dot(u, Ku).item() - C) <= 1e-7 * abs(C)
    v = torch.randn(u.numel(), generator=g, dtype=torch.float64).cuda()
    lhs = torch.dot(v, Ku).item()
    rhs = torch.dot(u, prob.apply_operator(xi, v)).item()
    assert abs(lhs - rhs) <= 1e-12 * (v.norm() * Ku.norm()).item()
    assert prob.filtered_rho.tensor.min().item() > 0.0


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_tail_matches_level_kernels(precision, monkeypatch):
    """The one-CTA coarse tail (all vectors and stencils in shared memory) runs
    the same per-node steps as the per-level kernels: the solves agree to
    rounding of the final refinement and take the same number of iterations."""
    import torch
    from topomax_gb300 import fem as F
    d = _design()
    results = []
    for tail in ("1", "0"):
        monkeypatch.setenv("TOPO_TAIL", tail)
        prob, V = _gpu_problem(d, 200, 100, precision=precision, rtol=1e-10)
        prob.set_penalization(3.0)
        g = torch.Generator().manual_seed(3)
        xi = F.Function(V, (torch.rand(V.dim(), generator=g, dtype=torch.float64) * 0.99 + 0.01).cuda())
        u = prob.forward(xi)
        results.append((prob.stats["state_iterations"], u.tensor.cpu().numpy()))
        del prob
    assert results[0][0] == results[1][0], [r[0] for r in results]
    ref = results[1][1]
    assert np.max(np.abs(results[0][1] - ref)) <= 1e-13 * np.max(np.abs(ref))


def test_pair_fp32_residual_operator_matches_fp64(monkeypatch):
    """Mixed precision computes its refinement residuals b - K u with the pair-of-FP32
    operator (FP32-pipe arithmetic, differences of the FP64 operand taken in FP64);
    TOPO_RESIDUAL_FP64=1 selects the FP64 operator.  On a high-contrast design both
    reach the true FP64 residual the solve asks for (1e-10, checked with the FP64
    operator) and their solutions agree to that tolerance."""
    import torch
    from topomax_gb300 import fem as F
    d = _design()
    results = []
    for flag in ("0", "1"):
        monkeypatch.setenv("TOPO_RESIDUAL_FP64", flag)
        prob, V = _gpu_problem(d, 200, 100, rtol=1e-10)
        prob.set_penalization(3.0)
        g = torch.Generator().manual_seed(5)
        xi = F.Function(V, (torch.rand(V.dim(), generator=g, dtype=torch.float64) * 0.99 + 0.01).cuda())
        u = prob.forward(xi).tensor.clone()
        b = prob.load_vector()
        r = b - prob.apply_operator(xi.tensor, u)
        assert (r.norm() / b.norm()).item() <= 1e-10
        results.append(u.cpu().numpy())
        del prob
    assert np.linalg.norm(results[0] - results[1]) <= 1e-9 * np.linalg.norm(results[1])


def test_contexts_of_different_sizes_interleave():
    """Kernel attributes are process-wide: a context created later (here a smaller
    mesh) must not break the launches of an earlier one."""
    import torch
    from topomax_gb300 import fem as F
    d = _design()
    big, Vb = _gpu_problem(d, 120, 60, rtol=1e-8)
    small, Vs = _gpu_problem(d, 40, 20, rtol=1e-8)
    for prob, V in ((big, Vb), (small, Vs), (big, Vb)):
        prob.set_penalization(3.0)
        xi = F.Function(V, torch.full((V.dim(),), 0.5, dtype=torch.float64, device="cuda"))
        c = prob.calculate_objective(xi)
        assert np.isfinite(c) and c > 0


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_reference_design_vector_at_the_api(precision):
    """The reference's saved triangle design (tests/test_data/FEM/triangle/data/correct_rho.dat,
    dolfin's CG1 dof order) goes straight into calculate_objective on a default CG1 space
    and gives the objective the reference saved beside it; read in lattice order the same
    numbers are a different design."""
    import json
    import os
    import topomax_gb300 as tg
    gold = json.load(open(os.path.join(GOLDEN, "triangle_N10.json")))
    dom, par = tg.parse_design(os.path.join(GOLDEN, "designs", "triangle.json"))
    mesh = tg.RectangleMesh(1.0, 1.0, 10, 10)
    results = {}
    for order in ("dolfin", "lattice"):
        V = tg.FunctionSpace(mesh, "CG", 1, dof_order=order)
        prob = tg.ElasticityProblem(mesh, V, dom, par, precision=precision, rtol=1e-11)
        prob.set_penalization(gold["penalty"])
        results[order] = prob.calculate_objective(np.array(gold["rho_dolfin"]))
        if order == "dolfin":
            xi = prob.filtered_rho.vector()[:]             # host view: dolfin order again
            assert np.max(np.abs(xi - prob.filter.apply(np.array(gold["rho_dolfin"])).vector()[:])) == 0
    assert abs(results["dolfin"] - gold["objective"]) <= 1e-6 * gold["objective"]
    assert abs(results["lattice"] - gold["objective"]) > 1e-3 * gold["objective"]


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_filter_manufactured_solution_converges(precision):
    """tests/test_filter.py:37-60 on the GPU filter: rho = (8 eps^2 pi^2 + 1) cos(2 pi x)
    cos(2 pi y) interpolated on the unit square with eps = e / pi filters to cos(2 pi x)
    cos(2 pi y); the L2 error (12-point rule per triangle, the exact solution evaluated at
    the quadrature points) over N = 10, 20, ..., 90 passes the reference's own test:
    tests/utils.py get_convergance returns Polynomial.fit(log N, log error, 1).coef[1],
    the slope in the fit's scaled window ([log 10, log 90] -> [-1, 1], a factor 1.0986),
    and requires it <= -2.  The unscaled slope is also checked (<= -1.9; the oracle's is
    -1.96).  At N = 40 the filtered field equals the oracle's."""
    import topomax_gb300 as tg
    from oracle.fem import rule_degree6
    eps = np.e / np.pi
    lam, w = rule_degree6()
    errs = []
    Ns = list(range(10, 91, 10))
    for N in Ns:
        L = Lattice(1.0, 1.0, N, N)
        X, Y = L.vertex_coords()
        rho = (8 * eps * eps * np.pi ** 2 + 1) * np.cos(2 * np.pi * X) * np.cos(2 * np.pi * Y)
        V = tg.FunctionSpace(tg.RectangleMesh(1.0, 1.0, N, N), "CG", 1, dof_order="lattice")
        xi = tg.HelmholtzFilter(eps, V, precision=precision, rtol=1e-12).apply(rho).vector()[:]
        e2 = 0.0
        for o in (0, 1):
            tv = L.triangle_vertices(o)
            area, _ = L.triangle_geometry(o)
            xq = lam @ X[tv].T                       # (12, T) quadrature points
            yq = lam @ Y[tv].T
            diff = lam @ xi[tv].T - np.cos(2 * np.pi * xq) * np.cos(2 * np.pi * yq)
            e2 += area * float(w @ (diff ** 2).sum(axis=1))
        errs.append(np.sqrt(e2))
        if N == 40:
            ref = FEMOracle(L, _design(width=1.0, height=1.0, filter_radius=eps)).filter_apply(rho)
            assert np.max(np.abs(xi - ref)) <= 1e-10 * np.max(np.abs(ref))
    fit = np.polynomial.Polynomial.fit(np.log(Ns), np.log(errs), 1)
    assert fit.coef[1] <= -2
    assert fit.convert().coef[1] <= -1.9


def test_kernel_clock_times_host_driven_launches(monkeypatch):
    """The kernel clock (topo_kernel_clock / topo_kernel_clock_report) times host-driven
    launches only: a state solve of a context created with TOPO_GRAPHS=0 is itemised per
    family with its algorithmic bytes (the P2 Apply launch moves 2 * dofs + vertices FP32
    values), a context whose solves are recorded as graphs adds no P2 smoothing launches,
    and the clock off records nothing."""
    import ctypes
    import torch
    from topomax_gb300 import _capi
    from topomax_gb300 import fem as F
    lib = _capi.load_library()

    def report():
        need = lib.topo_kernel_clock_report(None, 0)
        buf = ctypes.create_string_buffer(int(need))
        assert lib.topo_kernel_clock_report(buf, need) == need
        rows = {}
        for line in buf.value.decode().splitlines():
            fam, level, n, ms, nbytes = line.split("\t")
            rows[(fam, int(level))] = (int(n), float(ms), float(nbytes))
        return rows

    d = _design()
    nx, ny = 120, 60
    xi = torch.full(((nx + 1) * (ny + 1),), 0.5, dtype=torch.float64, device="cuda")
    monkeypatch.setenv("TOPO_GRAPHS", "0")
    prob, V = _gpu_problem(d, nx, ny, rtol=1e-8)
    prob.set_penalization(3.0)
    lib.topo_kernel_clock(1)
    prob.forward(F.Function(V, xi))
    lib.topo_kernel_clock(0)
    rows = report()
    n, ms, nbytes = rows[("P2 march FP32 Apply", 0)]
    assert n >= 1 and ms > 0
    assert nbytes / n == (2 * 2 * (2 * nx + 1) * (2 * ny + 1) + (nx + 1) * (ny + 1)) * 4
    assert ("P2 march FP32 Post2", 0) in rows and ("restriction", 0) in rows
    # graph-recorded solves: the V-cycle launches run inside graphs and are not timed
    monkeypatch.setenv("TOPO_GRAPHS", "1")
    prob2, V2 = _gpu_problem(d, nx, ny, rtol=1e-8)
    prob2.set_penalization(3.0)
    prob2.forward(F.Function(V2, xi))          # records the graphs
    lib.topo_kernel_clock(1)
    prob2.forward(F.Function(V2, xi))
    lib.topo_kernel_clock(0)
    assert ("P2 march FP32 Post2", 0) not in report()
    lib.topo_kernel_clock(1)                   # clears the totals
    lib.topo_kernel_clock(0)
    prob.forward(F.Function(V, xi))            # host-driven, clock off
    assert report() == {}


def test_design_loop_parity_at_320x160():
    """The cantilever at 320x160 (411,522 dofs, the largest grid the oracle's sparse LU
    runs in seconds): two design iterations of the mixed-precision loop against the
    oracle's loop, compliance history rel <= 1e-6 and the final design to 1e-5."""
    import topomax_gb300 as tg
    d = _design()
    so = OracleSolver(160, d, max_iterations=2)
    ref = so.solve()[0]
    s = tg.FEMSolver(160, _write_design(d), precision="mixed", rtol=1e-10, verbose=False, save=False,
                     max_iterations=2)
    hist = s.solve()[3.0]
    objs, robjs = np.array(hist["objectives"]), np.array(ref.objectives)
    assert len(objs) == len(robjs) == 3
    assert np.max(np.abs(objs - robjs) / np.abs(robjs)) <= 1e-6
    assert np.max(np.abs(s.rho.tensor.cpu().numpy() - ref.rho)) <= 1e-5


def test_state_warm_start_extrapolation():
    """topo_state_warm_start: u = sum_i (-1)^i binom(count, i + 1) h_i in one pass (count 1
    copies h_0); a history longer than five or a null entry is refused."""
    import ctypes
    import math
    import torch
    from topomax_gb300 import _capi
    prob, V = _gpu_problem(_design(), 40, 20)
    ctx = prob._ctx
    n = int(prob.solution_space.dim())
    gen = torch.Generator(device="cuda").manual_seed(7)
    hist = [torch.rand(n, dtype=torch.float64, device="cuda", generator=gen) for _ in range(6)]
    u = torch.empty(n, dtype=torch.float64, device="cuda")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for count in range(1, 6):
        ptrs = (ctypes.c_void_p * count)(*[h.data_ptr() for h in hist[:count]])
        ctx.check(ctx._lib.topo_state_warm_start(ctx.ptr, ptrs, count, ctypes.c_void_p(u.data_ptr()), stream))
        ref = sum((-1) ** i * math.comb(count, i + 1) * hist[i] for i in range(count))
        assert torch.max(torch.abs(u - ref)).item() <= 1e-14 * 2 ** count
    ptrs = (ctypes.c_void_p * 6)(*[h.data_ptr() for h in hist])
    assert ctx._lib.topo_state_warm_start(ctx.ptr, ptrs, 6, ctypes.c_void_p(u.data_ptr()), stream) == _capi.TOPO_ERR_ARG
    ptrs = (ctypes.c_void_p * 2)(hist[0].data_ptr(), None)
    assert ctx._lib.topo_state_warm_start(ctx.ptr, ptrs, 2, ctypes.c_void_p(u.data_ptr()), stream) == _capi.TOPO_ERR_ARG
