"""DEM energy kernels (csrc/topo_dem.cu) against the reference's outputs and the oracle.

Parity bars: the per-cell values of calculate_objective_and_gradient are
rounded exactly as the reference's float32 expressions round them, so the
known answers of tests/test_DEM_problem.py:14-43 are matched to the
reference's own bar (1e-14); sums over cells run in FP64 here (rel 1e-6 of the
reference's float32 torch.sum); the energy gradients (hand-written backward
kernels, FP32 with FMA) match the reference's torch autograd to 1e-4 of the
largest entry.
"""
import json
import os

import numpy as np
import pytest

from oracle import dem as O

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _t(a):
    import torch
    return torch.tensor(np.asarray(a), dtype=torch.float32, device="cuda")


@pytest.mark.parametrize("design,N", [("short_cantilever", 45), ("bridge", 30)])
def test_objective_and_gradient_known_answer(design, N):
    from topomax_gb300 import dem
    gold = np.load(os.path.join(GOLDEN, f"dem_{design}.npz"))
    d = json.load(open(os.path.join(GOLDEN, "designs", f"{design}.json")))["Elasticity"]
    dp, pp = d["domain_parameters"], d["problem_parameters"]
    W, H = dp["width"], dp["height"]
    n = int(N / min(W, H))
    mesh = dem.Mesh(int(W * n), int(H * n), W, H)
    se = dem.StrainEnergy(mesh, None, pp["young_modulus"], pp["poisson_ratio"], None)
    se.set_penalization(dp["penalties"][-1])
    x = np.array([mesh.x_grid.T.ravel(), mesh.y_grid.T.ravel()]).T.astype(np.float32)
    rho = np.full(mesh.intervals, dp["volume_fraction"], dtype=np.float32)
    obj, grad = se.calculate_objective_and_gradient(_t(x), mesh.shape, _t(rho))
    assert abs(float(obj) - float(gold["objective"])) <= 1e-6 * abs(float(gold["objective"]))
    g = grad.cpu().numpy()
    assert g.shape == gold["gradient"].shape
    assert np.max(np.abs(g - gold["gradient"])) < 1e-14


def _case(k):
    from tests.test_dem_oracle import _case as cpu_case
    return cpu_case(k)


@pytest.mark.parametrize("k", [0, 1, 2])
def test_energy_and_autograd_match_reference(k):
    import torch
    from topomax_gb300 import dem
    g, mesh, (Nx, Ny, W, H, young, nu, p), _, body, tps = _case(k)
    se = dem.StrainEnergy(mesh, body, young, nu, tps)
    se.set_penalization(p)
    u = _t(g[f"case{k}_u"]).requires_grad_(True)
    rho = _t(g[f"case{k}_rho"]).requires_grad_(True)
    e = se.calculate_energy(u, mesh.shape, rho)
    gu, gr = torch.autograd.grad(e, (u, rho))
    ref = float(g[f"case{k}_energy"])
    assert abs(float(e) - ref) <= 1e-5 * abs(ref)
    for got, want in ((gu, g[f"case{k}_grad_u"]), (gr, g[f"case{k}_grad_rho"])):
        got = got.cpu().numpy()
        assert np.max(np.abs(got - want)) <= 1e-4 * np.max(np.abs(want))
    obj, grad = se.calculate_objective_and_gradient(u.detach(), mesh.shape, rho.detach())
    assert abs(float(obj) - float(g[f"case{k}_objective"])) <= 1e-6 * abs(float(obj))
    want = g[f"case{k}_gradient"]
    assert np.max(np.abs(grad.cpu().numpy() - want)) <= 1e-6 * np.max(np.abs(want))


def test_energy_at_600x300_matches_oracle():
    """The DEM measurement workload: 600 x 300 cells, rho ~ U(0.01, 1), p = 3."""
    import torch
    from topomax_gb300 import dem
    from topomax_gb300.designs import Side, Traction
    Nx, Ny, W, H = 600, 300, 2.0, 1.0
    mesh = dem.Mesh(Nx, Ny, W, H)
    tps = [dem.TractionPoints(mesh, Traction(Side.RIGHT, 0.5, 0.5, (0.0, -1.0)))]
    se = dem.StrainEnergy(mesh, None, 1.0, 0.3, tps)
    se.set_penalization(3.0)
    gen = torch.Generator().manual_seed(4)
    rho = (torch.rand((Ny, Nx), generator=gen) * 0.99 + 0.01).float()
    u = (torch.randn(((Nx + 1) * (Ny + 1), 2), generator=gen) * 1e-2).float()
    ug, rg = u.cuda().requires_grad_(True), rho.cuda().requires_grad_(True)
    e = se.calculate_energy(ug, mesh.shape, rg)
    gu, gr = torch.autograd.grad(e, (ug, rg))
    wext = dem.external_weights(mesh, None, tps)
    psi, ogu, ogr = O.energy(u.numpy(), rho.numpy(), Nx, Ny, W, H, 1.0, 0.3, 3.0, wext)
    assert abs(float(e) - psi) <= 1e-5 * abs(psi)
    assert np.max(np.abs(gu.cpu().numpy() - ogu)) <= 1e-4 * np.max(np.abs(ogu))
    assert np.max(np.abs(gr.cpu().numpy() - ogr)) <= 1e-5 * np.max(np.abs(ogr))


def test_enforcer_and_fused_energy():
    import torch
    from topomax_gb300 import dem
    from topomax_gb300.designs import ElasticityParameters, Side, Traction
    Nx, Ny = 48, 20
    mesh = dem.Mesh(Nx, Ny, 2.0, 1.0)
    params = ElasticityParameters(fixed_sides=[Side.LEFT, Side.BOTTOM], body_force=None, tractions=None,
                                  filter_radius=0.05, young_modulus=1.0, poisson_ratio=0.3)
    enf = dem.ElasticityEnforcer(params, mesh, "cuda")
    gen = torch.Generator().manual_seed(7)
    uh = (torch.randn(((Nx + 1) * (Ny + 1), 2), generator=gen) * 1e-2).float().cuda()
    u = enf(uh)
    assert torch.equal(u, uh * enf.zero_enforcer)
    tps = [dem.TractionPoints(mesh, Traction(Side.RIGHT, 0.5, 0.5, (0.0, -1.0)))]
    se = dem.StrainEnergy(mesh, None, 1.0, 0.3, tps)
    se.set_penalization(3.0)
    rho = (torch.rand((Ny, Nx), generator=gen) * 0.99 + 0.01).float().cuda()
    a = uh.clone().requires_grad_(True)
    e1 = se.calculate_energy(enf(a), mesh.shape, rho)
    (g1,) = torch.autograd.grad(e1, (a,))
    b = uh.clone().requires_grad_(True)
    e2 = se.calculate_energy_enforced(b, enf, rho)
    (g2,) = torch.autograd.grad(e2, (b,))
    assert float(e1) == float(e2)
    assert torch.allclose(g1, g2, rtol=1e-5, atol=1e-7 * float(g1.abs().max()))


def test_network_energy_trains():
    """The DEM training objective: energy(enforcer(net(x))) with gradients reaching the
    network's parameters (the network itself is torch, as in the reference)."""
    import torch
    from topomax_gb300 import dem
    from topomax_gb300.designs import ElasticityParameters, Side, Traction
    torch.manual_seed(2022)
    Nx, Ny = 60, 30
    mesh = dem.Mesh(Nx, Ny, 2.0, 1.0)
    params = ElasticityParameters(fixed_sides=[Side.LEFT], body_force=None, tractions=None, filter_radius=0.05,
                                  young_modulus=1.0, poisson_ratio=0.3)
    enf = dem.ElasticityEnforcer(params, mesh, "cuda")
    tps = [dem.TractionPoints(mesh, Traction(Side.RIGHT, 0.5, 0.5, (0.0, -1.0)))]
    se = dem.StrainEnergy(mesh, None, 1.0, 0.3, tps)
    se.set_penalization(3.0)
    net = dem.MultiLayerNet(2, 2).cuda()
    x = torch.tensor(np.array([mesh.x_grid.T.ravel(), mesh.y_grid.T.ravel()]).T, dtype=torch.float32, device="cuda")
    rho = torch.full(mesh.intervals, 0.5, device="cuda")
    opt = torch.optim.Adam(net.parameters(), lr=1e-3)
    losses = []
    for _ in range(20):
        opt.zero_grad()
        loss = se.calculate_energy(enf(net(x)), mesh.shape, rho)
        loss.backward()
        opt.step()
        losses.append(float(loss))
    assert all(np.isfinite(losses))
    assert losses[-1] < losses[0]


def test_density_filter_matches_reference_bitwise():
    """create_density_filter on the GPU: W @ rho and W.T @ g equal the reference's scipy
    products bit for bit, and the stored-entry count matches (DEM_src/filter.py:8-31)."""
    from topomax_gb300 import dem
    d = np.load(os.path.join(GOLDEN, "dem_density_filter.npz"))
    k = 0
    while f"filter{k}_meta" in d:
        Nx, Ny, W, H, r = d[f"filter{k}_meta"]
        mesh = dem.Mesh(int(Nx), int(Ny), W, H)
        F = dem.create_density_filter(r, mesh)
        assert F.nnz == int(d[f"filter{k}_nnz"]), k
        assert np.array_equal(F @ d[f"filter{k}_rho"].flatten(), d[f"filter{k}_apply"]), k
        assert np.array_equal(F.T @ d[f"filter{k}_g"], d[f"filter{k}_transpose"]), k
        k += 1
    assert k == 5


def test_density_filter_at_600x300():
    """The 600x300 DEM workload's filter (radius 0.05 over 180,000 elements): against the
    oracle on sampled rows, and W.T consistent with W (x . W y == W^T x . y)."""
    import torch
    from topomax_gb300 import dem
    Nx, Ny, W, H, r = 600, 300, 2.0, 1.0, 0.05
    mesh = dem.Mesh(Nx, Ny, W, H)
    F = dem.create_density_filter(r, mesh)
    g = torch.Generator().manual_seed(6)
    x = torch.rand(Nx * Ny, generator=g, dtype=torch.float64).cuda()
    y = torch.rand(Nx * Ny, generator=g, dtype=torch.float64).cuda()
    Wy = F @ y
    WTx = F.T @ x
    lhs, rhs = float(x @ Wy), float(WTx @ y)
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)
    # a filter of a constant is the constant (rows sum to one)
    one = F @ torch.ones(Nx * Ny, dtype=torch.float64, device="cuda")
    assert float((one - 1).abs().max()) <= 1e-14


def test_dem_training_step_and_problem():
    """The DEM problem of DEM_src/elasisity_problem.py:131-216 end to end on a 40x20
    cantilever: filter (W of DEM_src/filter.py), L-BFGS training of the network on the
    fused enforcer + energy kernels (DEM_src/deep_energy_method.py:55-105), objective and
    gradient mapped back through W^T.  The trained network's energy equals the FP64
    oracle's energy of the same displacement; the training lowered it."""
    import torch
    from topomax_gb300 import dem
    from topomax_gb300.designs import parse_design_dict
    dd = {"Elasticity": {
        "domain_parameters": dict(width=2.0, height=1.0, fem_step_size=0.002, dem_step_size=0.002,
                                  penalties=[3.0], volume_fraction=0.5),
        "problem_parameters": dict(fixed_sides=["Left"], body_force=None,
                                   tractions=[dict(side="Right", center=0.5, length=0.5, value=[0.0, -1.0])],
                                   filter_radius=0.05, young_modulus=1.0, poisson_ratio=0.3)}}
    _, par = parse_design_dict(dd)
    Nx, Ny = 40, 20
    mesh = dem.Mesh(Nx, Ny, 2.0, 1.0)
    torch.manual_seed(2022)
    prob = dem.ElasticityProblem(mesh, "cuda", False, par)
    prob.set_penalization(3.0)
    prob.dem.nn_parameters.iteration_count = 4
    with pytest.raises(ValueError):
        prob.calculate_objective_gradient()
    rho = np.random.default_rng(4).uniform(0.3, 1.0, (Ny, Nx))
    C = prob.calculate_objective(rho)
    g = prob.calculate_objective_gradient()
    assert np.isfinite(C) and C > 0
    assert g.shape == rho.shape and np.all(np.isfinite(g))
    losses = prob.dem.loss_array
    assert len(losses) >= 4 and min(losses) < losses[0]
    # energy at the trained network: kernel vs FP64 oracle on the same displacement
    filtered = prob.filter @ rho.flatten()
    u = prob.dem.get_u(mesh=mesh).detach().double().cpu().numpy()
    tr = [dem.TractionPoints(mesh, t) for t in par.tractions]
    wext = dem.external_weights(mesh, None, tr)
    psi_ref = O.energy(u, filtered, Nx, Ny, 2.0, 1.0, 1.0, 0.3, 3.0, wext)[0]
    psi = prob.dem.get_loss(filtered, mesh)
    assert abs(psi - psi_ref) <= 1e-4 * abs(psi_ref)
    # the objective's gradient is W^T of the per-cell gradient at the trained displacement
    obj, cell_g = prob.dem.objective_calculator.calculate_objective_and_gradient(
        prob.dem.get_u(mesh=mesh), mesh.shape, torch.as_tensor(filtered).float().reshape(mesh.intervals).cuda())
    g_ref = (prob.filter.T @ cell_g.detach().double().cpu().numpy().flatten()).reshape(rho.shape)
    assert np.array_equal(g, g_ref)
