"""DEM energy path on the CPU: the FP64 oracle and the host-side restatements
(load domains, external-work weights, Dirichlet mask) against the reference's
own outputs.

``tests/golden/dem_energy.npz`` holds outputs of the reference's StrainEnergy,
ElasticityEnforcer, CircleDomain and boundary_integral (generated by
``tests/golden/make_dem_golden.py``); ``dem_{short_cantilever,bridge}.npz`` are
the known answers of ``tests/test_DEM_problem.py:14-43`` (u = node
coordinates, rho = the volume fraction, p = 3).  The reference computes in
float32, so the FP64 oracle agrees to float32 rounding.
"""
import os

import numpy as np
import pytest

from oracle import dem as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _g():
    return np.load(os.path.join(GOLDEN, "dem_energy.npz"))


def _case(k):
    from topomax_gb300 import dem
    from topomax_gb300.designs import CircularRegion, Force, Side, Traction
    g = _g()
    Nx, Ny, W, H, p, young, nu = g[f"case{k}_meta"]
    Nx, Ny = int(Nx), int(Ny)
    mesh = dem.Mesh(Nx, Ny, W, H)
    t = g[f"case{k}_traction"]
    tps = [dem.TractionPoints(mesh, Traction(Side(int(t[0])), t[1], t[2], (t[3], t[4])))]
    b = g[f"case{k}_body"]
    body = dem.BodyForce(mesh, Force(CircularRegion((b[0], b[1]), b[2]), (b[3], b[4]))) if b.size else None
    wext = dem.external_weights(mesh, body, tps)
    return g, mesh, (Nx, Ny, W, H, young, nu, p), wext, body, tps


@pytest.mark.parametrize("k", [0, 1, 2])
def test_oracle_energy_and_gradients_match_reference(k):
    g, mesh, (Nx, Ny, W, H, young, nu, p), wext, _, _ = _case(k)
    u, rho = g[f"case{k}_u"], g[f"case{k}_rho"]
    psi, gu, gr = O.energy(u, rho, Nx, Ny, W, H, young, nu, p, wext)
    ref = float(g[f"case{k}_energy"])
    assert abs(psi - ref) <= 2e-5 * abs(ref)
    for got, want in ((gu, g[f"case{k}_grad_u"]), (gr, g[f"case{k}_grad_rho"])):
        assert np.max(np.abs(got - want)) <= 1e-4 * np.max(np.abs(want))
    obj, grad = O.objective_and_gradient(u, rho, Nx, Ny, W, H, young, nu, p)
    assert abs(obj - float(g[f"case{k}_objective"])) <= 2e-5 * abs(obj)
    assert np.max(np.abs(grad - g[f"case{k}_gradient"])) <= 1e-5 * np.max(np.abs(grad))


@pytest.mark.parametrize("design,N", [("short_cantilever", 45), ("bridge", 30)])
def test_oracle_matches_reference_known_answer(design, N):
    """tests/test_DEM_problem.py:14-43: u = node coordinates, rho = volume fraction, p = 3."""
    import json
    from topomax_gb300 import dem
    gold = np.load(os.path.join(GOLDEN, f"dem_{design}.npz"))
    d = json.load(open(os.path.join(GOLDEN, "designs", f"{design}.json")))["Elasticity"]
    dp, pp = d["domain_parameters"], d["problem_parameters"]
    W, H = dp["width"], dp["height"]
    n = int(N / min(W, H))
    mesh = dem.Mesh(int(W * n), int(H * n), W, H)
    x = np.array([mesh.x_grid.T.ravel(), mesh.y_grid.T.ravel()]).T.astype(np.float32)
    rho = np.full(mesh.intervals, dp["volume_fraction"], dtype=np.float32)
    obj, grad = O.objective_and_gradient(x, rho, mesh.Nx, mesh.Ny, W, H, pp["young_modulus"],
                                         pp["poisson_ratio"], dp["penalties"][-1])
    # u = x makes grad u the identity, which the reference's float32 sums of
    # coordinate * shape-derivative products reproduce only to ~1e-5 (cancellation)
    assert abs(obj - float(gold["objective"])) <= 2e-5 * abs(obj)
    assert grad.shape == gold["gradient"].shape
    assert np.max(np.abs(grad - gold["gradient"])) <= 2e-5 * np.max(np.abs(grad))


@pytest.mark.parametrize("k", [0, 1, 2, 3])
def test_circle_domain_matches_reference(k):
    from topomax_gb300 import dem
    from topomax_gb300.designs import CircularRegion
    g = _g()
    Nx, Ny, W, H, cx, cy, r = g[f"circle{k}_meta"]
    mesh = dem.Mesh(int(Nx), int(Ny), W, H)
    cd = dem.CircleDomain(mesh, CircularRegion((cx, cy), r))
    assert np.array_equal(cd.indices, g[f"circle{k}_indices"])
    assert np.array_equal(cd.areas, g[f"circle{k}_areas"])


@pytest.mark.parametrize("k", [0, 1, 2, 3])
def test_side_domain_weights_match_reference(k):
    from topomax_gb300 import dem
    from topomax_gb300.designs import Side
    g = _g()
    Nx, Ny, W, H, side, center, length = g[f"side{k}_meta"]
    mesh = dem.Mesh(int(Nx), int(Ny), W, H)
    w = dem.SideDomain(mesh, Side(int(side)), center, length).weights(mesh)
    ref = g[f"side{k}_weights"]
    assert np.max(np.abs(w - ref)) <= 1e-15 * np.max(np.abs(ref))


@pytest.mark.parametrize("k", [0, 1, 2])
def test_enforcer_mask_matches_reference(k):
    from topomax_gb300 import dem
    from topomax_gb300.designs import ElasticityParameters, Side
    g = _g()
    Nx, Ny, W, H = g[f"mask{k}_meta"]
    mesh = dem.Mesh(int(Nx), int(Ny), W, H)
    params = ElasticityParameters(fixed_sides=[Side(int(s)) for s in g[f"mask{k}_sides"]], body_force=None,
                                  tractions=None, filter_radius=0.05, young_modulus=1.0, poisson_ratio=0.3)
    enf = dem.ElasticityEnforcer(params, mesh, "cpu")  # building the mask needs no GPU
    assert np.array_equal(enf.mask_host, g[f"mask{k}"])


def test_quadrature_constants_match_reference_table():
    D = O.shape_table(0.1, 0.05)
    # columns of the reference table times Jinv = diag(2/dx, 2/dy)
    assert np.allclose(D[0, 0], [-0.394337567 * 20, -0.394337567 * 40])
    assert np.allclose(D[3, 3], [0.105662433 * 20, 0.394337567 * 40])
    # partition of unity: the derivatives of the four shape functions sum to zero
    assert np.max(np.abs(D.sum(axis=0))) < 1e-12


def test_density_filter_oracle_matches_reference_bitwise():
    """The oracle's restatement of create_density_filter (DEM_src/filter.py:8-31) applied
    as W @ rho and W.T @ g equals the reference's scipy products bit for bit (fixtures
    written by tests/golden/make_dem_golden.py filter)."""
    d = np.load(os.path.join(GOLDEN, "dem_density_filter.npz"))
    k = 0
    while f"filter{k}_meta" in d:
        Nx, Ny, W, H, r = d[f"filter{k}_meta"]
        Nx, Ny = int(Nx), int(Ny)
        a = O.density_filter_apply(Nx, Ny, W, H, r, d[f"filter{k}_rho"])
        t = O.density_filter_apply(Nx, Ny, W, H, r, d[f"filter{k}_g"], transpose=True)
        assert np.array_equal(a, d[f"filter{k}_apply"]), k
        assert np.array_equal(t, d[f"filter{k}_transpose"]), k
        nnz = sum(len(nb) for nb, _, _ in O.density_filter_rows(Nx, Ny, W, H, r))
        assert nnz == int(d[f"filter{k}_nnz"]), k
        k += 1
    assert k == 5
