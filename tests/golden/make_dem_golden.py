"""Generate DEM golden vectors by running the reference's own DEM classes.

Run where a topomax reference checkout is available, naming its root in
``TOPOMAX_REFERENCE`` (required; there is no default); torch and scipy must import::

    TOPOMAX_REFERENCE=/path/to/topomax python tests/golden/make_dem_golden.py

The reference imports ``rff`` (random_fourier_features_pytorch), which is not
installed; a stub module written from the encoder's definition (gamma(x) =
[cos 2 pi B x, sin 2 pi B x], B ~ N(0, sigma^2)) is put on ``sys.path`` so that
``DEM_src.elasisity_problem`` imports.  None of the fixtures below runs the
encoder.  Output: ``tests/golden/dem_energy.npz`` with

* ``case*``: StrainEnergy.calculate_energy (DEM_src/elasisity_problem.py:97-118)
  and its torch-autograd gradients with respect to u and the density, plus
  calculate_objective_and_gradient (:120-129), on small meshes with a traction
  and a circular body force;
* ``mask*``: ElasticityEnforcer.zero_enforcer (DEM_src/dirichlet_enforcer.py:14-56);
* ``circle*``: CircleDomain cells and areas (DEM_src/domains.py:56-257);
* ``side*``: boundary_integral (DEM_src/integrator.py:70-99) of unit node vectors.

and ``tests/golden/dem_density_filter.npz`` with ``filter*``: the reference's
create_density_filter (DEM_src/filter.py:8-31) applied as ``W @ rho`` and
``W.T @ g`` (the two uses in DEM_src/elasisity_problem.py:162, 171) to seeded
vectors, on meshes whose radius spans no neighbour, a few, and an exact
grid distance.  ``python tests/golden/make_dem_golden.py filter`` writes only
this file.
"""
from __future__ import annotations

import math
import os
import sys
import tempfile

import numpy as np

REF = os.environ.get("TOPOMAX_REFERENCE", "")
HERE = os.path.dirname(os.path.abspath(__file__))

STUB = '''
import math
import torch


class GaussianEncoding(torch.nn.Module):
    def __init__(self, sigma, input_size, encoded_size):
        super().__init__()
        self.register_buffer("b", torch.randn((encoded_size, input_size)) * sigma)

    def forward(self, v):
        vp = 2 * math.pi * v @ self.b.T
        return torch.cat((torch.cos(vp), torch.sin(vp)), dim=-1)
'''


def _install_stub() -> None:
    root = tempfile.mkdtemp(prefix="rff_stub_")
    pkg = os.path.join(root, "rff")
    os.makedirs(pkg)
    open(os.path.join(pkg, "__init__.py"), "w").write("from . import layers\n")
    open(os.path.join(pkg, "layers.py"), "w").write(STUB)
    sys.path.insert(0, root)


FILTER_CASES = [
    # (Nx, Ny, width, height, radius)
    (12, 6, 2.0, 1.0, 0.3),
    (20, 10, 2.0, 1.0, 0.05),   # radius below the spacing: each row is the element itself
    (11, 5, 2.0, 1.0, 0.4),     # 0.4 is exactly twice the x spacing: weight-0 entries
    (17, 9, 3.0, 1.0, 0.45),
    (30, 2, 2.0, 1.0, 0.25),
]


def density_filter_cases() -> None:
    sys.path.insert(0, REF)
    from DEM_src.utils import Mesh
    from DEM_src.filter import create_density_filter

    out = {}
    rng = np.random.default_rng(5)
    for k, (Nx, Ny, W, H, r) in enumerate(FILTER_CASES):
        mesh = Mesh(Nx, Ny, W, H)
        F = create_density_filter(r, mesh)
        rho = rng.uniform(0.01, 1.0, (Ny, Nx))
        g = rng.standard_normal(Nx * Ny)
        out[f"filter{k}_meta"] = np.array([Nx, Ny, W, H, r])
        out[f"filter{k}_rho"] = rho
        out[f"filter{k}_g"] = g
        out[f"filter{k}_apply"] = F @ rho.flatten()
        out[f"filter{k}_transpose"] = F.T @ g
        out[f"filter{k}_nnz"] = np.array(F.nnz)
    np.savez(os.path.join(HERE, "dem_density_filter.npz"), **out)


def main() -> None:
    if len(sys.argv) > 1 and sys.argv[1] == "filter":
        density_filter_cases()
        return
    energy_cases()
    density_filter_cases()


def energy_cases() -> None:
    import torch
    if not hasattr(np, "trapz"):  # DEM_src/integrator.py uses np.trapz (removed in numpy 2)
        np.trapz = np.trapezoid
    _install_stub()
    sys.path.insert(0, REF)
    from DEM_src.utils import Mesh
    from DEM_src.domains import CircleDomain, SideDomain
    from DEM_src.integrator import boundary_integral
    from DEM_src.dirichlet_enforcer import ElasticityEnforcer
    from DEM_src.elasisity_problem import BodyForce, StrainEnergy, TractionPoints
    from designs.definitions import CircularRegion, ElasticityParameters, Force, Side, Traction

    out = {}
    cases = [
        # (Nx, Ny, W, H, traction (side, center, length, value), body force (center, radius, value), p, seed)
        (24, 12, 2.0, 1.0, (Side.RIGHT, 0.5, 0.5, (0.0, -1.0)), ((1.0, 0.5), 0.1, (0.0, -1.0)), 3.0, 11),
        (30, 10, 3.0, 1.0, (Side.TOP, 1.4, 0.37, (0.3, -2.0)), ((2.1, 0.45), 0.23, (1.0, 0.5)), 3.0, 12),
        (17, 23, 1.0, 1.5, (Side.LEFT, 0.8, 0.61, (-1.0, 0.25)), None, 2.0, 13),
    ]
    for k, (Nx, Ny, W, H, tr, bf, p, seed) in enumerate(cases):
        mesh = Mesh(Nx, Ny, W, H)
        tps = [TractionPoints(mesh, Traction(tr[0], tr[1], tr[2], tr[3]))]
        body = BodyForce(mesh, Force(CircularRegion(bf[0], bf[1]), bf[2]), torch.device("cpu")) if bf else None
        se = StrainEnergy(mesh, body, 200000.0 if k == 0 else 1.7, 0.3 if k != 1 else 0.27, tps)
        se.set_penalization(p)
        g = torch.Generator().manual_seed(seed)
        u = (torch.randn(((Nx + 1) * (Ny + 1), 2), generator=g) * 0.01).float().requires_grad_(True)
        rho = (torch.rand((Ny, Nx), generator=g) * 0.99 + 0.01).float().requires_grad_(True)
        e = se.calculate_energy(u, mesh.shape, rho)
        gu, gr = torch.autograd.grad(e, (u, rho))
        obj, grad = se.calculate_objective_and_gradient(u.detach(), mesh.shape, rho.detach())
        young, nu = (200000.0 if k == 0 else 1.7), (0.3 if k != 1 else 0.27)
        out[f"case{k}_meta"] = np.array([Nx, Ny, W, H, p, young, nu])
        out[f"case{k}_traction"] = np.array([tr[0].value, tr[1], tr[2], tr[3][0], tr[3][1]])
        out[f"case{k}_body"] = np.array([bf[0][0], bf[0][1], bf[1], bf[2][0], bf[2][1]]) if bf else np.zeros(0)
        out[f"case{k}_u"] = u.detach().numpy()
        out[f"case{k}_rho"] = rho.detach().numpy()
        out[f"case{k}_energy"] = np.array(float(e))
        out[f"case{k}_grad_u"] = gu.numpy()
        out[f"case{k}_grad_rho"] = gr.numpy()
        out[f"case{k}_objective"] = np.array(float(obj))
        out[f"case{k}_gradient"] = grad.detach().numpy()

    for k, (Nx, Ny, sides) in enumerate([(20, 10, ["Left"]), (13, 7, ["Left", "Bottom"]),
                                         (9, 9, ["Right", "Top", "Left"])]):
        mesh = Mesh(Nx, Ny, 2.0, 1.0)
        params = ElasticityParameters(fixed_sides=[Side.from_string(s) for s in sides], body_force=None,
                                      tractions=None, filter_radius=0.05, young_modulus=1.0, poisson_ratio=0.3)
        enf = ElasticityEnforcer(params, mesh, torch.device("cpu"))
        out[f"mask{k}_meta"] = np.array([Nx, Ny, 2.0, 1.0])
        out[f"mask{k}_sides"] = np.array([Side.from_string(s).value for s in sides])
        out[f"mask{k}"] = enf.zero_enforcer.numpy()

    for k, (Nx, Ny, W, H, c, r) in enumerate([(40, 20, 2.0, 1.0, (1.0, 0.5), 0.05),
                                             (40, 20, 2.0, 1.0, (0.73, 0.31), 0.17),
                                             (60, 30, 2.0, 1.0, (1.0, 0.7), 0.05),
                                             (25, 25, 1.0, 1.0, (0.5, 0.5), 0.3)]):
        mesh = Mesh(Nx, Ny, W, H)
        cd = CircleDomain(mesh, CircularRegion(c, r))
        out[f"circle{k}_meta"] = np.array([Nx, Ny, W, H, c[0], c[1], r])
        out[f"circle{k}_indices"] = cd.indices
        out[f"circle{k}_areas"] = cd.areas

    for k, (Nx, Ny, side, center, length) in enumerate([(24, 12, Side.RIGHT, 0.5, 0.5), (30, 10, Side.TOP, 1.4, 0.37),
                                                       (30, 10, Side.BOTTOM, 1.0, 0.4), (17, 23, Side.LEFT, 0.8, 0.61)]):
        W, H = (2.0, 1.0) if k == 0 else ((3.0, 1.0) if k < 3 else (1.0, 1.5))
        mesh = Mesh(Nx, Ny, W, H)
        dom = SideDomain(mesh, side, center, length)
        nn = (Nx + 1) * (Ny + 1)
        w = np.zeros(nn)
        for n in range(nn):  # the integral of each unit node vector = that node's weight
            e = torch.zeros(nn, dtype=torch.float64)
            e[n] = 1.0
            w[n] = float(boundary_integral(e, mesh, dom))
        out[f"side{k}_meta"] = np.array([Nx, Ny, W, H, side.value, center, length])
        out[f"side{k}_weights"] = w

    np.savez(os.path.join(HERE, "dem_energy.npz"), **out)
    print("wrote", os.path.join(HERE, "dem_energy.npz"), len(out), "arrays")


if __name__ == "__main__":
    if not REF or not os.path.isdir(REF):
        sys.exit("set TOPOMAX_REFERENCE to the root of a topomax checkout"
                 + (f" ({REF} is not a directory)" if REF else ""))
    main()
