"""FP64 CPU restatement of the DEM strain energy (test infrastructure only).

The product never imports this module; tests compare the CUDA kernels of
``topomax_gb300/csrc/topo_dem.cu`` against it and pin it against the
reference's own outputs (``tests/golden/dem_*.npz``).

Follows ``DEM_src/objective_calculator.py:19-125`` (bilinear cells, 2x2 Gauss
points, the rounded shape-derivative table a = 0.394337567, b = 0.105662433,
gradient = sum over the cell's four nodes of U * Jinv dN) and
``DEM_src/elasisity_problem.py:79-129`` (sigma:eps, SIMP r(rho) = m + rho^p (1 - m),
psi = 1/2 sum r SE detJ - external work; objective sum r SE detJ and
gradient -r' SE detJ).  The external work is the linear functional sum W*u
with W from ``topomax_gb300.dem.external_weights``.
"""
from __future__ import annotations

import numpy as np

A, B = 0.394337567, 0.105662433
M = 1e-6


def shape_table(dx: float, dy: float) -> np.ndarray:
    """D[i, g, k]: d N_i / dx_k at Gauss point g (DEM_src/objective_calculator.py:28-52)."""
    a, b = A, B
    dN = [np.array([[-a, -b, -b, -a], [-a, -a, -b, -b]]), np.array([[-b, -a, -a, -b], [a, a, b, b]]),
          np.array([[a, b, b, a], [-b, -b, -a, -a]]), np.array([[b, a, a, b], [b, b, a, a]])]
    Jinv = np.linalg.inv(np.array([[dx / 2, 0], [0, dy / 2]]))
    return np.array([[Jinv @ d[:, g] for g in range(4)] for d in dN])


def cell_corners(u: np.ndarray, Nx: int, Ny: int) -> np.ndarray:
    """U[i, j, iy, ix]: component j of corner i of cell (ix, iy); u in x-major flat order."""
    U = u.reshape(Nx + 1, Ny + 1, 2).transpose(1, 0, 2)  # [iy, ix, j]
    c = [U[:-1, :-1], U[1:, :-1], U[:-1, 1:], U[1:, 1:]]
    return np.stack([np.moveaxis(ci, -1, 0) for ci in c])


def strain_energy(u: np.ndarray, Nx: int, Ny: int, W: float, H: float, lam: float, mu: float):
    """SE[iy, ix] = sum over Gauss points of sigma:eps, and sigma at each point."""
    D = shape_table(W / Nx, H / Ny)
    U = cell_corners(u, Nx, Ny)
    se = np.zeros((Ny, Nx))
    sig = []
    for g in range(4):
        G = np.einsum("ijyx,ik->jkyx", U, D[:, g, :])  # grad[j][k]
        eps = 0.5 * (G + G.transpose(1, 0, 2, 3))
        div = G[0, 0] + G[1, 1]
        s = 2 * mu * eps
        s[0, 0] += lam * div
        s[1, 1] += lam * div
        sig.append(s)
        se += np.sum(s * eps, axis=(0, 1))
    return se, sig, D, U


def lame(young: float, nu: float):
    mu = young / (2 * (1 + nu))
    return mu * nu / (0.5 - nu), mu


def energy(u, rho, Nx, Ny, W, H, young, nu, p, wext=None):
    """psi, d psi / d u (x-major (nn, 2)), d psi / d rho ([Ny, Nx])."""
    lam, mu = lame(young, nu)
    se, sig, D, _ = strain_energy(np.asarray(u, float), Nx, Ny, W, H, lam, mu)
    detJ = (W / Nx / 2) * (H / Ny / 2)
    rho = np.asarray(rho, float).reshape(Ny, Nx)
    r = M + rho ** p * (1 - M)
    dr = p * rho ** (p - 1) * (1 - M)
    psi = 0.5 * np.sum(r * se * detJ)
    gu = np.zeros((Ny + 1, Nx + 1, 2))  # [iy, ix, j]
    off = [(0, 0), (1, 0), (0, 1), (1, 1)]  # corner i -> (diy, dix)
    for g in range(4):
        for i, (diy, dix) in enumerate(off):
            for j in range(2):
                c = r * detJ * (sig[g][j, 0] * D[i, g, 0] + sig[g][j, 1] * D[i, g, 1])
                gu[diy:diy + Ny, dix:dix + Nx, j] += c
    gu = gu.transpose(1, 0, 2).reshape(-1, 2)
    if wext is not None:
        psi -= float(np.sum(wext * np.asarray(u, float)))
        gu = gu - wext
    return psi, gu, 0.5 * dr * se * detJ


def objective_and_gradient(u, rho, Nx, Ny, W, H, young, nu, p):
    lam, mu = lame(young, nu)
    se, _, _, _ = strain_energy(np.asarray(u, float), Nx, Ny, W, H, lam, mu)
    detJ = (W / Nx / 2) * (H / Ny / 2)
    rho = np.asarray(rho, float).reshape(Ny, Nx)
    sel = se * detJ
    return float(np.sum((M + rho ** p * (1 - M)) * sel)), -(p * rho ** (p - 1) * (1 - M)) * sel


# ---------------------------------------------------------------------------
# density filter (DEM_src/filter.py:8-31)
# ---------------------------------------------------------------------------


def _linspace(L: float, n: int) -> np.ndarray:
    return np.linspace(0.0, L, n)


def density_filter_rows(Nx: int, Ny: int, W: float, H: float, radius: float):
    """Row i = iy*Nx + ix: the neighbours j (ascending) with dist <= radius, the weights
    radius - dist and the row sum, in the reference's order of operations (distances
    to the element points of np.linspace(0, W, Nx) x np.linspace(0, H, Ny); l1 row
    normalisation sums the weights in column order and divides each by the sum).
    Pure-Python loops: small meshes only."""
    xs, ys = _linspace(W, Nx), _linspace(H, Ny)
    X = np.tile(xs, Ny)
    Y = np.repeat(ys, Nx)
    rows = []
    for i in range(Nx * Ny):
        dist = np.sqrt((X - X[i]) ** 2 + (Y - Y[i]) ** 2)
        (nb,) = np.where(dist <= radius)
        w = radius - dist[nb]
        s = 0.0
        for v in w:
            s += abs(v)
        rows.append((nb, w, s))
    return rows


def density_filter_apply(Nx, Ny, W, H, radius, rho, transpose=False):
    """W @ rho (row sums, then sequential products in column order), or W.T @ g
    accumulated row by row into the outputs (the CSC product order)."""
    rows = density_filter_rows(Nx, Ny, W, H, radius)
    v = np.asarray(rho, dtype=np.float64).ravel()
    out = np.zeros(Nx * Ny)
    for i, (nb, w, s) in enumerate(rows):
        wn = w / s if s != 0.0 else w
        if not transpose:
            acc = 0.0
            for j, c in zip(nb, wn):
                acc += c * v[j]
            out[i] = acc
        else:
            for j, c in zip(nb, wn):
                out[j] += c * v[i]
    return out
