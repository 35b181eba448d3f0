"""Deep-energy-method (DEM) energy path on the GPU, behind the reference's DEM classes.

Mirrors ``DEM_src`` of topomax: ``Mesh`` and ``flatten``/``unflatten``
(``DEM_src/utils.py``), ``SideDomain``/``CircleDomain`` (``DEM_src/domains.py``),
``TractionPoints``/``BodyForce``/``StrainEnergy`` (``DEM_src/elasisity_problem.py:19-129``),
``ElasticityEnforcer`` (``DEM_src/dirichlet_enforcer.py:14-56``) and ``MultiLayerNet``
(``DEM_src/deep_energy_method.py:149-184``), ``create_density_filter``
(``DEM_src/filter.py:8-31``), the training step ``DeepEnergyMethod``
(``DEM_src/deep_energy_method.py:28-146``) and the DEM ``ElasticityProblem``
(``DEM_src/elasisity_problem.py:131-216``).  The energy, its gradients, the Dirichlet mask and the density
filter run in the CUDA kernels of ``csrc/topo_dem.cu`` through the C ABI; the network stays
in torch.  The external work (traction and body-force integrals) is linear in u, so the host
turns the reference's integration rules into per-node weights once.

There is no CPU path: without the library or a CUDA device these classes raise.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass
import math
from typing import Iterable

import numpy as np
import torch

from . import _capi
from .designs import Side

# ---------------------------------------------------------------------------
# mesh and layouts (DEM_src/utils.py)
# ---------------------------------------------------------------------------


class Mesh:
    """Structured Nx x Ny quadrilateral mesh of [0, width] x [0, height] (DEM_src/utils.py:9-31)."""

    def __init__(self, Nx: int, Ny: int, width: float, height: float):
        self.Nx, self.Ny = int(Nx), int(Ny)
        self.width, self.height = float(width), float(height)
        xs = np.linspace(0.0, self.width, self.Nx + 1)
        ys = np.linspace(0.0, self.height, self.Ny + 1)
        self.x_grid, self.y_grid = np.meshgrid(xs, ys)
        self.intervals = (self.Ny, self.Nx)
        self.shape = (self.Ny + 1, self.Nx + 1)
        self.dxdy = (self.width / self.Nx, self.height / self.Ny)


def flatten(grids: Iterable[np.ndarray]) -> np.ndarray:
    """(Ny, Nx) grids -> (Nx*Ny, n) in x-major order (node (ix, iy) at ix*Ny + iy)."""
    return np.array([np.asarray(g).T.ravel() for g in grids]).T


def unflatten(values, shape: tuple[int, int]):
    """(Nx*Ny, n) values and shape (Ny, Nx) -> (n, Ny, Nx)."""
    Ny, Nx = shape
    n, dim = values.shape
    if Ny * Nx != n:
        raise ValueError(f"Got an input array with {n} elements, but input shape only has {Nx}*{Ny}={Nx * Ny} elements")
    r = values.reshape(Nx, Ny, dim)
    return r.permute((2, 1, 0)) if isinstance(r, torch.Tensor) else r.T


# ---------------------------------------------------------------------------
# load domains (DEM_src/domains.py) -> linear external-work weights
# ---------------------------------------------------------------------------


class SideDomain:
    """Boundary nodes of one side inside [center - length/2, center + length/2] (DEM_src/domains.py:11-53)."""

    def __init__(self, mesh: Mesh, side: Side, center: float, length: float):
        lo, hi = center - length / 2, center + length / 2
        fx, fy = mesh.x_grid.T.ravel(), mesh.y_grid.T.ravel()
        if side == Side.LEFT:
            on, along = fx == 0, fy
        elif side == Side.RIGHT:
            on, along = fx == mesh.width, fy
        elif side == Side.TOP:
            on, along = fy == mesh.height, fx
        elif side == Side.BOTTOM:
            on, along = fy == 0, fx
        else:
            raise ValueError(f"Unknown side: '{side}'")
        vertical = side in (Side.LEFT, Side.RIGHT)
        self.side = side
        self.side_index = 1 if vertical else 0
        self.stride = 1 if vertical else mesh.Ny + 1
        self.width = mesh.Ny + 1 if vertical else mesh.Nx + 1
        (idx,) = np.where(on & (along >= lo) & (along <= hi))
        if idx.size == 0:
            raise ValueError("traction interval contains no boundary node")
        coord = np.array([fx[idx], fy[idx]]).T[:, self.side_index]
        self.indices = idx
        self.left_error = coord[0] - lo
        self.right_error = hi - coord[-1]

    def weights(self, mesh: Mesh) -> np.ndarray:
        """w with sum_n w[n] d[n] == the reference's boundary_integral(d) (DEM_src/integrator.py:70-99)."""
        nn = (mesh.Nx + 1) * (mesh.Ny + 1)
        w = np.zeros(nn)
        ds = mesh.dxdy[self.side_index]
        idx = self.indices
        if idx.size > 1:  # trapezoid rule with spacing ds
            w[idx[:-1]] += ds / 2
            w[idx[1:]] += ds / 2
        if (idx[0] / self.stride) % self.width != 0:
            t = self.left_error / ds  # lerp(d[i0 - stride], d[i0], t), then a trapezoid of width left_error
            w[(idx[0] - self.stride) % nn] += self.left_error * t / 2
            w[idx[0]] += self.left_error * ((1 - t) + 1) / 2
        if ((idx[-1] / self.stride) + 1) % self.width != 0:
            j = idx[-1] + self.stride
            if j >= nn:
                raise IndexError(f"index {j} is out of bounds for size {nn}")
            t = self.right_error / ds
            w[j] += self.right_error * t / 2
            w[idx[-1]] += self.right_error * ((1 - t) + 1) / 2
        return w


def _dist(values, point):
    values, point = np.asarray(values, dtype=float), np.asarray(point, dtype=float)
    if values.ndim == 1:
        return math.sqrt(float(np.sum((values - point) ** 2)))
    return np.sqrt(np.sum((values - point) ** 2, axis=1))


class CircleDomain:
    """Cells cut by a circle and the cut areas (DEM_src/domains.py:56-257): the same
    intersection walk and the same triangle / complement / trapezoid area rules."""

    def __init__(self, mesh: Mesh, region, device=None):
        self.center = tuple(float(v) for v in region.center)
        self.radius = float(region.radius)
        pts = self._intersections(mesh)
        self.indices, self.areas = self._areas(mesh, pts)
        exact = math.pi * self.radius ** 2
        self.area_error = abs(float(np.sum(self.areas)) - exact) / exact
        self.torch_areas = torch.from_numpy(self.areas).float().to(device) if device else None

    def _intersections(self, mesh: Mesh) -> np.ndarray:
        r2 = self.radius ** 2
        cx, cy = self.center
        pts: list[tuple[float, float]] = []
        for y in mesh.y_grid[:, 0]:
            h2 = (y - cy) ** 2
            if h2 <= r2:
                l = np.sqrt(r2 - h2)
                pts += [(cx - l, y), (cx + l, y)]
        for x in mesh.x_grid[0, :]:
            h2 = (x - cx) ** 2
            if h2 <= r2:
                l = np.sqrt(r2 - h2)
                pts += [(x, cy - l), (x, cy + l)]
        if not pts:
            raise ValueError("Tried to precompute circle areas, but circle does not intersect grid!")
        arr = np.array(pts)
        drop: set[int] = set()
        for i in range(len(arr)):
            if i in drop:
                continue
            for j in range(i + 1, len(arr)):
                if _dist(arr[i], arr[j]) < 1e-6 * self.radius:
                    drop.add(j)
        if drop:
            arr = arr[list(set(range(len(arr))).difference(drop))]
        return arr

    @staticmethod
    def _grid_position(mesh: Mesh, p):
        dx, dy = mesh.dxdy
        return (round(p[0] / dx, 12), round(p[1] / dy, 12))

    @classmethod
    def _grid_index(cls, mesh: Mesh, p):
        gx, gy = cls._grid_position(mesh, p)
        return (int(np.floor(gx)), int(np.floor(gy)))

    @classmethod
    def _corners(cls, mesh: Mesh, p):
        dx, dy = mesh.dxdy
        gx, gy = cls._grid_position(mesh, p)
        s: set[tuple[int, int]] = set()  # same insertion order as the reference: same iteration order
        s.add((int(np.ceil(gx)), int(np.ceil(gy))))
        s.add((int(np.ceil(gx)), int(np.floor(gy))))
        s.add((int(np.floor(gx)), int(np.ceil(gy))))
        s.add((int(np.floor(gx)), int(np.floor(gy))))
        return [(ix * dx, iy * dy) for ix, iy in list(s)]

    def _areas(self, mesh: Mesh, pts: np.ndarray):
        dx, dy = mesh.dxdy
        c = np.array(self.center)
        R = self.radius
        areas = np.full(mesh.intervals, dx * dy)
        cells: list[tuple[int, int]] = []
        diag = np.sqrt(dx ** 2 + dy ** 2)
        xs = (mesh.x_grid[0, :-1] + mesh.x_grid[0, 1:]) / 2
        ys = (mesh.y_grid[:-1, 0] + mesh.y_grid[1:, 0]) / 2
        for y in ys:
            for x in xs:
                if _dist(np.array([x, y]), c) > R + diag / 2:
                    continue
                near = np.array(self._corners(mesh, (x, y)))
                if np.min(_dist(near, c)) - R < -1e-6 * R:
                    ix, iy = self._grid_index(mesh, (x, y))
                    cells.append((iy, ix))
        cell_arr = np.array(cells)
        ang = np.angle((pts[:, 0] - c[0]) + 1j * (pts[:, 1] - c[1]))
        pts = pts[np.argsort(-ang)]
        for i, p0 in enumerate(pts):
            p1 = pts[(i + 1) % len(pts)]
            g0x, g0y = self._grid_position(mesh, p0)
            g1x, g1y = self._grid_position(mesh, p1)
            mid = (p0 + p1) / 2
            index = self._grid_index(mesh, mid)
            near = np.array(self._corners(mesh, mid))
            near = near[np.where((_dist(near, p0) > 1e-6 * diag) & (_dist(near, p1) > 1e-6 * diag))]
            if (g0x == int(g0x) and g1y == int(g1y)) or (g0y == int(g0y) and g1x == int(g1x)):
                corner = near[np.argmin(_dist(near, mid))]
                a, b = _dist(p0, corner), _dist(p1, corner)
                area = 0.5 * a * b if _dist(corner, c) <= R else dx * dy - 0.5 * a * b
            else:
                inside = near[np.where(_dist(near, c) <= R)]
                c0 = inside[np.argmin(_dist(inside, p0))]
                c1 = inside[np.argmin(_dist(inside, p1))]
                area = 0.5 * _dist(c0, c1) * (_dist(p0, c0) + _dist(p1, c1))
            areas[index[1], index[0]] = area
        return cell_arr, areas[tuple(cell_arr.T)]

    def weights(self, mesh: Mesh) -> np.ndarray:
        """w with sum_n w[n] d[n] == the reference's circular_integral(d) (DEM_src/integrator.py:44-67):
        each cut cell's area, times the mean of its four corners."""
        w = np.zeros((mesh.Nx + 1) * (mesh.Ny + 1))
        NY = mesh.Ny + 1
        for (iy, ix), a in zip(self.indices, self.areas):
            for dix in (0, 1):
                for diy in (0, 1):
                    w[(ix + dix) * NY + iy + diy] += a / 4
        return w


class TractionPoints:
    """DEM_src/elasisity_problem.py:19-22."""

    def __init__(self, mesh: Mesh, traction):
        side, center, length, self.value = traction.to_tuple()
        self.domain = SideDomain(mesh, side, center, length)


class BodyForce:
    """DEM_src/elasisity_problem.py:25-28."""

    def __init__(self, mesh: Mesh, force, device=None):
        self.value = force.value
        self.domain = CircleDomain(mesh, force.region, device)


def external_weights(mesh: Mesh, body_force: BodyForce | None,
                     traction_points_list: list[TractionPoints] | None) -> np.ndarray:
    """Per-node weights W (shape (nn, 2)) with external work = sum W * u, following
    calculate_traction_integral / calculate_body_force_integral (DEM_src/elasisity_problem.py:31-60)."""
    W = np.zeros(((mesh.Nx + 1) * (mesh.Ny + 1), 2))
    for tp in traction_points_list or []:
        w = tp.domain.weights(mesh)
        for k in range(2):
            if abs(tp.value[k]) > 1e-14:
                W[:, k] += w * tp.value[k]
    if body_force is not None:
        w = body_force.domain.weights(mesh)
        for k in range(2):
            if abs(body_force.value[k]) > 1e-14:
                W[:, k] += w * body_force.value[k]
    return W


# ---------------------------------------------------------------------------
# quadrature constants (DEM_src/objective_calculator.py:28-52)
# ---------------------------------------------------------------------------
_A, _B = 0.394337567, 0.105662433  # (1 +- 1/sqrt(3)) / 4, the reference's rounded values


def shape_derivatives():
    """d N_i / d(s, t) at the 4 Gauss points, nodes in get_gauss_points order."""
    a, b = _A, _B
    return [np.array([[-a, -b, -b, -a], [-a, -a, -b, -b]]),
            np.array([[-b, -a, -a, -b], [a, a, b, b]]),
            np.array([[a, b, b, a], [-b, -b, -a, -a]]),
            np.array([[b, a, a, b], [b, b, a, a]])]


def jacobian(dxdy):
    dx, dy = dxdy
    J = np.array([[dx / 2, 0], [0, dy / 2]])
    return np.linalg.inv(J), float(np.linalg.det(J))


# ---------------------------------------------------------------------------
# the energy through the C ABI
# ---------------------------------------------------------------------------


def _ptr(t: torch.Tensor) -> int:
    return t.data_ptr()


def _stream() -> int:
    return torch.cuda.current_stream().cuda_stream


class _DemContext:
    def __init__(self, mesh: Mesh, young_modulus: float, poisson_ratio: float):
        if not torch.cuda.is_available():
            raise RuntimeError("topomax_gb300.dem needs a CUDA device (there is no CPU path)")
        self.lib = _capi.load_library()
        Jinv, detJ = jacobian(mesh.dxdy)
        d = _capi.DemDesc()
        d.nx, d.ny = mesh.Nx, mesh.Ny
        table = np.zeros((4, 4, 2), dtype=np.float32)
        for i, dN in enumerate(shape_derivatives()):
            for g in range(4):
                table[i, g] = (Jinv @ dN[:, g].reshape((2, 1))).ravel().astype(np.float32)
        d.dshape[:] = [float(v) for v in table.ravel()]
        mu = young_modulus / (2 * (1 + poisson_ratio))
        lam = mu * poisson_ratio / (0.5 - poisson_ratio)
        d.detJ = float(np.float32(detJ))
        d.lame_lambda = float(np.float32(lam))
        d.two_mu = float(np.float32(2 * mu))
        st = ctypes.c_int(0)
        self.ptr = self.lib.topo_dem_create(ctypes.byref(d), ctypes.byref(st))
        if not self.ptr:
            raise RuntimeError(f"topo_dem_create failed ({st.value})")
        self.mesh = mesh
        self.detJ = detJ

    def check(self, rc: int) -> None:
        if rc == _capi.TOPO_OK:
            return
        msg = self.lib.topo_dem_last_error(self.ptr).decode()
        if rc == _capi.TOPO_ERR_CUDA:
            raise RuntimeError(f"topomax_gb300 CUDA error: {msg}")
        raise ValueError(msg or f"topomax_gb300 error {rc}")

    def __del__(self):
        ptr, self.ptr = getattr(self, "ptr", None), None
        if ptr:
            self.lib.topo_dem_destroy(ptr)


# ---------------------------------------------------------------------------
# density filter (DEM_src/filter.py:8-31)
# ---------------------------------------------------------------------------


class DensityFilter:
    """The reference's density filter W (a row-normalised radius-neighbour matrix over
    the element points) as a GPU operator: ``W @ rho`` and ``W.T @ g`` as the reference's
    ``DEM_src/elasisity_problem.py:162, 171`` use it, bit-identical to the scipy product.
    Accepts numpy arrays (returns numpy) or torch tensors (returns a CUDA FP64 tensor)
    of Nx*Ny values in the reference's flatten order (element iy*Nx + ix)."""

    def __init__(self, radius: float, mesh: Mesh):
        if not torch.cuda.is_available():
            raise RuntimeError("topomax_gb300.dem needs a CUDA device (there is no CPU path)")
        self.lib = _capi.load_library()
        self.n = mesh.Nx * mesh.Ny
        self.shape = (self.n, self.n)
        st = ctypes.c_int(0)
        self.ptr = self.lib.topo_density_filter_create(mesh.Nx, mesh.Ny, float(mesh.width), float(mesh.height),
                                                       float(radius), ctypes.byref(st))
        if not self.ptr:
            if st.value == _capi.TOPO_ERR_CUDA:
                raise RuntimeError("topo_density_filter_create: CUDA error")
            raise ValueError(f"invalid density filter (radius {radius}, mesh {mesh.Nx}x{mesh.Ny})")
        self._transpose = False

    @property
    def nnz(self) -> int:
        v = ctypes.c_int64(0)
        self.lib.topo_density_filter_nnz(self.ptr, ctypes.byref(v))
        return int(v.value)

    @property
    def T(self) -> "DensityFilter":
        t = object.__new__(DensityFilter)
        t.__dict__.update(self.__dict__)
        t._owner = self  # keeps the device object alive
        t._transpose = not self._transpose
        return t

    def __matmul__(self, v):
        as_numpy = isinstance(v, np.ndarray)
        x = torch.as_tensor(np.asarray(v) if as_numpy else v).to(device="cuda", dtype=torch.float64)
        x = x.reshape(-1).contiguous()
        if x.numel() != self.n:
            raise ValueError(f"dimension mismatch: filter of size {self.n}, vector of size {x.numel()}")
        y = torch.empty_like(x)
        rc = self.lib.topo_density_filter_apply(self.ptr, _ptr(x), _ptr(y), int(self._transpose), _stream())
        if rc != _capi.TOPO_OK:
            raise RuntimeError(f"topo_density_filter_apply failed ({rc})")
        return y.cpu().numpy() if as_numpy else y

    def __del__(self):
        if getattr(self, "_owner", None) is not None:
            return
        ptr, self.ptr = getattr(self, "ptr", None), None
        if ptr:
            self.lib.topo_density_filter_destroy(ptr)


def create_density_filter(radius: float, mesh: Mesh) -> DensityFilter:
    """Replaces DEM_src/filter.py:8-31 (same weights, no O(N^2) host construction)."""
    return DensityFilter(radius, mesh)


def _as_u(u: torch.Tensor, mesh: Mesh) -> torch.Tensor:
    nn = (mesh.Nx + 1) * (mesh.Ny + 1)
    if u.shape != (nn, 2):
        raise ValueError(f"u must have shape ({nn}, 2), got {tuple(u.shape)}")
    return u.detach().to(device="cuda", dtype=torch.float32).contiguous()


def _as_density(rho: torch.Tensor, mesh: Mesh) -> torch.Tensor:
    r = rho.detach().to(device="cuda", dtype=torch.float32).contiguous()
    if r.numel() != mesh.Nx * mesh.Ny:
        raise ValueError(f"density must have {mesh.Nx * mesh.Ny} cells, got {r.numel()}")
    return r.reshape(mesh.intervals)


class _EnergyFn(torch.autograd.Function):
    """psi(u, rho) with hand-written backward kernels (d psi/du, d psi/d rho)."""

    @staticmethod
    def forward(ctx, u, rho, dem, masked):
        uu, rr = _as_u(u, dem.mesh), _as_density(rho, dem.mesh)
        out = torch.empty((), dtype=torch.float64, device="cuda")
        dem.check(dem.lib.topo_dem_energy(dem.ptr, _ptr(uu), _ptr(rr), int(masked), _ptr(out), _stream()))
        ctx.save_for_backward(uu, rr)
        ctx.dem, ctx.masked = dem, masked
        ctx.rho_shape = rho.shape
        return out.to(torch.float32)

    @staticmethod
    def backward(ctx, grad):
        uu, rr = ctx.saved_tensors
        dem = ctx.dem
        scale = grad.detach().to(device="cuda", dtype=torch.float32).reshape(()).contiguous()
        du = torch.empty_like(uu) if ctx.needs_input_grad[0] else None
        dr = torch.empty_like(rr) if ctx.needs_input_grad[1] else None
        dem.check(dem.lib.topo_dem_energy_backward(dem.ptr, _ptr(uu), _ptr(rr), int(ctx.masked), _ptr(scale),
                                                   _ptr(du) if du is not None else None,
                                                   _ptr(dr) if dr is not None else None, _stream()))
        return du, (dr.reshape(ctx.rho_shape) if dr is not None else None), None, None


class StrainEnergy:
    """StrainEnergy of DEM_src/elasisity_problem.py:63-129 on the GPU.

    ``calculate_energy(u, shape, density)`` returns psi as a differentiable float32 tensor
    (torch autograd reaches u and density through the backward kernels);
    ``calculate_objective_and_gradient`` returns (sum r SE detJ, -r' SE detJ per cell).
    """

    def __init__(self, mesh: Mesh, body_force: BodyForce | None, Young_modulus: float, Poisson_ratio: float,
                 traction_points_list: list[TractionPoints] | None):
        self.mesh = mesh
        self.body_force = body_force
        self.traction_points_list = traction_points_list
        self.lamé_mu = Young_modulus / (2 * (1 + Poisson_ratio))
        self.lamé_lda = self.lamé_mu * Poisson_ratio / (0.5 - Poisson_ratio)
        self._dem = _DemContext(mesh, Young_modulus, Poisson_ratio)
        self.Jinv, self.detJ = jacobian(mesh.dxdy)
        W = external_weights(mesh, body_force, traction_points_list)
        self._has_ext = bool(np.any(W != 0))
        if self._has_ext:
            w32 = np.ascontiguousarray(W.astype(np.float32))
            self._dem.check(self._dem.lib.topo_dem_set_external(self._dem.ptr, w32.ctypes.data))
        self.penalization: float | None = None
        self._mask_owner = None

    def set_penalization(self, penalization: float):
        self.penalization = float(penalization)
        self._dem.check(self._dem.lib.topo_dem_set_penalization(self._dem.ptr, self.penalization))

    def _check_shape(self, shape):
        if tuple(shape) != self.mesh.shape:
            raise ValueError(f"shape must be the mesh shape {self.mesh.shape}, got {tuple(shape)}")

    def calculate_energy(self, u: torch.Tensor, shape, density: torch.Tensor) -> torch.Tensor:
        """psi(u; rho) = 1/2 int r(rho) sigma:eps dx - int f.u dx - int t.u ds."""
        self._check_shape(shape)
        return _EnergyFn.apply(u, density, self._dem, False)

    def calculate_energy_enforced(self, u_hat: torch.Tensor, enforcer: "ElasticityEnforcer",
                                  density: torch.Tensor) -> torch.Tensor:
        """calculate_energy(enforcer(u_hat), ...) in one pass (the mask applied while loading)."""
        enforcer._install(self._dem)
        return _EnergyFn.apply(u_hat, density, self._dem, True)

    def calculate_objective_and_gradient(self, u: torch.Tensor, shape, density: torch.Tensor):
        """(sum r(rho) SE detJ, -r'(rho) SE detJ) as float32 tensors (gradient shaped like density)."""
        self._check_shape(shape)
        uu, rr = _as_u(u, self.mesh), _as_density(density, self.mesh)
        obj = torch.empty((), dtype=torch.float64, device="cuda")
        grad = torch.empty_like(rr)
        self._dem.check(self._dem.lib.topo_dem_objective_gradient(self._dem.ptr, _ptr(uu), _ptr(rr), _ptr(obj),
                                                                  _ptr(grad), _stream()))
        return obj.to(torch.float32), grad.reshape(density.shape)


class ElasticityEnforcer:
    """u = u_hat * mask with the reference's zero enforcer (DEM_src/dirichlet_enforcer.py:14-56)."""

    def __init__(self, parameters, mesh: Mesh, device=None):
        self.mesh = mesh
        sides = sorted(set(parameters.fixed_sides), key=lambda v: v.value)
        nx = mesh.x_grid.T.ravel().reshape((-1, 1)) / mesh.width
        ny = mesh.y_grid.T.ravel().reshape((-1, 1)) / mesh.height
        z = np.ones((nx.size, 2))
        for side in sides:
            if side == Side.LEFT:
                z = z * nx
            elif side == Side.RIGHT:
                z = z * (1 - nx)
            elif side == Side.TOP:
                z = z * (1 - ny)
            elif side == Side.BOTTOM:
                z = z * ny
            else:
                raise ValueError(f"Unknown side: '{side}'")
        self.mask_host = np.ascontiguousarray(z.astype(np.float32))
        self.zero_enforcer = torch.from_numpy(self.mask_host).to(device or "cuda")
        self._dem = None

    def _install(self, dem: _DemContext) -> None:
        dem.check(dem.lib.topo_dem_set_mask(dem.ptr, self.mask_host.ctypes.data))
        self._dem = dem

    def __call__(self, u: torch.Tensor) -> torch.Tensor:
        return _EnforceFn.apply(u, self)


class _EnforceFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, u_hat, enf):
        if enf._dem is None:
            enf._install(_DemContext(enf.mesh, 1.0, 0.3))
        uh = _as_u(u_hat, enf.mesh)
        out = torch.empty_like(uh)
        enf._dem.check(enf._dem.lib.topo_dem_enforce(enf._dem.ptr, _ptr(uh), _ptr(out), _stream()))
        ctx.enf = enf
        return out

    @staticmethod
    def backward(ctx, grad):
        return grad * ctx.enf.zero_enforcer, None


# ---------------------------------------------------------------------------
# the network (stays in torch; DEM_src/deep_energy_method.py:149-184)
# ---------------------------------------------------------------------------


class GaussianEncoding(torch.nn.Module):
    """Random Fourier features gamma(x) = [cos 2 pi B x, sin 2 pi B x], B ~ N(0, sigma^2),
    B of shape (encoded_size, input_size)."""

    def __init__(self, sigma: float, input_size: int, encoded_size: int, b: torch.Tensor | None = None):
        super().__init__()
        if b is None:
            b = torch.randn((encoded_size, input_size)) * sigma
        self.register_buffer("b", b)

    def forward(self, v: torch.Tensor) -> torch.Tensor:
        vp = 2 * math.pi * v @ self.b.T
        return torch.cat((torch.cos(vp), torch.sin(vp)), dim=-1)


class MultiLayerNet(torch.nn.Module):
    """Fourier-feature MLP of DEM_src/deep_energy_method.py:149-184 (first linear layer unused,
    as there)."""

    def __init__(self, input_size: int, output_size: int, layer_count: int = 5, neuron_count: int = 68,
                 weight_deviation: float = 0.062264, fourier_deviation: float = 0.119297,
                 activation_function: str = "rrelu"):
        super().__init__()
        if layer_count < 2:
            raise ValueError("Can't create MultiLayerNet with less than 2 layers "
                             f"(tried to create one with {layer_count} layers)")
        self.layer_count = layer_count
        self.activation_function = getattr(torch, activation_function)
        self.encoding = GaussianEncoding(fourier_deviation, input_size, neuron_count // 2)
        self.linears = torch.nn.ModuleList()
        for i in range(layer_count):
            fan_in = input_size if i == 0 else neuron_count
            fan_out = output_size if i == layer_count - 1 else neuron_count
            lin = torch.nn.Linear(fan_in, fan_out)
            torch.nn.init.constant_(lin.bias, 0.0)
            torch.nn.init.normal_(lin.weight, mean=0, std=weight_deviation)
            self.linears.append(lin)

    def forward(self, x: torch.Tensor) -> torch.Tensor:
        y = self.encoding(x)
        for i in range(1, self.layer_count - 1):
            y = self.activation_function(self.linears[i](y))
        return self.linears[-1](y)


# ---------------------------------------------------------------------------
# training step and problem (DEM_src/deep_energy_method.py:28-146,
# DEM_src/elasisity_problem.py:131-216, DEM_src/problem.py:13-41)
# ---------------------------------------------------------------------------


@dataclass
class NNParameters:
    layer_count: int
    neuron_count: int
    learning_rate: float
    iteration_count: int
    weight_deviation: float
    fourier_deviation: float
    activation_function: str
    convergence_tolerance: float


def _network(input_size: int, output_size: int, p: NNParameters) -> MultiLayerNet:
    return MultiLayerNet(input_size, output_size, p.layer_count, p.neuron_count, p.weight_deviation,
                         p.fourier_deviation, p.activation_function)


class DeepEnergyMethod:
    """DeepEnergyMethod of DEM_src/deep_energy_method.py:28-146.  One L-BFGS closure
    evaluation = the network forward and backward in torch plus ONE fused kernel launch
    for the Dirichlet mask and the strain energy (and one for its gradient)."""

    def __init__(self, device, verbose: bool, output_size: int, nn_parameters: NNParameters,
                 dirichlet_enforcer: "ElasticityEnforcer", objective_calculator: StrainEnergy):
        self.device = torch.device(device) if device is not None else torch.device("cuda")
        self.model = _network(2, output_size, nn_parameters).to(self.device)
        self.verbose = verbose
        self.output_size = output_size
        self.nn_parameters = nn_parameters
        self.dirichlet_enforcer = dirichlet_enforcer
        self.objective_calculator = objective_calculator
        self.loss_array: list[float] = []

    def set_nn_parameters(self, nn_parameters: NNParameters):
        self.model = _network(2, self.output_size, nn_parameters).to(self.device)
        self.nn_parameters = nn_parameters

    def _coordinates(self, mesh: Mesh) -> torch.Tensor:
        return torch.from_numpy(flatten([mesh.x_grid, mesh.y_grid])).float().to(self.device)

    def train_model(self, rho, mesh: Mesh):
        """L-BFGS on the energy (lr, max_iter 20, strong-Wolfe line search, the loss-mean
        convergence test), then (objective, gradient) at the trained displacement."""
        x = self._coordinates(mesh)
        x.requires_grad_(True)
        density = torch.as_tensor(np.asarray(rho)).float().reshape(mesh.intervals).to(self.device)
        opt = torch.optim.LBFGS(self.model.parameters(), lr=self.nn_parameters.learning_rate, max_iter=20,
                                line_search_fn="strong_wolfe")
        energy = self.objective_calculator

        def closure_generator(t: int):
            def closure():
                loss = energy.calculate_energy_enforced(self.model(x), self.dirichlet_enforcer, density)
                opt.zero_grad()
                loss.backward()
                value = float(loss)
                if self.verbose:
                    print(f"\rIter: {t + 1:^3} - Loss: {value:.6g}", end="")
                self.loss_array.append(value)
                return value
            return closure

        for t in range(self.nn_parameters.iteration_count):
            opt.step(closure_generator(t))
            if self.convergence_check(self.loss_array, self.nn_parameters.convergence_tolerance):
                break
        if self.verbose:
            print()
        return energy.calculate_objective_and_gradient(self.get_u(x), mesh.shape, density)

    def get_loss(self, rho, mesh: Mesh) -> float:
        density = torch.as_tensor(np.asarray(rho)).float().reshape(mesh.intervals).to(self.device)
        return float(self.objective_calculator.calculate_energy(self.get_u(mesh=mesh), mesh.shape, density))

    def get_u(self, x: torch.Tensor | None = None, mesh: Mesh | None = None) -> torch.Tensor:
        if x is None:
            if mesh is None:
                raise ValueError("get_u must get either x or mesh, they can't both be None")
            x = self._coordinates(mesh)
        return self.dirichlet_enforcer(self.model(x))

    @staticmethod
    def convergence_check(loss_array, tolerance: float) -> bool:
        """The mean of the last 10 losses against the 10 before (at least 20 evaluations)."""
        num_check = 10
        if len(loss_array) < 2 * num_check:
            return False
        mean1 = float(np.mean(loss_array[-2 * num_check:-num_check]))
        mean2 = float(np.mean(loss_array[-num_check:]))
        if abs(mean2) < 1e-6:
            return True
        return abs(mean1 - mean2) / abs(mean2) < tolerance


class ElasticityProblem:
    """The DEM compliance problem of DEM_src/elasisity_problem.py:131-216: the density is
    filtered (classical radius = 2 sqrt(3) x the Helmholtz radius), the network trained
    on it, and the gradient mapped back through the filter's transpose."""

    def __init__(self, mesh: Mesh, device, verbose: bool, parameters):
        self.parameters = parameters
        self.mesh = mesh
        self.device = device
        self.verbose = verbose
        dirichlet_enforcer, objective_calculator = self.create_dem_parameters()
        self.dem = self.create_dem(dirichlet_enforcer, objective_calculator)
        self.filter = create_density_filter(self.parameters.filter_radius * 2 * np.sqrt(3), self.mesh)
        self.objective_gradient: np.ndarray | None = None

    def set_penalization(self, penalization: float):
        self.dem.objective_calculator.set_penalization(penalization)

    def calculate_objective_gradient(self):
        if self.objective_gradient is None:
            raise ValueError("You must call calculate_objective before calling calculate_objective_gradient")
        return self.objective_gradient

    def calculate_objective(self, rho) -> float:
        rho = np.asarray(rho)
        filtered_rho = self.filter @ rho.flatten()
        objective, gradient = self.dem.train_model(filtered_rho, self.mesh)
        g = gradient.detach().double().cpu().numpy().flatten()
        self.objective_gradient = (self.filter.T @ g).reshape(rho.shape)
        return float(objective)

    def forward(self, rho):
        return None

    def create_dem_parameters(self):
        body_force = BodyForce(self.mesh, self.parameters.body_force, self.device) if self.parameters.body_force \
            else None
        tractions = [TractionPoints(self.mesh, t) for t in self.parameters.tractions] \
            if self.parameters.tractions else None
        enforcer = ElasticityEnforcer(self.parameters, self.mesh, self.device)
        energy = StrainEnergy(self.mesh, body_force, self.parameters.young_modulus, self.parameters.poisson_ratio,
                              tractions)
        return enforcer, energy

    def create_dem(self, dirichlet_enforcer, objective_calculator) -> DeepEnergyMethod:
        nn_parameters = NNParameters(layer_count=5, neuron_count=68, learning_rate=1.73553, iteration_count=100,
                                     weight_deviation=0.062264, fourier_deviation=0.119297,
                                     activation_function="rrelu", convergence_tolerance=5e-5)
        return DeepEnergyMethod(self.device, self.verbose, 2, nn_parameters, dirichlet_enforcer,
                                objective_calculator)
