"""ctypes wrappers around the CPU emulator of the kernel phases (tests only)."""
from __future__ import annotations

import ctypes

import numpy as np

from tests.native.build_emulator import load

_E = None
C_D = ctypes.c_double
C_I = ctypes.c_int
P_D = ctypes.POINTER(ctypes.c_double)
P_I = ctypes.POINTER(ctypes.c_int)

SIDE = {"Left": 1, "Right": 2, "Top": 4, "Bottom": 8}


def lib():
    global _E
    if _E is None:
        E = load()
        E.emu_dir_ints.restype = C_I
        E.emu_lean_warps.restype = ctypes.c_long
        E.emu_set_segment.argtypes = [C_I]
        E.emu_p2_apply.argtypes = [C_I, C_I, C_I, C_D, C_D, C_D, C_D, C_D, C_D, P_I, P_D, P_D, P_D, C_I]
        E.emu_p1_apply.argtypes = [C_I, C_I, C_I, C_D, C_D, C_D, C_D, P_I, P_D, P_D, C_D, C_D, P_D, P_D, C_I]
        E.emu_transfer.argtypes = [C_I, C_I, C_I, P_I, C_I, C_I, P_I, P_D, P_D, C_I]
        E.emu_kappa.argtypes = [C_I, C_I, C_D, C_D, P_D, P_D]
        E.emu_coarsen_kappa.argtypes = [P_D, C_I, C_I, P_D, C_I, C_I]
        E.emu_build_levels.argtypes = [C_I, C_I, C_I, C_D, C_D, P_I, C_I, C_I, P_I]
        E.emu_sensitivity.argtypes = [C_I, C_I, C_I, C_D, C_D, C_D, C_D, C_D, C_D, P_D, P_D, P_D]
        E.emu_make_dir.argtypes = [C_I, C_I, C_D, C_D, C_I, C_I, P_D, P_I]
        E.emu_load.argtypes = [C_I, C_I, C_D, C_D, P_I, C_I, C_D, C_D, C_D, C_D, C_D, C_I, P_D, P_D]
        E.emu_vertex_weights.argtypes = [C_I, C_I, C_D, C_D, P_D]
        E.emu_smooth.argtypes = [C_I, C_I, C_I, C_I, C_I, C_D, C_D, C_D, C_D, C_D, C_D, P_I, P_D, P_D,
                                 ctypes.POINTER(P_D), P_D, C_I, C_I, P_I, P_D, P_D, C_I, P_D]
        _E = E
    return _E


def dp(a):
    return None if a is None else a.ctypes.data_as(P_D)


def ip(a):
    return a.ctypes.data_as(P_I)


def dir_ints():
    return lib().emu_dir_ints()


def no_dir(NX, NY):
    d = np.zeros(dir_ints(), np.int32)
    d[2] = NX
    d[3] = NY
    return d


def make_dir(nx, ny, hx, hy, sides=(), points=()):
    mask = 0
    for s in sides:
        mask |= SIDE[s]
    pts = np.array(points, dtype=np.float64).reshape(-1)
    out = np.zeros(dir_ints(), np.int32)
    rc = lib().emu_make_dir(nx, ny, hx, hy, mask, len(points), dp(pts) if len(points) else None, ip(out))
    assert rc == 0
    return out


def p2_apply(nx, ny, hx, hy, lam, mu, p, dirv, xi, u, prec=0, mode=0, pmin=1e-6):
    y = np.zeros(2 * (2 * nx + 1) * (2 * ny + 1))
    xi = np.ascontiguousarray(xi, dtype=np.float64)
    uu = None if u is None else np.ascontiguousarray(u, dtype=np.float64)
    lib().emu_p2_apply(prec, nx, ny, hx, hy, lam, mu, p, pmin, ip(dirv), dp(xi), dp(uu), dp(y), mode)
    return y


def set_segment(seg: int) -> None:
    """Cell rows per warp segment of the emulated P2 marches (0: the one-wave rule)."""
    lib().emu_set_segment(int(seg))


def lean_warps() -> int:
    """Warps of the last emulated P2 launch that ran the lean (unchecked) phases."""
    return int(lib().emu_lean_warps())


def p1_apply(NC, nx, ny, hx, hy, lam, mu, dirv, kK, kM, u, kKc=0.0, kMc=0.0, diag=False):
    y = np.zeros(NC * (nx + 1) * (ny + 1))
    u = np.ascontiguousarray(u, dtype=np.float64) if u is not None else None
    lib().emu_p1_apply(NC, nx, ny, hx, hy, lam, mu, ip(dirv), dp(kK), dp(kM), kKc, kMc, dp(u), dp(y), int(diag))
    return y


def restrict(NC, NXf, NYf, dirf, NXc, NYc, dirc, rf):
    out = np.zeros(NC * NXc * NYc)
    lib().emu_transfer(NC, NXf, NYf, ip(dirf), NXc, NYc, ip(dirc), dp(np.ascontiguousarray(rf)), dp(out), 0)
    return out


def prolong(NC, NXf, NYf, dirf, NXc, NYc, dirc, xc):
    out = np.zeros(NC * NXf * NYf)
    lib().emu_transfer(NC, NXf, NYf, ip(dirf), NXc, NYc, ip(dirc), dp(np.ascontiguousarray(xc)), dp(out), 1)
    return out


def kappa(nx, ny, p, xi, pmin=1e-6):
    k = np.zeros(2 * nx * ny)
    lib().emu_kappa(nx, ny, p, pmin, dp(np.ascontiguousarray(xi)), dp(k))
    return k


def coarsen_kappa(kf, nxf, nyf, nxc, nyc):
    kc = np.zeros(2 * nxc * nyc)
    lib().emu_coarsen_kappa(dp(np.ascontiguousarray(kf)), nxf, nyf, dp(kc), nxc, nyc)
    return kc


def build_levels(p2_top, nx, ny, hx, hy, dirv, NC, max_levels=64):
    w = 6 + dir_ints()
    out = np.zeros(max_levels * w, np.int32)
    n = lib().emu_build_levels(int(p2_top), nx, ny, hx, hy, ip(dirv), NC, max_levels, ip(out))
    levels = []
    for l in range(n):
        o = out[l * w:(l + 1) * w]
        levels.append(dict(p2=bool(o[0]), nx=int(o[1]), ny=int(o[2]), NX=int(o[3]), NY=int(o[4]),
                           NC=int(o[5]), dir=o[6:].copy()))
    return levels


def sensitivity(nx, ny, hx, hy, lam, mu, p, u, xi, prec=0, pmin=1e-6):
    b = np.zeros((nx + 1) * (ny + 1))
    lib().emu_sensitivity(prec, nx, ny, hx, hy, lam, mu, p, pmin, dp(np.ascontiguousarray(u)),
                          dp(np.ascontiguousarray(xi)), dp(b))
    return b


def load_vector(nx, ny, W, H, dirv, body_force=None, tractions=()):
    b = np.zeros(2 * (2 * nx + 1) * (2 * ny + 1))
    tr = np.array([[SIDE[t["side"]], t["center"], t["length"], t["value"][0], t["value"][1]]
                   for t in tractions], dtype=np.float64).reshape(-1)
    if body_force is None:
        bf = (0, 0.0, 0.0, 0.0, 0.0, 0.0)
    else:
        bf = (1, body_force["region"]["center"][0], body_force["region"]["center"][1],
              body_force["region"]["radius"], body_force["value"][0], body_force["value"][1])
    lib().emu_load(nx, ny, W, H, ip(dirv), *bf, len(tractions), dp(tr) if len(tractions) else None, dp(b))
    return b


def vertex_weights(nx, ny, hx, hy):
    w = np.zeros((nx + 1) * (ny + 1))
    lib().emu_vertex_weights(nx, ny, hx, hy, dp(w))
    return w


MODE = {"pre": 2, "res": 3, "first": 4, "post2": 5}


def smooth(mode, p2, NC, nx, ny, hx, hy, lam, mu, p, dirv, xi, kK, bufs, cheb, NXc=1, NYc=1, dirc=None,
           xc=None, bc=None, pmin=1e-6, stencil=False, march=False, kM=None):
    """Runs one fused smoothing step in place on bufs = dict(b, dinv, x, x2, r, d)."""
    arrs = [bufs[k] for k in ("b", "dinv", "x", "x2", "r", "d")]
    ptrs = (P_D * 6)(*[dp(a) for a in arrs])
    cheb = np.ascontiguousarray(cheb, dtype=np.float64)
    if dirc is None:
        dirc = no_dir(NXc, NYc)
    lib().emu_smooth(int(p2), NC, MODE[mode], nx, ny, hx, hy, lam, mu, p, pmin, ip(dirv),
                     dp(xi) if xi is not None else None, dp(kK) if kK is not None else None, ptrs, dp(cheb),
                     NXc, NYc, ip(dirc), dp(xc) if xc is not None else None, dp(bc) if bc is not None else None,
                     2 if march else int(stencil), dp(kM) if kM is not None else None)


def coarse_cheb(nx, ny, hx, hy, eps2, b, deg=0):
    """Chebyshev coarse solve of eps2 K + M from x = 0; returns (x, lo, hi, planned degree)."""
    E = lib()
    E.emu_coarse_cheb.argtypes = [C_I, C_I, C_D, C_D, C_D, C_I, P_D, P_D, P_D]
    b = np.ascontiguousarray(b, dtype=np.float64)
    x = np.zeros_like(b)
    info = np.zeros(3)
    rc = E.emu_coarse_cheb(nx, ny, hx, hy, eps2, deg, dp(b), dp(x), dp(info))
    assert rc == 0
    return x, info[0], info[1], int(info[2])


# ---- Stokes-Brinkman fluid ------------------------------------------------------------
def _fluid(E):
    E.emu_fluid_tables.argtypes = [C_D, C_D, P_D]
    E.emu_fluid_bc.argtypes = [C_I, C_I, C_D, C_D, C_I, P_D, P_D]
    E.emu_fluid_bc.restype = C_I
    E.emu_fluid_alpha.argtypes = [C_D, C_D, C_I]
    E.emu_fluid_alpha.restype = C_D
    E.emu_fluid_apply.argtypes = [C_I, C_I, C_D, C_D, C_D, P_D, P_D, P_D, C_I]
    E.emu_fluid_objective.argtypes = [C_I, C_I, C_D, C_D, C_D, C_D, P_D, P_D]
    E.emu_fluid_objective.restype = C_D
    E.emu_fluid_gradient_rhs.argtypes = [C_I, C_I, C_D, C_D, C_D, P_D, P_D, P_D]
    E.emu_p2_node_incidence.argtypes = [C_I, C_I, C_I, C_I, ctypes.POINTER(ctypes.c_longlong), P_I]
    return E


FLUID_TABLES = [  # (name, shape) in FluidTables' member order
    ("area", ()), ("lam6", (12, 3)), ("w6", (12,)), ("lam7", (16, 3)), ("w7", (16,)),
    ("N6", (12, 6)), ("N7", (16, 6)), ("dN6", (2, 12, 6, 2)), ("lap", (2, 6, 6)),
    ("grad", (2, 6, 2, 3)), ("div", (2, 3, 6, 2)),
]


def fluid_tables(hx, hy):
    E = _fluid(lib())
    n = E.emu_fluid_tables_doubles()
    buf = np.zeros(n)
    E.emu_fluid_tables(hx, hy, dp(buf))
    out, off = {}, 0
    for name, shape in FLUID_TABLES:
        size = int(np.prod(shape)) if shape else 1
        out[name] = buf[off:off + size].reshape(shape) if shape else float(buf[off])
        off += size
    assert off == n
    return out


def fluid_bc(nx, ny, W, H, flows):
    E = _fluid(lib())
    f = np.array([[SIDE[s], c, l, r] for s, c, l, r in flows], dtype=np.float64).reshape(-1)
    ub = np.zeros(2 * (2 * nx + 1) * (2 * ny + 1))
    assert E.emu_fluid_bc(nx, ny, W, H, len(flows), dp(f) if len(flows) else None, dp(ub)) == 0
    return ub


def fluid_alpha(q, rho, derivative=False):
    return _fluid(lib()).emu_fluid_alpha(q, rho, int(derivative))


def fluid_apply(nx, ny, W, H, q, rho, x, clamp=False):
    y = np.zeros_like(x)
    _fluid(lib()).emu_fluid_apply(nx, ny, W, H, q, dp(np.ascontiguousarray(rho)), dp(np.ascontiguousarray(x)),
                                  dp(y), int(clamp))
    return y


def fluid_objective(nx, ny, W, H, q, mu, rho, u):
    return _fluid(lib()).emu_fluid_objective(nx, ny, W, H, q, mu, dp(np.ascontiguousarray(rho)),
                                             dp(np.ascontiguousarray(u)))


def fluid_gradient_rhs(nx, ny, W, H, q, rho, u):
    b = np.zeros((nx + 1) * (ny + 1))
    _fluid(lib()).emu_fluid_gradient_rhs(nx, ny, W, H, q, dp(np.ascontiguousarray(rho)),
                                         dp(np.ascontiguousarray(u)), dp(b))
    return b


def p2_node_incidence(a, b, nx, ny):
    t = (ctypes.c_longlong * 6)()
    loc = (ctypes.c_int * 6)()
    n = _fluid(lib()).emu_p2_node_incidence(a, b, nx, ny, t, loc)
    return [(int(t[e]), int(loc[e])) for e in range(n)]
