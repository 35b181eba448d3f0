"""Kernel phase logic (run on the CPU through the emulator) against the FP64 oracle.

The GPU kernels are built from phases shared with the host (the P2 column
march: load / compute / finish per lane, with the warp shuffles replaced by
copies between lane states); here they run on the CPU so the segment, halo
and index logic is checked against the oracle's assembled operators before
any GPU run.  The same comparisons run on the GPU in ``test_gpu_parity.py``.
"""
import numpy as np
import pytest

from oracle.fem import Design, FEMOracle, Lattice, lame
from tests import emu


def make_design(**kw):
    base = dict(width=2.0, height=1.0, fem_step_size=0.002, penalties=[3.0], volume_fraction=0.5,
                fixed_sides=["Left"], body_force=None,
                tractions=[dict(side="Right", center=0.5, length=0.5, value=[0.0, -1.0])],
                filter_radius=0.05, young_modulus=1.0, poisson_ratio=0.3)
    base.update(kw)
    return Design(**base)


CASES = [
    # (W, H, nx, ny, sides, p)
    (1.0, 1.0, 3, 2, ["Left"], 3.0),
    (1.0, 1.0, 10, 10, ["Bottom"], 3.0),
    (2.0, 1.0, 33, 9, ["Left", "Right", "Top"], 3.0),      # 2 warps x 2 row segments, ragged
    (2.0, 1.0, 70, 17, [], 3.5),                            # non-integer p, no clamping
    (3.0, 1.0, 65, 24, ["Bottom", "Right"], 4.0),
]


def _problem(W, H, nx, ny, sides, p, seed=0):
    d = make_design(width=W, height=H, fixed_sides=sides)
    L = Lattice(W, H, nx, ny)
    o = FEMOracle(L, d)
    o.set_penalization(p)
    rng = np.random.default_rng(seed)
    xi = rng.uniform(0.01, 1.0, L.n_vertices)
    u = rng.standard_normal(2 * L.n_p2)
    dirv = emu.make_dir(nx, ny, L.hx, L.hy, sides)
    return d, L, o, xi, u, dirv


@pytest.mark.parametrize("case", CASES)
def test_p2_apply_fp64_matches_oracle(case):
    W, H, nx, ny, sides, p = case
    d, L, o, xi, u, dirv = _problem(*case)
    lam, mu = lame(d.young_modulus, d.poisson_ratio)
    y = emu.p2_apply(nx, ny, L.hx, L.hy, lam, mu, p, dirv, xi, u)
    ref = o.apply_state(xi, u)
    assert np.max(np.abs(y - ref)) <= 1e-12 * np.max(np.abs(ref))


@pytest.mark.parametrize("case", CASES[3:])
def test_p2_lean_warps_match_oracle(case):
    """Interior warps skip every per-node test (P2March::lean_region); on these lattices
    some warps take that path and the result still matches the oracle."""
    W, H, nx, ny, sides, p = case
    d, L, o, xi, u, dirv = _problem(*case)
    lam, mu = lame(d.young_modulus, d.poisson_ratio)
    for prec, tol in ((0, 1e-12), (1, 2e-5)):
        y = emu.p2_apply(nx, ny, L.hx, L.hy, lam, mu, p, dirv, xi, u, prec=prec)
        assert emu.lean_warps() > 0
        ref = o.apply_state(xi, u)
        assert np.max(np.abs(y - ref)) <= tol * np.max(np.abs(ref))


def test_p2_march_result_does_not_depend_on_the_segment():
    """The march tile (cell rows per warp segment) is tuned at run time; every node value
    must come out bit for bit the same for any segment length (a segment recomputes the
    cell row below it, so each node sums the same contributions in the same order)."""
    case = CASES[3]
    W, H, nx, ny, sides, p = case
    d, L, o, xi, u, dirv = _problem(*case)
    lam, mu = lame(d.young_modulus, d.poisson_ratio)
    try:
        for prec in (0, 1):
            ys = []
            for seg in (0, 1, 2, 3, 5, 8, ny):
                emu.set_segment(seg)
                ys.append(emu.p2_apply(nx, ny, L.hx, L.hy, lam, mu, p, dirv, xi, u, prec=prec))
            assert all(np.array_equal(ys[0], y) for y in ys[1:])
    finally:
        emu.set_segment(0)


@pytest.mark.parametrize("case", CASES)
def test_p2_apply_pair_fp32_matches_oracle(case):
    """The refinement residual's operator in pair-of-FP32 arithmetic (dd, about 48
    significant bits on the FP32 pipe) against the oracle's assembled FP64 matrix, at
    the FP64 march's tolerance."""
    W, H, nx, ny, sides, p = case
    d, L, o, xi, u, dirv = _problem(*case)
    lam, mu = lame(d.young_modulus, d.poisson_ratio)
    y = emu.p2_apply(nx, ny, L.hx, L.hy, lam, mu, p, dirv, xi, u, prec=2)
    ref = o.apply_state(xi, u)
    assert np.max(np.abs(y - ref)) <= 1e-12 * np.max(np.abs(ref))


def test_p2_pair_fp32_residual_accuracy_at_a_smooth_field():
    """A refinement residual b - K u cancels K u against b to many digits, so the
    operator's rounding must stay small against |K| |u|, not against |K u|: at a smooth
    field riding on a large translation (K u is 1e-5 of |K| |u| here) the pair-of-FP32
    apply agrees with the FP64 one to 1e-13 of |K| |u|."""
    W, H, nx, ny, sides, p = CASES[3]   # no clamped nodes (their identity rows return u itself)
    d, L, o, xi, u, dirv = _problem(*CASES[3])
    lam, mu = lame(d.young_modulus, d.poisson_ratio)
    xs = np.arange(2 * nx + 1) * (L.hx / 2)
    ys = np.arange(2 * ny + 1) * (L.hy / 2)
    X, Y = np.meshgrid(xs, ys)
    us = np.empty(2 * L.n_p2)
    us[0::2] = (250.0 + 0.01 * X * X + 0.003 * X * Y).ravel()
    us[1::2] = (-75.0 + 0.02 * np.sin(3.0 * X) * Y).ravel()
    y64 = emu.p2_apply(nx, ny, L.hx, L.hy, lam, mu, p, dirv, xi, us)
    ydd = emu.p2_apply(nx, ny, L.hx, L.hy, lam, mu, p, dirv, xi, us, prec=2)
    # |K| |u| scale: the operator's row magnitudes times the field's size
    scale = np.max(np.abs(emu.p2_apply(nx, ny, L.hx, L.hy, lam, mu, p, dirv, xi, u))) / np.max(np.abs(u)) * \
        np.max(np.abs(us))
    assert np.max(np.abs(y64)) < 1e-3 * scale   # the cancellation this test is about
    assert np.max(np.abs(ydd - y64)) <= 1e-13 * scale


def test_p2_pair_fp32_residual_at_a_solved_state():
    """At the oracle's solved displacement of a high-contrast design (xi ~ U(0.01, 1),
    p = 3) the pair-of-FP32 operator reproduces K u as closely as the FP64 march does:
    both differ from the oracle's assembled product by ~3e-11 of |b| (the attainable
    residual of this problem in FP64), and from each other by less."""
    W, H, nx, ny, sides, p = 2.0, 1.0, 80, 40, ["Left"], 3.0
    d = make_design(width=W, height=H, fixed_sides=sides)
    L = Lattice(W, H, nx, ny)
    o = FEMOracle(L, d)
    o.set_penalization(p)
    xi = np.random.default_rng(1).uniform(0.01, 1.0, L.n_vertices)
    u = o.state_solve(xi)
    b = o.apply_state(xi, u)
    dirv = emu.make_dir(nx, ny, L.hx, L.hy, sides)
    lam, mu = lame(d.young_modulus, d.poisson_ratio)
    y64 = emu.p2_apply(nx, ny, L.hx, L.hy, lam, mu, p, dirv, xi, u)
    ydd = emu.p2_apply(nx, ny, L.hx, L.hy, lam, mu, p, dirv, xi, u, prec=2)
    nb = np.linalg.norm(b)
    assert np.linalg.norm(y64 - b) <= 1e-10 * nb
    assert np.linalg.norm(ydd - b) <= 1e-10 * nb
    assert np.linalg.norm(ydd - y64) <= 2e-11 * nb


@pytest.mark.parametrize("case", CASES[:3])
def test_p2_apply_fp32_matches_oracle(case):
    W, H, nx, ny, sides, p = case
    d, L, o, xi, u, dirv = _problem(*case)
    lam, mu = lame(d.young_modulus, d.poisson_ratio)
    y = emu.p2_apply(nx, ny, L.hx, L.hy, lam, mu, p, dirv, xi, u, prec=1)
    ref = o.apply_state(xi, u)
    assert np.max(np.abs(y - ref)) <= 2e-5 * np.max(np.abs(ref))


def test_p2_fp32_operator_consistent_at_smooth_fields():
    """The FP32 operator at a solved (smooth, large) displacement of a high-contrast
    design: its arithmetic must stay far below the FP32 representation error of u
    itself (the element products work on u - u_A; products of u itself lose
    ~|K||u|/|Ku| ~ 1e5 in relative accuracy and reach the representation error)."""
    nx, ny = 40, 20
    d = make_design(tractions=[dict(side="Right", center=0.5, length=0.2, value=[0.0, -1.0])])
    L = Lattice(2.0, 1.0, nx, ny)
    o = FEMOracle(L, d)
    o.set_penalization(3.0)
    lam, mu = lame(d.young_modulus, d.poisson_ratio)
    dirv = emu.make_dir(nx, ny, L.hx, L.hy, ["Left"])
    X, Y = np.meshgrid(L.xv, L.yv)
    X, Y = X.ravel(), Y.ravel()
    bars = np.zeros_like(X)  # a truss of solid bars in a void of density 1e-3
    for (x0, y0, x1, y1) in [(0, 0.05, 2, 0.45), (0, 0.95, 2, 0.55), (0, 0.05, 0, 0.95), (0.5, 0.2, 1.0, 0.8),
                             (0, 0.5, 2, 0.5)]:
        t = np.clip(((X - x0) * (x1 - x0) + (Y - y0) * (y1 - y0)) / ((x1 - x0) ** 2 + (y1 - y0) ** 2), 0, 1)
        dist = np.hypot(X - x0 - t * (x1 - x0), Y - y0 - t * (y1 - y0))
        bars = np.maximum(bars, np.clip(1.5 - dist / 0.03, 0, 1))
    xi = 1e-3 + (1 - 1e-3) * bars
    u = o.state_solve(xi)
    f = o.apply_state(xi, u)
    u32 = u.astype(np.float32).astype(np.float64)
    y64 = o.apply_state(xi, u32)
    y32 = emu.p2_apply(nx, ny, L.hx, L.hy, lam, mu, 3.0, dirv, xi, u32, prec=1)
    fn = np.linalg.norm(f)
    representation = np.linalg.norm(y64 - f) / fn   # ~2e-3
    arithmetic = np.linalg.norm(y32 - y64) / fn     # ~6e-5 (~3e-3 without differences)
    assert representation > 5e-4
    assert arithmetic <= 3e-4 and arithmetic <= 0.1 * representation


TINY = [
    # one-cell strips and a single-row warp segment: the halo columns and rows of
    # the march fall outside the lattice on both sides
    (1.0, 1.0, 1, 1, ["Left"], 3.0),
    (1.0, 1.0, 1, 1, [], 3.0),
    (1.0, 1.0, 1, 5, ["Bottom"], 3.0),
    (1.0, 1.0, 5, 1, ["Left"], 3.0),
    (4.0, 1.0, 31, 1, ["Left"], 3.0),
    (4.0, 1.0, 32, 2, ["Top"], 3.0),
]


@pytest.mark.parametrize("case", TINY)
def test_p2_apply_on_tiny_lattices(case):
    W, H, nx, ny, sides, p = case
    d, L, o, xi, u, dirv = _problem(*case)
    lam, mu = lame(d.young_modulus, d.poisson_ratio)
    ref = o.apply_state(xi, u)
    for prec, tol in ((0, 1e-12), (1, 2e-5)):
        y = emu.p2_apply(nx, ny, L.hx, L.hy, lam, mu, p, dirv, xi, u, prec=prec)
        assert np.max(np.abs(y - ref)) <= tol * np.max(np.abs(ref))


@pytest.mark.parametrize("case", CASES + TINY[:2])
def test_p2_diag_matches_oracle(case):
    W, H, nx, ny, sides, p = case
    d, L, o, xi, u, dirv = _problem(*case)
    lam, mu = lame(d.young_modulus, d.poisson_ratio)
    dg = emu.p2_apply(nx, ny, L.hx, L.hy, lam, mu, p, dirv, xi, None, mode=1)
    K = o.stiffness(xi)
    ref = K.diagonal().copy()
    dd = np.concatenate([2 * o.dirichlet_nodes, 2 * o.dirichlet_nodes + 1])
    ref[dd] = 1.0
    assert np.max(np.abs(dg - ref)) <= 1e-12 * np.max(np.abs(ref))


def test_load_vector_matches_oracle():
    designs = [
        make_design(),   # cantilever, traction on the right side
        make_design(width=1.0, height=1.0, fixed_sides=["Bottom"], tractions=None,
                    body_force=dict(region=dict(center=[0.5, 0.5], radius=0.05), value=[0.0, -10.0])),
        make_design(width=3.0, height=1.0, tractions=[
            dict(side="Top", center=1.5, length=1.0, value=[1.0, -2.0]),
            dict(side="Bottom", center=2.95, length=0.1, value=[0.5, 0.0]),
            dict(side="Left", center=0.5, length=1.0, value=[0.0, 3.0])],
            body_force=dict(region=dict(center=[2.9, 0.5], radius=0.05), value=[0.0, -1.0])),
    ]
    for d, (nx, ny) in zip(designs, [(80, 40), (10, 10), (30, 10)]):
        L = Lattice(d.width, d.height, nx, ny)
        o = FEMOracle(L, d)
        dirv = emu.make_dir(nx, ny, L.hx, L.hy, d.fixed_sides)
        b = emu.load_vector(nx, ny, d.width, d.height, dirv, d.body_force, d.tractions or ())
        ref = o.load.copy()
        dd = np.concatenate([2 * o.dirichlet_nodes, 2 * o.dirichlet_nodes + 1])
        ref[dd] = 0.0
        assert np.max(np.abs(b - ref)) <= 1e-14 * max(1.0, np.max(np.abs(ref)))
        tiny = 1e-12 * np.max(np.abs(ref))
        assert np.count_nonzero(np.abs(b) > tiny) == np.count_nonzero(np.abs(ref) > tiny)


def test_vertex_weights_match_oracle():
    d = make_design()
    L = Lattice(2.0, 1.0, 12, 7)
    o = FEMOracle(L, d)
    w = emu.vertex_weights(12, 7, L.hx, L.hy)
    assert np.allclose(w, o.vertex_weights, rtol=0, atol=1e-16)
    assert abs(w.sum() - 2.0) < 1e-13


@pytest.mark.parametrize("p", [3.0, 4.0, 3.3])
def test_sensitivity_rhs_matches_oracle(p):
    d, L, o, xi, u, dirv = _problem(2.0, 1.0, 20, 9, ["Left"], p, seed=3)
    lam, mu = lame(d.young_modulus, d.poisson_ratio)
    u = u * 1e-2
    b = emu.sensitivity(20, 9, L.hx, L.hy, lam, mu, p, u, xi)
    ref = o.sensitivity_rhs(u, xi)
    assert np.max(np.abs(b - ref)) <= 1e-12 * np.max(np.abs(ref))
    b32 = emu.sensitivity(20, 9, L.hx, L.hy, lam, mu, p, u, xi, prec=1)
    assert np.max(np.abs(b32 - ref)) <= 1e-5 * np.max(np.abs(ref))


def test_filter_operator_matches_oracle():
    d = make_design(filter_radius=0.05)
    L = Lattice(2.0, 1.0, 40, 20)
    o = FEMOracle(L, d)
    x = np.random.default_rng(1).standard_normal(L.n_vertices)
    dirv = emu.no_dir(41, 21)
    y = emu.p1_apply(1, 40, 20, L.hx, L.hy, 0.0, 0.0, dirv, None, None, x, kKc=0.05 ** 2, kMc=1.0)
    ref = o.A_filter @ x
    assert np.max(np.abs(y - ref)) <= 1e-13 * np.max(np.abs(ref))
    m = emu.p1_apply(1, 40, 20, L.hx, L.hy, 0.0, 0.0, dirv, None, None, x, kKc=0.0, kMc=1.0)
    assert np.max(np.abs(m - o.M1 @ x)) <= 1e-15


def _free_rows(dirv, NX, NY, NC):
    a, b = np.meshgrid(np.arange(NX), np.arange(NY))
    a = a.ravel()
    b = b.ravel()
    clamped = np.zeros(NX * NY, bool)
    if dirv[0]:
        clamped |= a == 0
    if dirv[1]:
        clamped |= b == 0
    clamped |= a >= dirv[2]
    clamped |= b >= dirv[3]
    for k in range(dirv[4]):
        clamped |= (a == dirv[5 + 2 * k]) & (b == dirv[6 + 2 * k])
    return np.repeat(~clamped, NC)


@pytest.mark.parametrize("nx,ny,sides", [(8, 6, ["Left"]), (33, 9, ["Bottom", "Right"]), (12, 12, [])])
def test_p1_level_is_galerkin_projection_of_p2(nx, ny, sides):
    """K_P1(kappa) x = P^T K_P2(xi) P x on the free rows (exact Galerkin)."""
    W, H, p = 2.0, 1.0, 3.0
    d, L, o, xi, _, dirv = _problem(W, H, nx, ny, sides, p, seed=5)
    lam, mu = lame(d.young_modulus, d.poisson_ratio)
    lv = emu.build_levels(True, nx, ny, L.hx, L.hy, dirv, 2)
    f, c = lv[0], lv[1]
    x1 = np.random.default_rng(7).standard_normal(2 * c["NX"] * c["NY"])
    x1[~_free_rows(c["dir"], c["NX"], c["NY"], 2)] = 0.0
    x2 = emu.prolong(2, f["NX"], f["NY"], f["dir"], c["NX"], c["NY"], c["dir"], x1)
    y2 = emu.p2_apply(nx, ny, L.hx, L.hy, lam, mu, p, f["dir"], xi, x2)
    y1 = emu.restrict(2, f["NX"], f["NY"], f["dir"], c["NX"], c["NY"], c["dir"], y2)
    kk = emu.kappa(nx, ny, p, xi)
    z1 = emu.p1_apply(2, nx, ny, L.hx, L.hy, lam, mu, c["dir"], kk, None, x1)
    free = _free_rows(c["dir"], c["NX"], c["NY"], 2)
    assert np.max(np.abs(z1[free] - y1[free])) <= 1e-12 * np.max(np.abs(y1))


@pytest.mark.parametrize("NC,clamp_all", [(1, False), (2, False), (1, True)])
def test_p1_coarsening_is_galerkin_on_even_grids(NC, clamp_all):
    nx, ny, hx, hy = 16, 8, 0.125, 0.125
    rng = np.random.default_rng(11)
    kf = rng.uniform(1e-3, 1.0, 2 * nx * ny)
    # the filter's mass coefficient is constant: averaging it is exact Galerkin
    km = np.ones(2 * nx * ny) if NC == 1 else None
    dirv = emu.no_dir(nx + 1, ny + 1)
    if NC == 2:
        dirv[0] = 1
    if clamp_all:  # the fluid velocity preconditioner's scalar levels: every side clamped
        dirv = emu.make_dir(nx, ny, hx, hy, ["Left", "Right", "Top", "Bottom"])
    lv = emu.build_levels(False, nx, ny, hx, hy, dirv, NC)
    f, c = lv[0], lv[1]
    assert (c["nx"], c["ny"]) == (8, 4)
    kc = emu.coarsen_kappa(kf, nx, ny, 8, 4)
    kmc = emu.coarsen_kappa(km, nx, ny, 8, 4) if km is not None else None
    lam, mu = 0.5, 0.4
    xc = rng.standard_normal(NC * c["NX"] * c["NY"])
    free_c = _free_rows(c["dir"], c["NX"], c["NY"], NC)
    xc[~free_c] = 0.0
    xf = emu.prolong(NC, f["NX"], f["NY"], f["dir"], c["NX"], c["NY"], c["dir"], xc)
    yf = emu.p1_apply(NC, nx, ny, hx, hy, lam, mu, f["dir"], kf, km, xf)
    yc = emu.restrict(NC, f["NX"], f["NY"], f["dir"], c["NX"], c["NY"], c["dir"], yf)
    zc = emu.p1_apply(NC, 8, 4, 2 * hx, 2 * hy, lam, mu, c["dir"], kc, kmc, xc)
    assert np.max(np.abs(zc[free_c] - yc[free_c])) <= 1e-12 * np.max(np.abs(yc))


def test_level_chain_shapes():
    dirv = emu.make_dir(1000, 500, 0.002, 0.002, ["Left"])
    lv = emu.build_levels(True, 1000, 500, 0.002, 0.002, dirv, 2)
    dims = [(l["nx"], l["ny"]) for l in lv]
    assert dims[0] == (1000, 500) and lv[0]["p2"] and not lv[1]["p2"]
    assert dims[1] == (1000, 500)
    assert dims[-1] == (4, 2) and 2 * lv[-1]["NX"] * lv[-1]["NY"] <= 64
    assert all(l["dir"][0] == 1 for l in lv)          # left side stays clamped
    # odd sizes pad: 125 -> 63
    assert (125, 63) in dims
    # a clamped right side on an odd level clamps the last two coarse columns
    dr = emu.make_dir(10, 10, 0.1, 0.1, ["Right"])
    lv = emu.build_levels(True, 10, 10, 0.1, 0.1, dr, 2)
    p1 = lv[1]
    assert p1["dir"][2] == 10
    c = lv[2]                                         # 10 cells -> 5
    assert c["nx"] == 5 and c["dir"][2] == 5
    c2 = lv[3]                                        # 5 cells -> 3 (padded)
    assert c2["nx"] == 3 and c2["dir"][2] == 2


@pytest.mark.parametrize("level", ["p2", "p2-wide", "p1x2", "p1x1", "p1x2-stencil", "p1x1-stencil", "p1x2-march",
                                   "p1x1-march", "p1x1-dir", "p1x1-dir-stencil", "p1x1-dir-march"])
def test_fused_smoothing_steps_match_composition(level):
    """PRE / RES / FIRST / POST2 against the same steps composed from plain applies
    (P1 levels also through their assembled 7-point stencil and the column march).
    The "-dir" scalar levels are the fluid velocity preconditioner's: every side
    clamped, unit stiffness and a mass coefficient spanning six decades.  "p2-wide"
    is wide and tall enough for interior warps, which take the lean phases."""
    stencil = level.endswith("-stencil")
    march = level.endswith("-march")
    dirichlet = "-dir" in level
    wide = level.endswith("-wide")
    level = level.replace("-stencil", "").replace("-march", "").replace("-dir", "").replace("-wide", "")
    nx, ny, hx, hy, p = (70, 17, 0.025, 0.05, 3.0) if wide else (34, 10, 0.05, 0.05, 3.0)
    lam, mu = lame(1.0, 0.3)
    rng = np.random.default_rng(21)
    xi = rng.uniform(0.05, 1.0, (nx + 1) * (ny + 1))
    p2 = level == "p2"
    NC = 1 if level == "p1x1" else 2
    kM = None
    if p2:
        dirv = emu.make_dir(nx, ny, hx, hy, ["Left"])
        lv = emu.build_levels(True, nx, ny, hx, hy, dirv, 2)
        f, c = lv[0], lv[1]
        A = lambda u: emu.p2_apply(nx, ny, hx, hy, lam, mu, p, dirv, xi, u)
        kK = None
    else:
        dirv = emu.no_dir(nx + 1, ny + 1)
        if NC == 2:
            dirv[0] = 1
        if dirichlet:
            dirv = emu.make_dir(nx, ny, hx, hy, ["Left", "Right", "Top", "Bottom"])
            kM = 10.0 ** rng.uniform(-3.0, 3.0, 2 * nx * ny)
        lv = emu.build_levels(False, nx, ny, hx, hy, dirv, NC)
        f, c = lv[0], lv[1]
        kK = emu.kappa(nx, ny, p, xi) if NC == 2 else np.full(2 * nx * ny, 1.0 if dirichlet else 0.05 ** 2)
        A = lambda u: emu.p1_apply(NC, nx, ny, hx, hy, lam, mu, dirv, kK, kM, u,
                                   kMc=1.0 if NC == 1 and kM is None else 0.0)
    n = NC * f["NX"] * f["NY"]
    free = _free_rows(f["dir"], f["NX"], f["NY"], NC)
    b = rng.standard_normal(n) * free
    x = rng.standard_normal(n) * free
    dinv = 1.0 / (A(np.ones(n)) * 0 + 1.0)        # any positive scaling is fine for the algebra
    dinv = rng.uniform(0.5, 2.0, n)
    dinv[~free] = 1.0
    cheb = np.array([0.7, 0.3, 0.9])
    bufs = dict(b=b.copy(), dinv=dinv.copy(), x=x.copy(), x2=np.zeros(n), r=np.zeros(n), d=np.zeros(n))
    # PRE
    emu.smooth("pre", p2, NC, nx, ny, hx, hy, lam, mu, p, dirv, xi, kK, bufs, cheb, stencil=stencil,
               march=march, kM=kM)
    if wide:
        assert emu.lean_warps() > 0
    d0 = cheb[0] * dinv * b
    ref = d0 + cheb[1] * d0 + cheb[2] * dinv * (b - A(d0))
    assert np.max(np.abs(bufs["x"] - ref)) <= 1e-12 * np.max(np.abs(ref))
    # RES
    bufs["x"] = x.copy()
    emu.smooth("res", p2, NC, nx, ny, hx, hy, lam, mu, p, dirv, xi, kK, bufs, cheb, stencil=stencil,
               march=march, kM=kM)
    rr = b - A(x)
    assert np.max(np.abs(bufs["r"] - rr)) <= 1e-12 * np.max(np.abs(rr))
    # FIRST (coarse correction already added to x) then POST2
    xc = rng.standard_normal(NC * c["NX"] * c["NY"]) * _free_rows(c["dir"], c["NX"], c["NY"], NC)
    u = x + emu.prolong(NC, f["NX"], f["NY"], f["dir"], c["NX"], c["NY"], c["dir"], xc)
    bufs["x"] = u.copy()
    emu.smooth("first", p2, NC, nx, ny, hx, hy, lam, mu, p, dirv, xi, kK, bufs, cheb, stencil=stencil,
               march=march, kM=kM)
    r0 = b - A(u)
    dd0 = cheb[0] * dinv * r0
    # P2: FIRST stores w = u + d0 + c2 Dinv r0 for the second step (r is not needed)
    x2_ref = u + dd0 + cheb[2] * dinv * r0 if p2 else u + dd0
    if not p2:
        assert np.max(np.abs(bufs["r"] - r0)) <= 1e-12 * np.max(np.abs(r0))
    assert np.max(np.abs(bufs["x2"] - x2_ref)) <= 1e-12 * np.max(np.abs(x2_ref))
    emu.smooth("post2", p2, NC, nx, ny, hx, hy, lam, mu, p, dirv, xi, kK, bufs, cheb, stencil=stencil,
               march=march, kM=kM)
    if wide:
        assert emu.lean_warps() > 0
    r1 = r0 - A(dd0)
    ref = u + dd0 + cheb[1] * dd0 + cheb[2] * dinv * r1
    assert np.max(np.abs(bufs["x"] - ref)) <= 1e-12 * np.max(np.abs(ref))
    if p2:
        # FIRST with the coarse correction prolonged on the fly (x itself not updated)
        bufs2 = dict(b=b.copy(), dinv=dinv.copy(), x=x.copy(), x2=np.zeros(n), r=np.zeros(n), d=np.zeros(n))
        emu.smooth("first", p2, NC, nx, ny, hx, hy, lam, mu, p, dirv, xi, kK, bufs2, cheb,
                   NXc=c["NX"], NYc=c["NY"], dirc=c["dir"], xc=xc)
        assert np.max(np.abs(bufs2["x2"] - x2_ref)) <= 1e-12 * np.max(np.abs(x2_ref))
        assert np.array_equal(bufs2["x"], x)


@pytest.mark.parametrize("nx,ny,radius", [(16, 8, 0.05), (24, 12, 0.05), (12, 6, 0.2)])
def test_coarse_chebyshev_solve(nx, ny, radius):
    """Truncated filter hierarchy: the planned interval holds the spectrum of
    Dinv A (A = eps^2 K + M), the node phases equal the textbook recurrence on the
    oracle's assembled matrix, the solve is a symmetric operator, and it reduces
    the error (A-norm) by the planned factor."""
    W, H = 2.0, 1.0
    d = make_design(width=W, height=H, filter_radius=radius)
    L = Lattice(W, H, nx, ny)
    o = FEMOracle(L, d)
    eps2 = (radius / (2.0 * np.sqrt(3.0))) ** 2
    A = (eps2 * o.K1 + o.M1).toarray()
    Dg = np.diag(A)
    rng = np.random.default_rng(4)
    b1, b2 = rng.standard_normal(L.n_vertices), rng.standard_normal(L.n_vertices)
    x1, lo, hi, deg = emu.coarse_cheb(nx, ny, L.hx, L.hy, eps2, b1)
    ev = np.linalg.eigvals(A / Dg[:, None]).real
    assert lo <= ev.min() and ev.max() <= hi
    assert 1 <= deg <= 16
    # textbook Chebyshev iteration (Saad, Alg. 12.1) from x = 0
    theta, delta = 0.5 * (hi + lo), 0.5 * (hi - lo)
    sigma = theta / delta
    rho = 1.0 / sigma
    r = b1.copy()
    dd = r / Dg / theta
    x = np.zeros_like(b1)
    for _ in range(deg - 1):
        x += dd
        r -= A @ dd
        rn = 1.0 / (2.0 * sigma - rho)
        dd = rn * rho * dd + 2.0 * rn / delta * r / Dg
        rho = rn
    x += dd
    assert np.max(np.abs(x1 - x)) <= 1e-12 * np.max(np.abs(x))
    x2, *_ = emu.coarse_cheb(nx, ny, L.hx, L.hy, eps2, b2)
    assert abs(x1 @ b2 - x2 @ b1) <= 1e-12 * abs(x1 @ b1)
    e = np.linalg.solve(A, b1)
    err = np.sqrt((x1 - e) @ A @ (x1 - e) / (e @ A @ e))
    assert err <= 1e-2
