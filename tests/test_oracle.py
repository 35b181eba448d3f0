"""The FP64 oracle against the reference's own known answers (CPU only).

tests/test_elasticity_solver.py:30-55 of the reference: triangle design, N=10,
25 objective evaluations, objective 0.0018191324070894702 at k=24 and the
final rho (121 CG1 values, compared sorted because the reference stores them
in dolfin's dof order).  tests/test_filter.py:25-60: identity at eps=0 and
second-order convergence on a manufactured solution.
"""
import json
import os

import numpy as np
import pytest

from oracle.fem import Design, FEMOracle, Lattice, OracleSolver, rule_degree5, rule_degree6

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def test_triangle_known_answer():
    gold = json.load(open(os.path.join(GOLDEN, "triangle_N10.json")))
    d = Design.from_file(os.path.join(GOLDEN, "designs", "triangle.json"))
    run = OracleSolver(gold["N"], d).solve()[0]
    assert run.exit_condition == "Convergence treshold reached"
    assert run.iterations == gold["iteration"]
    assert abs(run.objectives[-1] - gold["objective"]) <= 1e-12 * gold["objective"]
    assert np.max(np.abs(np.sort(run.rho) - np.array(gold["rho_sorted"]))) <= 1e-10
    assert abs(run.rho.sum() - gold["rho_sum"]) <= 1e-10
    # the reference's own bar (tests/test_elasticity_solver.py:54-55): int (rho - rho*)^2 dx
    # < 1e-14 against its saved design, read in dolfin's dof order
    from topomax_gb300.fem import from_dolfin_order
    e = np.asarray(run.rho) - from_dolfin_order(np.asarray(gold["rho_dolfin"]), 10, 10)
    M1 = FEMOracle(Lattice(1.0, 1.0, 10, 10), d).M1
    assert float(e @ (M1 @ e)) < 1e-14


@pytest.mark.parametrize("rule", [rule_degree5, rule_degree6])
def test_quadrature_rules_integrate_monomials_exactly(rule):
    from math import factorial
    pts, w = rule()
    deg = 5 if rule is rule_degree5 else 6
    assert abs(w.sum() - 1.0) < 1e-14
    for a in range(deg + 1):
        for b in range(deg + 1 - a):
            # int_T l0^a l1^b / |T| = 2 a! b! / (a+b+2)!
            exact = 2.0 * factorial(a) * factorial(b) / factorial(a + b + 2)
            num = np.sum(w * pts[:, 0] ** a * pts[:, 1] ** b)
            assert abs(num - exact) < 5e-14


def _filter_design(eps):
    return Design(width=1.0, height=1.0, fem_step_size=1.0, penalties=[3.0], volume_fraction=0.5,
                  fixed_sides=[], body_force=None, tractions=None, filter_radius=eps, young_modulus=1.0,
                  poisson_ratio=0.3)


def test_filter_identity_at_zero_radius():
    o = FEMOracle(Lattice(1.0, 1.0, 10, 10), _filter_design(0.0))
    np.random.seed(198)
    rho = np.random.random(o.L.n_vertices)
    assert np.max(np.abs(o.filter_apply(rho) - rho)) < 1e-14


def test_filter_manufactured_solution_converges_second_order():
    eps = np.e / np.pi
    errs = []
    Ns = [10, 20, 40, 80]
    for N in Ns:
        o = FEMOracle(Lattice(1.0, 1.0, N, N), _filter_design(eps))
        X, Y = o.L.vertex_coords()
        rho = (8 * eps * eps * np.pi ** 2 + 1) * np.cos(2 * np.pi * X) * np.cos(2 * np.pi * Y)
        xi = o.filter_apply(rho)
        exact = np.cos(2 * np.pi * X) * np.cos(2 * np.pi * Y)
        errs.append(np.sqrt(o.integrate((xi - exact) ** 2)))
    slope = np.polyfit(np.log(Ns), np.log(errs), 1)[0]
    assert slope <= -2 + 0.05


def test_design_parser_matches_reference_semantics(tmp_path):
    from topomax_gb300.designs import Side, parse_design, parse_design_dict
    dom, par = parse_design(os.path.join(GOLDEN, "designs", "cantilever.json"))
    assert dom.width == 3.0 and par.fixed_sides == [Side.LEFT]
    assert par.body_force.region.radius == 0.05 and par.tractions is None
    with pytest.raises(ValueError):
        parse_design_dict({"Elasticity": {}, "Fluid": {}})
    with pytest.raises(ValueError):
        Side.from_string("Middle")
    # every design the reference ships parses (fluid designs into Flow records)
    from topomax_gb300.designs import FluidParameters, Flow
    for name in sorted(os.listdir(os.path.join(GOLDEN, "designs"))):
        dom, par = parse_design(os.path.join(GOLDEN, "designs", name))
        if isinstance(par, FluidParameters):
            assert all(isinstance(f, Flow) and isinstance(f.side, Side) for f in par.flows)
            assert par.flows[0].to_tuple()[1:] == (par.flows[0].center, par.flows[0].length, par.flows[0].rate)


def test_oracle_projection_failure_paths():
    """The oracle's projection follows src/solver.py:149-186 and src/utils.py:138-157: an
    unreachable volume ends in smart_brentq's ValueError; a Newton breakdown falls back to
    the bracketing search (radius doubled from 2) and still meets the volume."""
    import pytest
    from oracle.fem import Design, OracleSolver, expit
    d = Design(width=2.0, height=1.0, fem_step_size=0.002, penalties=[3.0], volume_fraction=0.5,
               fixed_sides=["Left"], body_force=None,
               tractions=[dict(side="Right", center=0.5, length=0.5, value=[0.0, -1.0])],
               filter_radius=0.05, young_modulus=1.0, poisson_ratio=0.3)
    s = OracleSolver(10, d)
    n = s.lattice.n_vertices
    with pytest.raises(ValueError, match=r"^f\(-max_radius\) and f\(max_radius\) must have different signs!$"):
        s.project(np.zeros(n), 3.0)
    half = -40.0 + np.random.default_rng(5).uniform(-0.5, 0.5, n)
    psi = s.project(half, s.volume)
    c = float(np.mean(psi - half))
    assert 32.0 < c < 64.0 and np.allclose(psi - half, c, rtol=0, atol=1e-13)
    assert abs(s.integrate(expit(psi)) - s.volume) <= 1e-12
