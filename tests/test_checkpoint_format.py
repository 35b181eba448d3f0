"""Saved designs in the reference's format (FEM_src/utils.py:47-109, FEM_src/solver.py:86-89).

The reference pickles {N, domain_size, problem, vector} with the vector in dolfin's serial
CG1 dof order.  ``dolfin_cg1_order`` must reproduce that order: checked against the two
design vectors the reference ships (tests/test_data/FEM/{triangle,diffuser}, copied into
the golden fixtures by tests/golden/make_golden.py) with the oracle's final designs.
"""
import json
import os
import pickle

import numpy as np

from oracle.fem import Design, OracleSolver
from oracle.fluid import FluidDesign, FluidOracleSolver
from topomax_gb300.fem import (RectangleMesh, design_record, dolfin_cg1_order, from_dolfin_order, mesh_to_N,
                               to_dolfin_order)

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _gold(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


def test_order_reproduces_the_reference_triangle_design_exactly():
    gold = _gold("triangle_N10.json")
    run = OracleSolver(gold["N"], Design.from_file(os.path.join(GOLDEN, "designs", "triangle.json"))).solve()[0]
    ref = np.asarray(gold["rho_dolfin"])
    assert np.max(np.abs(to_dolfin_order(run.rho, 10, 10) - ref)) <= 1e-12
    assert np.max(np.abs(np.asarray(run.rho) - ref)) > 0.5  # lattice order is not it


def test_order_reproduces_the_reference_diffuser_design():
    """The fluid oracle reproduces the diffuser only to ~1e-2 (its pressure closure differs
    from MUMPS's); the order still has to line every value up."""
    gold = _gold("diffuser_N20.json")
    with open(os.path.join(GOLDEN, "designs", "diffuser.json")) as f:
        d = FluidDesign.from_dict(json.load(f))
    run = FluidOracleSolver(gold["N"], d, pressure="mean").solve()[0]
    ref = np.asarray(gold["rho_dolfin"])
    err = np.abs(to_dolfin_order(run.rho, 20, 20) - ref)
    assert np.max(err) < 0.05 and np.mean(err) < 1e-3
    assert np.mean(np.abs(np.asarray(run.rho) - ref)) > 0.3


def test_order_is_a_permutation_grown_from_the_top_left_corner():
    for nx, ny in [(1, 1), (3, 2), (80, 40), (7, 19)]:
        p = dolfin_cg1_order(nx, ny)
        assert np.array_equal(np.sort(p), np.arange((nx + 1) * (ny + 1)))
        i, j = p % (nx + 1), p // (nx + 1)
        assert (i[0], j[0]) == (0, ny) and (i[-1], j[-1]) == (nx, 0)
        level = i + (ny - j)
        assert np.all(np.diff(level) >= 0)
        x = np.random.default_rng(0).standard_normal(p.size)
        assert np.array_equal(from_dolfin_order(to_dolfin_order(x, nx, ny), nx, ny), x)


def test_design_record_has_the_reference_layout(tmp_path):
    gold = _gold("triangle_N10.json")
    mesh = RectangleMesh(1.0, 1.0, 10, 10)
    lattice = from_dolfin_order(np.asarray(gold["rho_dolfin"]), 10, 10)
    rec = design_record(lattice, mesh)
    assert set(rec) == {"N", "domain_size", "problem", "vector"}
    assert rec["N"] == gold["N"] and rec["problem"] == gold["problem"] == "design"
    assert list(rec["domain_size"]) == gold["domain_size"]
    assert np.array_equal(rec["vector"], np.asarray(gold["rho_dolfin"]))
    p = tmp_path / "rho.dat"
    with open(p, "wb") as f:
        pickle.dump(rec, f)
    with open(p, "rb") as f:
        back = pickle.load(f)
    assert np.array_equal(back["vector"], rec["vector"])
    assert mesh_to_N(RectangleMesh(2.0, 1.0, 80, 40)) == 40


def test_function_space_host_order():
    """CG1 spaces speak dolfin's dof order on the host by default (arrays handed in and out
    by the API, as the reference's to_array/set_from_array, FEM_src/solver.py:75-79) and the
    lattice order on request; the vector CG2 space is always the lattice."""
    import pytest
    from topomax_gb300.fem import FunctionSpace, VectorFunctionSpace
    gold = _gold("triangle_N10.json")
    mesh = RectangleMesh(1.0, 1.0, 10, 10)
    V = FunctionSpace(mesh, "CG", 1)
    assert V.dof_order == "dolfin"
    ref = np.asarray(gold["rho_dolfin"])
    lattice = V.from_host_order(ref)
    assert np.array_equal(lattice, from_dolfin_order(ref, 10, 10))
    assert np.array_equal(V.to_host_order(lattice), ref)
    L = FunctionSpace(mesh, "CG", 1, dof_order="lattice")
    assert L.dolfin_permutation() is None and np.array_equal(L.from_host_order(ref), ref)
    assert VectorFunctionSpace(mesh).dof_order == "lattice"
    with pytest.raises(ValueError):
        FunctionSpace(mesh, "CG", 1, dof_order="vertex")
