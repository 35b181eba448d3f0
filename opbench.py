"""Operator micro-benchmark: the matrix-free P2 state operator alone.

    python opbench.py --nx 1000 --ny 500 --precision mixed --reps 20

Sets up a cantilever (2 x 1, left side clamped, unit downward traction on the
central half of the right side) with a seeded density, runs one state solve so that the operator
coefficients are in place, then times ``reps`` launches of the operator with
CUDA events (an L2 flush before each) and prints one JSON line.  With
``--what solve`` it times whole warm state solves instead.  The timed
launches are bracketed by cudaProfilerStart/Stop, so a profiler started with
``--profile-from-start off`` sees only them.

``--what fluid --n N --reps K`` runs K design iterations of the Stokes-Brinkman
diffuser (1 x 1, parabolic inflow on the left side, a three times faster outflow a
third as wide on the right, penalty 0.1) at N cells per unit length through
``FEMSolver`` and prints the wall time per design iteration and the state solve's
Krylov iterations.
"""
from __future__ import annotations

import argparse
import ctypes
import json

import os
import sys

import torch

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
from topomax_gb300 import fem as F  # noqa: E402
from topomax_gb300.designs import parse_design_dict  # noqa: E402

DESIGN = {"Elasticity": {
    "domain_parameters": dict(width=2.0, height=1.0, fem_step_size=0.002, dem_step_size=0.002,
                              penalties=[3.0], volume_fraction=0.5),
    "problem_parameters": dict(fixed_sides=["Left"], body_force=None,
                               tractions=[dict(side="Right", center=0.5, length=0.5, value=[0.0, -1.0])],
                               filter_radius=0.05, young_modulus=1.0, poisson_ratio=0.3)}}


FLUID = {"Fluid": {
    "domain_parameters": dict(width=1.0, height=1.0, fem_step_size=0.0011, dem_step_size=0.0002, penalties=[0.1],
                              volume_fraction=0.5),
    "problem_parameters": dict(flows=[dict(side="Left", center=0.5, length=1.0, rate=1.0),
                                      dict(side="Right", center=0.5, length=1.0 / 3.0, rate=-3.0)],
                               viscosity=1.0)}}


def time_fluid(args):
    import time
    from topomax_gb300.solver import FEMSolver
    s = FEMSolver(args.n, dict(FLUID, name="diffuser"), precision="fp64", rtol=1e-10, verbose=False, save=False,
                  max_iterations=args.reps)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    h = s.solve()[0.1]
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    solves = len(h["objectives"])
    print(json.dumps({"fluid": "diffuser design loop (FP64)", "N": args.n, "design_iterations": h["iterations"],
                      "s_per_design_iteration": dt / max(1, h["iterations"]),
                      "gmres_iterations_per_solve": s.problem.stats["state_iterations"] / solves,
                      "objective": h["objectives"][-1], "exit": h["exit_condition"],
                      "launches": s.problem.launch_count()}), flush=True)


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--nx", type=int, default=1000)
    ap.add_argument("--ny", type=int, default=500)
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--reps", type=int, default=20)
    ap.add_argument("--what", default="operator", choices=["operator", "solve", "fluid"],
                    help="time operator launches, whole warm state solves, or fluid design iterations")
    ap.add_argument("--n", type=int, default=80, help="fluid: cells per unit length")
    args = ap.parse_args(argv)
    if args.what == "fluid":
        return time_fluid(args)

    dom, par = parse_design_dict(DESIGN)
    mesh = F.RectangleMesh(dom.width, dom.height, args.nx, args.ny)
    V = F.FunctionSpace(mesh, "CG", 1, dof_order="lattice")
    prob = F.ElasticityProblem(mesh, V, dom, par, precision=args.precision, rtol=1e-8)
    prob.set_penalization(3.0)
    g = torch.Generator().manual_seed(0)
    xi = F.Function(V, (torch.rand(V.dim(), generator=g, dtype=torch.float64) * 0.99 + 0.01).cuda())
    prob.forward(xi)

    if args.what == "solve":
        return time_solves(prob, xi, args)
    lib, ctx = prob._ctx._lib, prob._ctx
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MB > L2
    ms = ctypes.c_double(0.0)
    times = []
    torch.cuda.synchronize()
    torch.cuda.profiler.start()
    for _ in range(args.reps):
        flush.fill_(1.0)
        ctx.check(lib.topo_time_operator(ctx.ptr, ctypes.byref(ms), F._stream()))
        times.append(ms.value)
    torch.cuda.profiler.stop()
    torch.cuda.synchronize()

    ndof = 2 * (2 * args.nx + 1) * (2 * args.ny + 1)
    nv = (args.nx + 1) * (args.ny + 1)
    word = 4 if args.precision == "mixed" else 8
    # algorithmic bytes: operand read, result written, density read once
    alg = 2 * ndof * word + nv * word
    times.sort()
    med = times[len(times) // 2]
    print(json.dumps({"operator": f"P2 state operator ({args.precision})", "nx": args.nx, "ny": args.ny,
                      "dofs": ndof, "reps": args.reps, "median_ms": med, "min_ms": times[0],
                      "algorithmic_bytes": alg, "gbs": alg / (med * 1e-3) / 1e9}), flush=True)


def time_solves(prob, xi, args):
    """Warm state solves (the previous displacement as start), each timed with CUDA events."""
    times = []
    its0 = prob.stats["state_iterations"]
    torch.cuda.synchronize()
    torch.cuda.profiler.start()
    for _ in range(args.reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        prob.forward(xi)
        e1.record()
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    torch.cuda.profiler.stop()
    its = (prob.stats["state_iterations"] - its0) / args.reps
    times.sort()
    print(json.dumps({"solve": f"state solve ({args.precision}), warm start", "nx": args.nx, "ny": args.ny,
                      "reps": args.reps, "median_ms": times[len(times) // 2], "min_ms": times[0],
                      "inner_iterations_per_solve": its}), flush=True)


if __name__ == "__main__":
    main()
