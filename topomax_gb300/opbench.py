"""Operator micro-benchmark: the matrix-free P2 state operator alone.

    python -m topomax_gb300.opbench --nx 1000 --ny 500 --precision mixed --reps 20

Sets up a cantilever (2 x 1, left side clamped, unit downward traction on the
central half of the right side) with a seeded density, runs one state solve so that the operator
coefficients are in place, then times ``reps`` launches of the operator with
CUDA events (an L2 flush before each) and prints one JSON line.  With
``--what solve`` it times whole warm state solves instead.  The timed
launches are bracketed by cudaProfilerStart/Stop, so a profiler started with
``--profile-from-start off`` sees only them.
"""
from __future__ import annotations

import argparse
import ctypes
import json

import torch

from . import fem as F
from .designs import parse_design_dict

DESIGN = {"Elasticity": {
    "domain_parameters": dict(width=2.0, height=1.0, fem_step_size=0.002, dem_step_size=0.002,
                              penalties=[3.0], volume_fraction=0.5),
    "problem_parameters": dict(fixed_sides=["Left"], body_force=None,
                               tractions=[dict(side="Right", center=0.5, length=0.5, value=[0.0, -1.0])],
                               filter_radius=0.05, young_modulus=1.0, poisson_ratio=0.3)}}


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--nx", type=int, default=1000)
    ap.add_argument("--ny", type=int, default=500)
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--reps", type=int, default=20)
    ap.add_argument("--what", default="operator", choices=["operator", "solve"],
                    help="time operator launches, or whole warm state solves")
    args = ap.parse_args(argv)

    dom, par = parse_design_dict(DESIGN)
    mesh = F.RectangleMesh(dom.width, dom.height, args.nx, args.ny)
    V = F.FunctionSpace(mesh, "CG", 1)
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
