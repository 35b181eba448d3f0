"""Benchmark: design iterations per second of the elasticity design loop on GB300.

Workload (default): the cantilever of the design-iteration metric at 4.0M
displacement dofs -- domain 2x1, 1000x500 squares split into 4M... no: into
1,000,000 triangles with vector P2 (4,006,002 dofs), left side clamped,
traction (0,-1) on the right side centred at y=0.5 with length 0.5, E=1,
nu=0.3, p=3, volume fraction 0.5, filter radius 0.05.  rho is drawn i.i.d.
U(0.01, 1) per vertex from torch.Generator seed 0 (FP64) and filtered by the
first objective evaluation.  Every linear solve runs to relative residual
1e-8.  One step = one pass of the reference's design-loop body
(src/solver.py:253-266): gradient (sensitivity + filter solve), EMD step with
volume projection, design update, objective (filter solve + state solve +
compliance).

``value``: mixed precision (FP32 multigrid CG inside FP64 refinement), design
resident in HBM.  ``e2e``: the same step through the reference-facing API with
host numpy buffers (the reference's own to_array / project / set_from_array
pattern), host<->device copies inside the timed region.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "design iters/sec at 4M DOF: FP32+FP64-refine vs plain FP64 on GB300, compliance err<=1e-6"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--nx", type=int, default=1000)
    ap.add_argument("--ny", type=int, default=500)
    ap.add_argument("--rtol", type=float, default=1e-8)
    ap.add_argument("--fp64-steps", type=int, default=3)
    ap.add_argument("--no-e2e", action="store_true")
    return ap.parse_args()


def design_dict(step=0.002):
    return {"Elasticity": {
        "domain_parameters": dict(width=2.0, height=1.0, fem_step_size=step, dem_step_size=step, penalties=[3.0],
                                  volume_fraction=0.5),
        "problem_parameters": dict(fixed_sides=["Left"], body_force=None,
                                   tractions=[dict(side="Right", center=0.5, length=0.5, value=[0.0, -1.0])],
                                   filter_radius=0.05, young_modulus=1.0, poisson_ratio=0.3)}}


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self):
        self.p = None
        self.path = os.path.join(ROOT, "gpurun_out", "bench_clocks.csv")

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200", "-i", str(self._index())],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    @staticmethod
    def _index():
        v = os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0]
        return v if v.isdigit() else "0"

    def stop(self):
        if not self.p:
            return None
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.close()
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = max(mx, float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def run_reference(args):
    from oracle.fem import Design, OracleSolver
    print(json.dumps({"impl": "reference", "unavailable": "not wired yet"}))


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    import torch
    import topomax_gb300 as tg
    from topomax_gb300 import fem as F
    from topomax_gb300.designs import parse_design_dict

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
    dom, par = parse_design_dict(design_dict())
    mesh = tg.RectangleMesh(2.0, 1.0, args.nx, args.ny)
    V = tg.FunctionSpace(mesh, "CG", 1)

    def make(precision):
        prob = tg.ElasticityProblem(mesh, V, dom, par, precision=precision, rtol=args.rtol)
        prob.set_penalization(3.0)
        return prob

    g = torch.Generator().manual_seed(0)
    rho0 = (torch.rand(V.dim(), generator=g, dtype=torch.float64) * 0.99 + 0.01).cuda()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def device_loop(prob, steps, warmup):
        from topomax_gb300.solver import FEMSolver  # noqa
        lib = prob._ctx._lib
        rho = F.Function(V, rho0.clone())
        psi = torch.log(rho.tensor / (1 - rho.tensor))
        C = prob.calculate_objective(rho)
        import ctypes
        times = []
        objs = [C]
        for k in range(warmup + steps):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            gvec = prob.calculate_objective_gradient()
            new_psi = torch.empty_like(psi)
            c = ctypes.c_double(0)
            prob._ctx.check(lib.topo_emd_step(prob._ctx.ptr, F._ptr(psi), F._ptr(gvec.tensor), 0.002 * (k + 1),
                                              1.0, F._ptr(new_psi), ctypes.byref(c), F._stream()))
            d = ctypes.c_double(0)
            prob._ctx.check(lib.topo_emd_finish(prob._ctx.ptr, F._ptr(new_psi), F._ptr(psi), F._ptr(rho.tensor),
                                                ctypes.byref(d), F._stream()))
            psi = new_psi
            C = prob.calculate_objective(rho)
            e1.record()
            torch.cuda.synchronize()
            if k >= warmup:
                times.append(e0.elapsed_time(e1))
            objs.append(C)
        return times, objs

    prob = make("mixed")
    clocks = Clocks()
    torch.cuda.synchronize()
    clocks.start()
    t0 = time.time()
    times, objs = device_loop(prob, args.steps, args.warmup)
    wall = time.time() - t0
    ck = clocks.stop()
    ms = float(np.sum(times)) / len(times)
    st = dict(prob.stats)
    del prob
    torch.cuda.empty_cache()
    prob64 = make("fp64")
    times64, objs64 = device_loop(prob64, args.fp64_steps, 1)
    ms64 = float(np.sum(times64)) / len(times64)
    n_iter = min(len(objs), len(objs64))
    rel = max(abs(a - b) / abs(b) for a, b in zip(objs[:n_iter], objs64[:n_iter]))
    out = {
        "metric": METRIC, "value": 1000.0 / ms, "unit": "design_iters/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
        "config": {"workload": f"cantilever 2x1, {args.nx}x{args.ny} squares, P2 dofs "
                               f"{2 * (2 * args.nx + 1) * (2 * args.ny + 1)}, rtol {args.rtol}",
                   "l2": "flushed (256 MB write) before every step"},
        "fp64": {"value": 1000.0 / ms64, "ms_per_step": ms64, "steps": len(times64)},
        "mixed_over_fp64": ms64 / ms, "compliance_rel_diff_vs_fp64": rel,
        "clocks": ck, "stats": st, "wall_s": wall,
    }
    print(json.dumps(out))


if __name__ == "__main__":
    main()
