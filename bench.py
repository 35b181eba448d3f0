"""Benchmark: design iterations per second of the elasticity design loop on GB300.

Workload: the cantilever of the design-iteration metric at 4.0M displacement
dofs -- domain 2x1, 1000x500 squares (1,000,000 triangles, vector P2:
4,006,002 dofs), left side clamped, traction (0,-1) on the right side centred
at y=0.5 with length 0.5, E=1, nu=0.3, p=3, volume fraction 0.5, filter
radius 0.05.  rho is drawn i.i.d. U(0.01, 1) per vertex (torch.Generator seed
0, FP64) and filtered by the first objective evaluation.  Every linear solve
runs to relative residual 1e-8.

One step = one pass of the reference's design-loop body (src/solver.py:253-266):
objective gradient (sensitivity + filter solve), entropic mirror-descent step
with the Newton volume projection, design update, objective (filter solve +
state solve + compliance).

* ``value``: mixed precision (FP32 multigrid CG inside FP64 flexible GMRES),
  design resident in HBM, CUDA events per step, L2 flushed (256 MB write)
  before every step.
* ``fp64``: the same loop with plain FP64 multigrid CG (the metric's
  comparison) over the same design steps as the timed mixed steps (by default all
  of them), and the max relative compliance difference between the two.
* ``e2e``: the same steps (same warm-up, same step sizes) through the
  reference-facing API with host (pinned) arrays, as the reference's
  Solver.step/project/set_from_array drive it.
* ``kernels``: time and HBM GB/s per kernel family on the headline grid (the
  library's kernel clock over host-driven design iterations; ``sum_ms_per_step``
  against ``ms_per_step`` shows what launches and host round trips add).
* ``c2_2000x1000``: the same loop on the 2000x1000 grid of the throughput
  configuration (16,012,002 dofs), with its operator's bandwidth, and the same
  per-family table there (``kernels``).
* ``c4_batch``: the 64-design ragged batch (domain 2x1, N in {100..300}), run one
  design after another and by concurrent workers; ``march_tiles``: the tiles the
  march-kernel autotuner chose in this run.
* ``fluid``: the Stokes-Brinkman diffuser's design loop on the GPU beside the fluid
  oracle on the host.
* ``solver_iterations``: inner Krylov iterations of the headline problem over its
  device-resident and end-to-end runs (warm-ups included), and per timed step of the
  device-resident run (``per_timed_step``: the state solve's, and the two filter
  solves' together).
* ``roofline``: the dominant kernel (the FP32 matrix-free P2 operator),
  algorithmic bytes 2*V2u*4 + V1*4 per launch over its CUDA-event duration
  measured in this run, against the measured HBM copy bandwidth.
* ``cpu_baseline`` / ``--impl reference``: the FP64 oracle (the reference
  algorithm: filter solves, sparse assembly + SuperLU, Newton projection) timed
  on this host's cores over real design iterations of the same loop, on the
  --ref-grid cantilever (160x80 by default: SuperLU cannot factor the 1000x500
  state matrix on a 62 GB host).  ``same_grid``: the GPU loop on that grid, so
  that a same-grid comparison exists beside the headline one.  ``size_sweep``
  (--size-sweep, off by default): the GPU loop and the oracle side by side on
  several grids, design iterations/s each.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "design iters/sec at 4M DOF: FP32+FP64-refine vs plain FP64 on GB300, compliance err≤1e-6"
UNIT = "design_iters/s"
STEP = 0.002           # EMD step size of the benchmark design
PENALTY = 3.0


def job_throughput(total_ms: float, steps: int, world: int, dist=None, device="cuda"):
    """Replicas: the job takes as long as its slowest rank, and every rank did `steps`
    design iterations.  Returns (max-over-ranks total ms, whole-job iterations/s)."""
    if dist is not None:
        import torch
        t = torch.tensor([float(total_ms)], device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    return total_ms, world * steps / (total_ms / 1000.0)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--nx", type=int, default=1000)
    ap.add_argument("--ny", type=int, default=500)
    ap.add_argument("--rtol", type=float, default=1e-8)
    ap.add_argument("--fp64-steps", type=int, default=None, help="default: --steps (the same design steps)")
    ap.add_argument("--e2e-steps", type=int, default=None, help="default: --steps (the same design steps)")
    ap.add_argument("--c2-steps", type=int, default=50,
                    help="timed design iterations on the 2000x1000 grid (16,012,002 dofs); 0 skips it")
    ap.add_argument("--c4-designs", type=int, default=64,
                    help="designs of the ragged batch (domain 2x1, N in {100..300}); 0 skips the batch leg")
    ap.add_argument("--c4-iterations", type=int, default=20, help="design iterations per design in the batch leg")
    ap.add_argument("--c4-workers", type=int, default=8, help="concurrent workers (streams) of the batched run")
    ap.add_argument("--fluid-n", type=int, default=40,
                    help="cells per unit length of the fluid (Stokes-Brinkman diffuser) leg; 0 skips it")
    ap.add_argument("--fluid-iterations", type=int, default=3, help="design iterations of the fluid leg")
    ap.add_argument("--kernel-steps", type=int, default=2,
                    help="host-driven design iterations on the 2000x1000 grid timed kernel by kernel "
                         "(HBM GB/s per kernel family); 0 skips them")
    ap.add_argument("--ref-grid", default="160x80",
                    help="grid of the CPU oracle legs (cpu_baseline, --impl reference) and of the GPU same-grid leg")
    ap.add_argument("--cpu-steps", type=int, default=5, help="timed oracle design iterations of cpu_baseline")
    ap.add_argument("--size-sweep", default="",
                    help="comma-separated 2:1 grids (e.g. 80x40,160x80,320x160) timed on the GPU (mixed) and "
                         "by the CPU oracle (--cpu-steps iterations each); empty skips the sweep")
    ap.add_argument("--clocks-dir", default=None,
                    help="keep the raw nvidia-smi samples of the timed region here (default: a temporary file)")
    args = ap.parse_args()
    if args.fp64_steps is None:
        args.fp64_steps = args.steps
    if args.e2e_steps is None:
        args.e2e_steps = args.steps
    return args


def design_dict():
    return {"Elasticity": {
        "domain_parameters": dict(width=2.0, height=1.0, fem_step_size=STEP, dem_step_size=STEP,
                                  penalties=[PENALTY], volume_fraction=0.5),
        "problem_parameters": dict(fixed_sides=["Left"], body_force=None,
                                   tractions=[dict(side="Right", center=0.5, length=0.5, value=[0.0, -1.0])],
                                   filter_radius=0.05, young_modulus=1.0, poisson_ratio=0.3)}}


def dofs(nx, ny):
    return 2 * (2 * nx + 1) * (2 * ny + 1)


# ----------------------------------------------------------------------------
# CPU side: the oracle (the reference algorithm) on this host
# ----------------------------------------------------------------------------
def seeded_density(nx, ny):
    """rho ~ i.i.d. U(0.01, 1) per CG1 vertex (torch.Generator seed 0, FP64, lattice order)."""
    import torch
    g = torch.Generator().manual_seed(0)
    return torch.rand((nx + 1) * (ny + 1), generator=g, dtype=torch.float64) * 0.99 + 0.01


def _grid(text):
    nx, ny = (int(v) for v in text.lower().split("x"))
    if nx != 2 * ny:
        raise SystemExit(f"grid {text}: the cantilever is 2x1, so nx must be 2*ny")
    return nx, ny


def _blas_threads():
    try:
        from threadpoolctl import threadpool_info
        return str(max((i.get("num_threads", 1) for i in threadpool_info() if i.get("user_api") == "blas"),
                       default=1))
    except Exception:
        for var in ("OPENBLAS_NUM_THREADS", "OMP_NUM_THREADS"):
            if os.environ.get(var):
                return os.environ[var]
        return "the BLAS library's default"


class OracleLoop:
    """The FP64 oracle's design loop (src/solver.py:253-266) on one nx x ny cantilever,
    built once.  Each step() is one design iteration: the objective gradient (filter
    solve), the entropic mirror-descent step with the Newton volume projection, the
    design update and the objective (filter solve, sparse P2 assembly, SuperLU state
    solve, compliance) -- the same pass the GPU arm times, from the same seeded design."""

    def __init__(self, nx, ny):
        from oracle.fem import Design, OracleSolver, logit
        pp = design_dict()["Elasticity"]["problem_parameters"]
        d = Design(width=2.0, height=1.0, fem_step_size=STEP, penalties=[PENALTY], volume_fraction=0.5,
                   fixed_sides=["Left"], body_force=None, tractions=pp["tractions"], filter_radius=0.05,
                   young_modulus=1.0, poisson_ratio=0.3)
        self.s = OracleSolver(ny, d)
        assert (self.s.lattice.nx, self.s.lattice.ny) == (nx, ny)
        self.s.problem.set_penalization(PENALTY)
        rho = seeded_density(nx, ny).numpy()
        self.psi = logit(rho)
        self.s.problem.calculate_objective(rho)
        self.k = 0

    def step(self):
        from oracle.fem import expit
        self.psi = self.s.step(self.psi, STEP * (self.k + 1))
        self.k += 1
        return self.s.problem.calculate_objective(expit(self.psi))


def time_oracle(nx, ny, steps, warmup):
    """Measured oracle design iterations on the nx x ny grid: (iterations/s, seconds per step)."""
    loop = OracleLoop(nx, ny)
    for _ in range(warmup):
        loop.step()
    t0 = time.perf_counter()
    for _ in range(steps):
        loop.step()
    sec = (time.perf_counter() - t0) / steps
    return 1.0 / sec, sec


def oracle_sample(nx, ny, steps, warmup, sec):
    return (f"{steps} timed FP64 oracle design iterations (after {warmup} untimed) on the {nx}x{ny} cantilever "
            f"({dofs(nx, ny)} P2 dofs; the reference algorithm: filter solves, sparse P2 assembly, SuperLU with "
            f"a minimum-degree ordering, Newton volume projection), {sec:.2f} s each, measured on this host; "
            f"SuperLU and the assembly run on one core, BLAS ({_blas_threads()} threads) is not on the path; "
            f"host cores {os.cpu_count()}")


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    nx, ny = _grid(args.ref_grid)
    value, sec = time_oracle(nx, ny, args.steps, args.warmup)
    sample = oracle_sample(nx, ny, args.steps, args.warmup, sec)
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": 1000.0 * sec, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded U(0.01,1) density)", "impl": "reference",
           "config": {"workload": f"cantilever 2x1, {nx}x{ny} squares, vector P2, {dofs(nx, ny)} dofs "
                                  f"(sized so that the run ends in about a minute; on the GPU arm's "
                                  f"{args.nx}x{args.ny} grid SuperLU cannot factor the state matrix on a "
                                  f"62 GB host)",
                      "same_config": False},
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": 1, "kind": "port", "sample": sample},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


# ----------------------------------------------------------------------------
# GPU side
# ----------------------------------------------------------------------------
class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, tag, out_dir=None):
        self.p = None
        self.path = os.path.join(out_dir or tempfile.gettempdir(), f"bench_clocks_{tag}_{os.getpid()}.csv")

    def start(self, index):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200", "-i", str(index)],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

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


def measured_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def ncu_counts(nx, ny):
    """DRAM bytes and executed FP32 thread instructions per launch of the FP32 operator from
    the committed ncu summary, scaled to this grid by the dof count."""
    try:
        with open(os.path.join(ROOT, "profiles", "p2_operator_fp32_traffic.json")) as f:
            d = json.load(f)
        s = dofs(nx, ny) / d["dofs"]
        return d["bytes_per_launch"] * s, d.get("fp32_thread_inst_per_launch", 0) * s or None
    except Exception:
        return None, None


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    import ctypes
    import torch
    import topomax_gb300 as tg
    from topomax_gb300 import fem as F
    from topomax_gb300.designs import parse_design_dict
    from topomax_gb300.solver import FEMSolver  # noqa: F401  (API import check)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    dom, par = parse_design_dict(design_dict())
    mesh = tg.RectangleMesh(2.0, 1.0, args.nx, args.ny)
    V = tg.FunctionSpace(mesh, "CG", 1, dof_order="lattice")
    nv = V.dim()
    rho0 = seeded_density(args.nx, args.ny)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def make(precision):
        prob = tg.ElasticityProblem(mesh, V, dom, par, precision=precision, rtol=args.rtol)
        prob.set_penalization(PENALTY)
        return prob

    def launches(prob):
        n = ctypes.c_int64(0)
        prob._ctx._lib.topo_launch_count(prob._ctx.ptr, ctypes.byref(n))
        return n.value

    def device_loop(prob, steps, warmup, time_operator=False, profile=False, space=None, start=None, on_start=None,
                    step_iterations=None):
        """Design-resident loop; returns per-step ms (CUDA events), objectives, launches, operator ms.

        With profile=True the timed steps are bracketed by cudaProfilerStart/Stop, so that a
        profiler run with --profile-from-start off records exactly those launches.  on_start()
        runs once, after the warm-up steps.  step_iterations (a dict of two lists), when
        given, receives each timed step's inner Krylov iterations: its state solve's, and
        its two filter solves' together (host counters the solves return anyway)."""
        lib = prob._ctx._lib
        rho = F.Function(space or V, (start if start is not None else rho0).cuda())
        psi = torch.log(rho.tensor / (1 - rho.tensor))
        objs = [prob.calculate_objective(rho)]
        times, op_ms = [], []
        l0 = 0
        for k in range(warmup + steps):
            if k == warmup:
                barrier()
                l0 = launches(prob)
                if on_start is not None:
                    on_start()
                if profile:
                    torch.cuda.profiler.start()
            flush.zero_()
            it0 = dict(prob.stats)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            gvec = prob.calculate_objective_gradient()
            new_psi = torch.empty_like(psi)
            c = ctypes.c_double(0)
            prob._ctx.check(lib.topo_emd_step(prob._ctx.ptr, F._ptr(psi), F._ptr(gvec.tensor), STEP * (k + 1),
                                              prob.domain_size[0] * prob.domain_size[1] * 0.5, F._ptr(new_psi),
                                              ctypes.byref(c), F._stream()))
            d = ctypes.c_double(0)
            prob._ctx.check(lib.topo_emd_finish(prob._ctx.ptr, F._ptr(new_psi), F._ptr(psi), F._ptr(rho.tensor),
                                                ctypes.byref(d), F._stream()))
            psi = new_psi
            objs.append(prob.calculate_objective(rho))
            e1.record()
            torch.cuda.synchronize()
            if k >= warmup:
                times.append(e0.elapsed_time(e1))
                if step_iterations is not None:
                    step_iterations["state"].append(prob.stats["state_iterations"] - it0["state_iterations"])
                    step_iterations["filter"].append(prob.stats["filter_iterations"] - it0["filter_iterations"])
        barrier()
        if profile:
            torch.cuda.profiler.stop()
        nl = launches(prob) - l0
        if time_operator:
            for _ in range(10):
                flush.zero_()
                ms = ctypes.c_double(0)
                prob._ctx.check(lib.topo_time_operator(prob._ctx.ptr, ctypes.byref(ms), F._stream()))
                op_ms.append(ms.value)
        return times, objs, nl, op_ms

    def e2e_loop(prob, steps, warmup):
        """Reference-facing API with host arrays: Solver.step / project / set_from_array pattern."""
        rho = F.Function(V, rho0.cuda())
        rho_host = rho0.clone().pin_memory()
        psi_host = torch.log(rho_host / (1 - rho_host))
        half_host = torch.empty_like(rho_host).pin_memory()
        prob.calculate_objective(rho)
        volume = prob.domain_size[0] * prob.domain_size[1] * 0.5
        solver = _E2ESolver(prob, V, volume)
        times = []
        for k in range(warmup + steps):  # the same EMD step sizes as the device loop's steps
            flush.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            gdev = prob.calculate_objective_gradient()
            g_host = gdev.tensor.to("cpu", non_blocking=False)                 # D2H: to_array(gradient)
            torch.sub(psi_host, g_host, alpha=STEP * (k + 1), out=half_host)
            psi_dev = solver.project(half_host, volume)                          # H2D half, projection on device
            psi_host = psi_dev.to("cpu")                                         # D2H psi
            rho_host = torch.sigmoid(psi_host).pin_memory()
            C = prob.calculate_objective(rho_host)                               # H2D rho, D2H objective
            torch.cuda.synchronize()
            if k >= warmup:
                times.append(time.perf_counter() - t0)
            assert math.isfinite(C)
        return times

    # --- mixed precision: value, roofline, launches
    prob = make("mixed")
    clocks = Clocks(f"r{rank}", args.clocks_dir)
    barrier()
    clocks.start(local if not os.environ.get("CUDA_VISIBLE_DEVICES") else 0)
    per_step = {"state": [], "filter": []}
    times, objs, nlaunch, op_ms = device_loop(prob, args.steps, args.warmup, time_operator=True, profile=True,
                                              step_iterations=per_step)
    ck = clocks.stop()
    total_ms, value = job_throughput(float(np.sum(times)), args.steps, world, dist)
    ms = total_ms / args.steps
    e2e_times = e2e_loop(prob, args.e2e_steps, args.warmup)
    e2e_value = 1.0 / float(np.mean(e2e_times))
    stats = dict(prob.stats)
    stats["per_timed_step"] = per_step
    del prob
    torch.cuda.empty_cache()

    # --- plain FP64 comparison: the same design steps as the first timed mixed steps
    prob64 = make("fp64")
    times64, objs64, _, _ = device_loop(prob64, args.fp64_steps, args.warmup)
    ms64 = float(np.mean(times64))
    ms_mixed_same = float(np.mean(times[:len(times64)]))
    del prob64
    torch.cuda.empty_cache()
    n = min(len(objs), len(objs64))
    comp_rel = max(abs(a - b) / abs(b) for a, b in zip(objs[:n], objs64[:n]))

    # --- the 2000 x 1000 grid of the throughput configuration (16,012,002 P2 dofs)
    c2 = None
    if args.c2_steps > 0:
        mesh2 = tg.RectangleMesh(2.0, 1.0, 2000, 1000)
        V2 = tg.FunctionSpace(mesh2, "CG", 1, dof_order="lattice")
        rho02 = seeded_density(2000, 1000)
        prob2 = tg.ElasticityProblem(mesh2, V2, dom, par, precision="mixed", rtol=args.rtol)
        prob2.set_penalization(PENALTY)
        t2, _, _, op2 = device_loop(prob2, args.c2_steps, args.warmup, time_operator=True, space=V2, start=rho02)
        alg2 = 2 * dofs(2000, 1000) * 4 + V2.dim() * 4
        c2 = {"workload": "cantilever 2x1, 2000x1000 squares, vector P2, 16012002 dofs, rtol %g" % args.rtol,
              "value": 1000.0 / float(np.mean(t2)), "ms_per_step": float(np.mean(t2)), "steps": len(t2),
              "operator_launch_ms": float(np.mean(op2)), "operator_gbs": alg2 / (float(np.mean(op2)) * 1e-3) / 1e9}
        del prob2
        torch.cuda.empty_cache()
        if args.kernel_steps > 0 and world == 1:
            c2["kernels"] = kernel_table(tg, mesh2, V2, dom, par, rho02, device_loop, args, measured_peak()[0])
            c2["kernels"]["sum_ms_per_step"] = sum(r["ms_per_step"] for r in c2["kernels"]["families"])
            torch.cuda.empty_cache()

    # --- the same per-family table on the headline grid; its sum against the recorded
    # step shows what the host-driven launches and round trips add
    kernels = None
    if args.kernel_steps > 0 and world == 1:
        kernels = kernel_table(tg, mesh, V, dom, par, rho0, device_loop, args, measured_peak()[0])
        kernels["sum_ms_per_step"] = sum(r["ms_per_step"] for r in kernels["families"])
        torch.cuda.empty_cache()

    # --- the fluid problem: its GPU design loop beside the fluid oracle on the host
    fluid = fluid_leg(args) if args.fluid_n > 0 and world == 1 else None

    # --- the ragged 64-design batch: batched (concurrent workers) against the un-batched loop
    c4 = c4_batch(args) if args.c4_designs > 0 and world == 1 else None

    # --- the CPU oracle legs' grid on the GPU: a same-grid comparison with cpu_baseline and --impl reference
    rnx, rny = _grid(args.ref_grid)
    meshr = tg.RectangleMesh(2.0, 1.0, rnx, rny)
    Vr = tg.FunctionSpace(meshr, "CG", 1, dof_order="lattice")
    same_grid = {"workload": f"cantilever 2x1, {rnx}x{rny} squares, vector P2, {dofs(rnx, rny)} dofs, "
                             f"rtol {args.rtol}"}
    for precision in ("mixed", "fp64"):
        pr = tg.ElasticityProblem(meshr, Vr, dom, par, precision=precision, rtol=args.rtol)
        pr.set_penalization(PENALTY)
        tr, _, _, _ = device_loop(pr, args.steps, args.warmup, space=Vr, start=seeded_density(rnx, rny))
        same_grid[precision] = {"value": 1000.0 / float(np.mean(tr)), "ms_per_step": float(np.mean(tr)),
                                "steps": len(tr)}
        del pr
    torch.cuda.empty_cache()

    # --- the GPU loop and the CPU oracle side by side over a size sweep (off by default)
    sweep = None
    if args.size_sweep and world == 1:
        sweep = []
        for text in args.size_sweep.split(","):
            snx, sny = _grid(text)
            mesh_s = tg.RectangleMesh(2.0, 1.0, snx, sny)
            V_s = tg.FunctionSpace(mesh_s, "CG", 1, dof_order="lattice")
            ps = tg.ElasticityProblem(mesh_s, V_s, dom, par, precision="mixed", rtol=args.rtol)
            ps.set_penalization(PENALTY)
            ts, _, _, _ = device_loop(ps, args.steps, args.warmup, space=V_s, start=seeded_density(snx, sny))
            del ps
            torch.cuda.empty_cache()
            oval, osec = time_oracle(snx, sny, args.cpu_steps, 1)
            gval = 1000.0 / float(np.mean(ts))
            sweep.append({"grid": f"{snx}x{sny}", "dofs": dofs(snx, sny), "gpu_mixed": gval, "gpu_steps": len(ts),
                          "oracle": oval, "oracle_steps": args.cpu_steps, "gpu_over_oracle": gval / oval})

    # --- roofline of the dominant kernel
    peak, peak_kind = measured_peak()
    alg_bytes = 2 * dofs(args.nx, args.ny) * 4 + nv * 4
    op = float(np.mean(op_ms))
    achieved = alg_bytes / (op * 1e-3) / 1e9
    traffic, fp32_inst = ncu_counts(args.nx, args.ny)

    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return
    cpu = None
    if world == 1:
        rnx, rny = _grid(args.ref_grid)
        cval, csec = time_oracle(rnx, rny, args.cpu_steps, 1)
        cpu = {"value": cval, "unit": UNIT, "cores": 1, "kind": "port",
               "sample": oracle_sample(rnx, rny, args.cpu_steps, 1, csec)}
    nbytes = nv * 8
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic (seeded U(0.01,1) density)",
        "config": {"workload": f"cantilever 2x1, {args.nx}x{args.ny} squares, vector P2, "
                               f"{dofs(args.nx, args.ny)} dofs, rtol {args.rtol}, replicas: {world}",
                   "l2": "flushed (256 MB write) before every timed step"},
        "fp64": {"value": 1000.0 / ms64 * world, "ms_per_step": ms64, "steps": len(times64)},
        "mixed_over_fp64": ms64 / ms_mixed_same,
        "compliance_rel_diff_mixed_vs_fp64": comp_rel,
        "e2e": {"value": e2e_value * world, "unit": UNIT, "h2d_bytes_per_step": 2 * nbytes,
                "d2h_bytes_per_step": 2 * nbytes + 8},
        "roofline": {"bound": "hbm", "kernel": "k_p2_march<float, Apply> (FP32 matrix-free P2 operator)",
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_kind, "traffic": traffic, "algorithmic_bytes": alg_bytes,
                     "launch_ms": op,
                     # FP32 work the launch executes (ncu instruction counters, an FMA
                     # counted once), over this run's CUDA-event launch time
                     "executed_fp32_inst": fp32_inst,
                     "executed_fp32_tinst_per_s": fp32_inst / (op * 1e-3) / 1e12 if fp32_inst else None},
        "cpu_baseline": cpu,
        "same_grid": same_grid,
        "size_sweep": sweep,
        "gpu_launches": int(nlaunch),
        "kernels": kernels,
        "c2_2000x1000": c2,
        "c4_batch": c4,
        "march_tiles": march_tiles(),
        "fluid": fluid,
        "clocks": ck,
        "solver_iterations": stats,
    }
    print(json.dumps(out), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def march_tiles():
    """The autotuner's choices in this run: (kernel family, grid) -> cell rows per warp segment."""
    import ctypes
    from topomax_gb300 import _capi
    lib = _capi.load_library()
    need = lib.topo_march_tiles_report(None, 0)
    buf = ctypes.create_string_buffer(int(need))
    lib.topo_march_tiles_report(buf, need)
    out = []
    for line in buf.value.decode().splitlines():
        fam, nx, ny, seg = line.split("\t")
        out.append({"family": fam, "grid": f"{nx}x{ny}", "segment": int(seg)})
    return out


FLUID = {"Fluid": {
    "domain_parameters": dict(width=1.0, height=1.0, fem_step_size=0.0011, dem_step_size=0.0002, penalties=[0.1],
                              volume_fraction=0.5),
    "problem_parameters": dict(flows=[dict(side="Left", center=0.5, length=1.0, rate=1.0),
                                      dict(side="Right", center=0.5, length=1.0 / 3.0, rate=-3.0)],
                               viscosity=1.0)}}


def fluid_leg(args):
    """The Stokes-Brinkman diffuser (unit square, parabolic inflow on the left side, a three
    times faster outflow a third as wide on the right, penalty 0.1) at args.fluid_n cells per
    unit length: args.fluid_iterations design iterations of the GPU loop (FP64, rtol 1e-10)
    and of the FP64 fluid oracle (sparse LU, the reference algorithm) on the host, each
    from the uniform start, timed around solve() (set-up excluded; one GPU warm-up run)."""
    import torch
    from oracle.fluid import FluidDesign, FluidOracleSolver
    from topomax_gb300.solver import FEMSolver
    n, k = args.fluid_n, args.fluid_iterations
    FEMSolver(n, dict(FLUID, name="diffuser"), precision="fp64", rtol=1e-10, verbose=False, save=False,
              max_iterations=1).solve()
    s = FEMSolver(n, dict(FLUID, name="diffuser"), precision="fp64", rtol=1e-10, verbose=False, save=False,
                  max_iterations=k)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    h = s.solve()[0.1]
    torch.cuda.synchronize()
    t_gpu = time.perf_counter() - t0
    o = FluidOracleSolver(n, FluidDesign.from_dict(FLUID), max_iterations=k, pressure="mean")
    t0 = time.perf_counter()
    run = o.solve()[0]
    t_cpu = time.perf_counter() - t0
    return {"workload": f"diffuser 1x1, {n}x{n} squares, Taylor-Hood, penalty 0.1, {k} design iterations",
            "gpu": {"design_iters_per_s": h["iterations"] / t_gpu, "s": t_gpu, "iterations": h["iterations"],
                    "objective": h["objectives"][-1],
                    "krylov_iterations_per_solve": s.problem.stats["state_iterations"] / len(h["objectives"])},
            "cpu_oracle": {"design_iters_per_s": run.iterations / t_cpu, "s": t_cpu, "iterations": run.iterations,
                           "objective": run.objectives[-1], "cores": 1},
            "objective_rel_diff": abs(h["objectives"][-1] - run.objectives[-1]) / abs(run.objectives[-1])}


def c4_batch(args):
    """The ragged design batch: args.c4_designs designs of the step-size sweep (domain 2x1,
    N drawn from {100, 150, 200, 250, 300}, clamped bottom corners, circular body force,
    p in {3, 4, 5}, random volume fraction and step size; seed 3), each run for
    args.c4_iterations design iterations, once one design after another (the un-batched
    loop) and once by args.c4_workers concurrent workers on their own streams.  Wall time
    of each whole run, context set-up included (its per-design sums are reported beside:
    set-up allocates device memory under the library's device lock, so it does not overlap
    between workers); one design of every size runs first so that both timed runs find the
    march tiles tuned."""
    import torch
    from topomax_gb300.batch import BatchItem, config4_designs, run_batch
    items = config4_designs(args.c4_designs, seed=3)
    seen = {}
    for it in items:
        seen.setdefault(it.N, it)
    run_batch([BatchItem(it.N, it.design, it.name) for it in seen.values()], 1, workers=1, rtol=args.rtol)
    out = {}
    for leg, workers in (("sequential", 1), ("batched", args.c4_workers)):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        res = run_batch(items, args.c4_iterations, workers=workers, rtol=args.rtol)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        iters = sum(h["iterations"] for r in res for h in r.history.values())
        out[leg] = {"workers": workers, "s": dt, "design_iterations": iters,
                    "design_iters_per_s": iters / dt, "errors": sum(1 for r in res if r.error),
                    "setup_s_sum": sum(r.setup_s for r in res), "loop_s_sum": sum(r.solve_s for r in res),
                    "loop_ms_per_design_iteration": 1000.0 * sum(r.solve_s for r in res) / max(1, iters)}
        out[leg + "_histories"] = res
    a, b = out.pop("sequential_histories"), out.pop("batched_histories")
    keys = ("objectives", "deltas", "exit_condition", "iterations")  # not the wall times
    same = all({p: {k: h[k] for k in keys} for p, h in x.history.items()}
               == {p: {k: h[k] for k in keys} for p, h in y.history.items()} for x, y in zip(a, b))
    sizes = sorted({it.N for it in items})
    return {"workload": f"{len(items)} designs, domain 2x1, N in {sizes} (nx = 2N), "
                        f"{args.c4_iterations} design iterations each, mixed precision, rtol {args.rtol}",
            **out, "batched_over_sequential": out["sequential"]["s"] / out["batched"]["s"],
            "histories_bitwise_equal": same}


def kernel_table(tg, mesh, V, dom, par, rho0, device_loop, args, peak):
    """HBM GB/s per kernel family: a context with host-driven solves (TOPO_GRAPHS=0, the
    same kernels as the recorded graphs) runs args.kernel_steps design iterations after one
    warm-up with the library's kernel clock on, which brackets every annotated launch with
    CUDA events and sums the algorithmic bytes of its family (no L2 flush between
    launches: the vectors of the two finest levels exceed L2, the small levels stay
    L2-resident as they do in the solve)."""
    import ctypes
    from topomax_gb300 import _capi
    lib = _capi.load_library()
    old = os.environ.get("TOPO_GRAPHS")
    os.environ["TOPO_GRAPHS"] = "0"
    try:
        prob = tg.ElasticityProblem(mesh, V, dom, par, precision="mixed", rtol=args.rtol)
        prob.set_penalization(PENALTY)
        device_loop(prob, args.kernel_steps, 1, space=V, start=rho0, on_start=lambda: lib.topo_kernel_clock(1))
        lib.topo_kernel_clock(0)
        need = lib.topo_kernel_clock_report(None, 0)
        buf = ctypes.create_string_buffer(int(need))
        lib.topo_kernel_clock_report(buf, need)
        del prob
    finally:
        if old is None:
            os.environ.pop("TOPO_GRAPHS", None)
        else:
            os.environ["TOPO_GRAPHS"] = old
    rows = []
    for line in buf.value.decode().splitlines():
        fam, level, n, ms, nbytes = line.split("\t")
        n, ms, nbytes = int(n), float(ms), float(nbytes)
        row = {"family": fam, "level": int(level), "launches_per_step": n / args.kernel_steps,
               "us_per_launch": 1000.0 * ms / n, "ms_per_step": ms / args.kernel_steps}
        if nbytes > 0:
            row["bytes_per_launch"] = nbytes / n
            row["gbs"] = nbytes / (ms * 1e-3) / 1e9
            row["frac_of_peak"] = row["gbs"] / peak
        rows.append(row)
    rows.sort(key=lambda r: -r["ms_per_step"])
    return {"method": "host-driven launches (TOPO_GRAPHS=0), each bracketed by CUDA events; algorithmic "
                      "bytes per family as the library counts them; per design iteration over "
                      f"{args.kernel_steps} iterations after 1 warm-up", "families": rows}


class _E2ESolver:
    """The projection entry of FEMSolver (src/solver.py:149-186) bound to a problem."""

    def __init__(self, prob, V, volume):
        self.prob = prob
        self.V = V

    def project(self, half_host, volume):
        import ctypes
        import torch
        from topomax_gb300 import fem as F
        half = half_host.to("cuda", non_blocking=False)
        zero = torch.zeros_like(half)
        psi = torch.empty_like(half)
        c = ctypes.c_double(0)
        lib = self.prob._ctx._lib
        self.prob._ctx.check(lib.topo_emd_step(self.prob._ctx.ptr, F._ptr(half), F._ptr(zero), 0.0, volume,
                                               F._ptr(psi), ctypes.byref(c), F._stream()))
        return psi


if __name__ == "__main__":
    main()
