#!/usr/bin/env python
"""bench.py -- throughput of the les-model time step on GB300.

Workload (default): the 256x128x128 configuration (obstacle scaled 4x,
u = 1 + U(-0.01, 0.01) noise), one step = SGS nu_t + momentum + velocity BCs +
divergence RHS + pressure solve to relative residual 1e-8 + projection +
velocity BCs.  The pressure solve is Chebyshev(4)-PCG, mixed precision (FP32
inner PCG, FP64 defect correction); the plain FP64 GPU path runs the same
trajectory beside it for the FP64-vs-mixed comparison and per-step errors.

Metric: Mcell-steps/s = cells x steps / device seconds (CUDA events on the
library's stream, L2 flushed before every timed step).  Also reported:
  e2e           the same steps timed end to end through the C ABI: the
                step's Field arrays copied in from pinned host buffers,
                les_step, and its outputs copied back, per step;
  roofline      HBM bytes/s of the dominant kernel against the measured copy
                bandwidth (MEASURED_PEAKS.json);
  cpu_baseline  the CPU oracle (OpenMP, all host threads): one full time
                step of the same workload from the initial state, also
                compared field by field with the GPU's first FP64 step.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
Multi-GPU (torchrun): independent replicas, one per GPU (the step has no
exchange to shard); rank 0 prints the max-over-ranks result.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for sub in (os.path.join(ROOT, "les-model_gb300", "py"), os.path.join(ROOT, "les-model_gb300"),
            os.path.join(ROOT, "oracle")):
    if sub not in sys.path:
        sys.path.insert(0, sub)

import numpy as np  # noqa: E402

METRIC = "Mcell-steps/s @256x128x128, mixed vs FP64 GPU at div<=1e-8; HBM GB/s % peak"
UNIT = "Mcell-steps/s"
FALLBACK_HBM_GBS = 6800.0

def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=("ours", "reference"))
    ap.add_argument("--workload", default="large", choices=("small", "large", "xlarge", "batch", "adjoint"))
    ap.add_argument("--adj-steps", type=int, default=50, help="adjoint workload: forward steps")
    ap.add_argument("--fd-step", type=float, default=1e-6, help="adjoint workload: finite-difference step")
    ap.add_argument("--adj-tol", type=float, default=1e-12,
                    help="adjoint workload: relative residual of every forward and adjoint pressure solve")
    ap.add_argument("--batch", type=int, default=64, help="cases of the batch workload")
    ap.add_argument("--ens-batched", type=int, default=1,
                    help="batch workload: 1 the cases' solves in shared kernels, 0 one graph branch per case")
    ap.add_argument("--tune", type=int, default=1,
                    help="run the strip-shape autotuner before warm-up (column passes, built-in rows/chunks)")
    ap.add_argument("--solver", default="pcg", choices=("pcg", "gs"),
                    help="pressure solver: PCG (mixed precision, FP64 beside it) or GS-SOR (FP64, omega 1.7)")
    ap.add_argument("--precond", default="cheb", choices=("cheb", "jacobi", "ic"))
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 comparison run")
    ap.add_argument("--truth", type=int, default=1,
                    help="also run the trajectory with converged solves (FP64 defect correction to relative "
                         "residual 1e-12) to split the pressure error into each run's own solve error")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--cpu-steps", type=int, default=1, help="full CPU oracle steps in the CPU baseline sample")
    ap.add_argument("--seed", type=int, default=1234)
    ap.add_argument("--inner-rtol", type=float, default=1e-4, help="mixed path: inner FP32 solve reduction")
    ap.add_argument("--tma", type=int, default=0, help="stage the tile passes with TMA (LES_OPT_TMA)")
    ap.add_argument("--fused", type=int, default=1, help="inner passes: 1 register columns, 2 smem tiles, 0 unfused")
    ap.add_argument("--rows", default="0,0", help="rows per strip of the column passes A,B (0 = built-in)")
    ap.add_argument("--chunks", default="0,0", help="planes per march chunk of the column passes A,B (0 = auto)")
    ap.add_argument("--graph", type=int, default=1, help="replay each time step as one CUDA graph (LES_OPT_GRAPH)")
    ap.add_argument("--pdl", type=int, default=None,
                    help="column passes as programmatic dependent launches (LES_OPT_PDL; default: the library's, "
                         "on for a single case, off for ensemble cases)")
    ap.add_argument("--phys32", type=int, default=1, help="mixed path: nu_t and momentum in FP32 (LES_OPT_PHYS32)")
    ap.add_argument("--prof-steps", type=int, default=2, help="extra steps timed per kernel for the roofline")
    return ap.parse_args()


def max_over_ranks(x, pg, device="cpu"):
    """The slowest rank's value of x, on every rank (x itself without a group)."""
    if not pg:
        return x
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def shard_cases(sizes, rank, world):
    """Independent cases over ranks with no exchange: longest first onto the
    least-loaded rank (by cell count).  Returns this rank's case indices."""
    load = [0] * world
    owner = [0] * len(sizes)
    for i in sorted(range(len(sizes)), key=lambda q: (-sizes[q], q)):
        r = min(range(world), key=lambda q: (load[q], q))
        owner[i] = r
        load[r] += sizes[i]
    return [i for i in range(len(sizes)) if owner[i] == rank]


def dist_env():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, dev):
        self.dev = dev
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[q] for r in rows for q in range(4) if r[5 + q].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# algorithmic HBM bytes per cell of one launch of each profiled kernel
def alg_bytes_per_cell(name, fused=1):
    # fused FP32 inner passes.  Register columns (fused=1, the default): pass B
    # reads r, q and writes r', z (the whole Chebyshev apply stays on chip);
    # pass A reads z, p_old, e and writes p, q, e.  Shared-memory tiles
    # (fused=2): pass B reads r, q, p, e and the stencil code and writes r',
    # e', z; pass A reads z, p_old, code and writes p, q.
    if fused == 1 and name in ("inner_precond_f32", "inner_spmv_f32"):
        # the column passes take the matrix from the cell position (no code byte)
        return {"inner_precond_f32": 16.0, "inner_spmv_f32": 24.0}[name]
    return {"inner_precond_f32": 29.0, "inner_spmv_f32": 17.0, "inner_update_f32": 28.0, "spmv_f64": 17.0,
            "update_f64": 48.0, "cheb_f64": 41.0, "outer_resid_f64": 21.0}.get(name)


def pc_code(G, name):
    return {"cheb": G.PC_CHEBYSHEV, "jacobi": G.PC_JACOBI, "ic": G.PC_IC}[name]


def make_ctx(G, les_cases, shape, h, solid, f, dev, precond):
    m = G.Mesh(*shape, h, h, h)
    c = G.Context(m, dev)
    c.upload_mask(np.zeros(m.n, np.uint8))
    c.build_stencil()            # src/main.cpp:66: A before the obstacle
    if precond == "ic":
        c.build_ic()
    lmax = c.lambda_max(20)      # :74
    c.upload_mask(solid)         # :81
    c.upload_fields(f)
    return c, lmax


def step_params(G, les_cases, precond, lmax, precision, inner_rtol=1e-4, solver="pcg"):
    pc = pc_code(G, precond)
    if solver == "gs":   # solve_pressure_GS, src/pressure.cpp:186-247: omega 1.7, 200 sweeps, max |dp| < 1e-6
        return G.step_params(nu=les_cases.NU, rho=les_cases.RHO, cs=les_cases.CS, cfl_conv=les_cases.CFL_CONV,
                             cfl_visc=les_cases.CFL_VISC, dt_max=les_cases.DT_MAX, solver=G.SOLVER_GS,
                             stat_max_iter=200, stat_tol=1e-6, omega=1.7)
    # IC(0)-PCG does not converge on this non-symmetric system (the reference's
    # own run stalls): it runs to the reference's cap of 1000 iterations
    # (src/main.cpp:137) in both precisions
    cap = 1000 if precond == "ic" else None
    if precision == G.MIXED:
        opts = G.pcg_opts(precond=pc, max_iter=cap or 50000, lambda_min=3 * np.pi ** 2, lambda_max=lmax, degree=4,
                          precision=G.MIXED, inner_rtol=inner_rtol, inner_max_iter=cap or 5000,
                          max_outer=1 if cap else 40)
    else:
        opts = G.pcg_opts(precond=pc, max_iter=cap or 10000, lambda_min=3 * np.pi ** 2, lambda_max=lmax, degree=4)
    return G.step_params(nu=les_cases.NU, rho=les_cases.RHO, cs=les_cases.CS, cfl_conv=les_cases.CFL_CONV,
                         cfl_visc=les_cases.CFL_VISC, dt_max=les_cases.DT_MAX, solver=G.SOLVER_PCG,
                         rel_tol=1e-8, pcg=opts)


class OracleCase:
    """The CPU oracle (OpenMP, `threads` host threads) set up the way
    make_ctx sets up the device: A assembled before the obstacle
    (src/main.cpp:66-81), the IC factor from it, lambda_max by the power
    iteration from the reference's std::mt19937(1337) start vector, then the
    same initial fields; step() is one full reference time step
    (src/main.cpp:115-144) with the same solver settings as the GPU's FP64
    run."""

    def __init__(self, shape, h, solid, f, precond, solver, threads):
        import les_cases
        import oracle as O
        self.orc = O.Oracle()
        self.orc.set_threads(threads)
        self.threads = threads
        self.m = O.Mesh(*shape, h, h, h)
        n = self.m.n
        self.A0 = self.orc.build_stencil(self.m, np.zeros(n, np.uint8))
        self.L0 = self.orc.ic_build(self.m, self.A0) if (solver == "pcg" and precond == "ic") else None
        self.lmax = (self.orc.lambda_max(self.m, self.A0, O.mt19937_start_vector(n), 20)
                     if (solver == "pcg" and precond == "cheb") else 0.0)
        self.f = {k: f[k].copy() for k in O.FIELD_KEYS}
        self.f["solid"] = solid.copy()
        pc = {"cheb": O.PC_CHEB, "jacobi": O.PC_JACOBI, "ic": O.PC_IC}[precond]
        common = dict(nu=les_cases.NU, rho=les_cases.RHO, cs=les_cases.CS, cfl_conv=les_cases.CFL_CONV,
                      cfl_visc=les_cases.CFL_VISC, dt_max=les_cases.DT_MAX, omega=1.7, lmin=3 * np.pi ** 2,
                      lmax=self.lmax, degree=4, dt_fixed=-1.0, pc=pc)
        if solver == "gs":
            self.prm = O.StepParams(solver=2, max_iter=200, tol=1e-6, rel_tol=0.0, **common)
        else:
            self.prm = O.StepParams(solver=0, max_iter=1000 if precond == "ic" else 10000, tol=0.0, rel_tol=1e-8,
                                    **common)

    def step(self):
        """One full step; returns (seconds, solver iterations)."""
        t = time.perf_counter()
        it, _ = self.orc.step(self.m, self.f, self.A0, self.L0, self.prm)
        return time.perf_counter() - t, it


def run_reference(args):
    """The reference's CPU path for the same workload: full time steps of the
    CPU oracle (the C restatement of the reference, pinned bit-exact to it on
    the golden fixtures), OpenMP on every host core, from the same initial
    state; W untimed warm-up steps, then K timed steps, so the timed steps
    are the same trajectory steps the GPU arm times."""
    rank, world, local = dist_env()
    if rank != 0:
        return 0
    import les_cases
    if args.workload not in ("small", "large", "xlarge"):
        print(json.dumps({"impl": "reference", "unavailable": "the CPU arm times single cases "
                          "(small, large, xlarge); the ensemble and adjoint workloads have no CPU counterpart"}),
              flush=True)
        return 0
    shape, h, solid, f = les_cases.case(args.workload, args.seed)
    n = int(np.prod(shape))
    oc = OracleCase(shape, h, solid, f, args.precond, args.solver, os.cpu_count() or 1)
    for _ in range(args.warmup):
        oc.step()
    secs, iters = [], []
    for _ in range(args.steps):
        t, it = oc.step()
        secs.append(t)
        iters.append(it)
    value = n * args.steps / sum(secs) / 1e6
    solver = "GS-SOR (omega 1.7)" if args.solver == "gs" else "%s-PCG" % args.precond
    sample = ("%d full FP64 time steps of the CPU oracle at %s (%s to %s; steps %d..%d of the trajectory after "
              "%d warm-up steps), %.1f s timed" %
              (args.steps, "x".join(map(str, shape)), solver,
               "max |dp| < 1e-6" if args.solver == "gs" else "relative residual 1e-8",
               args.warmup, args.warmup + args.steps - 1, args.warmup, sum(secs)))
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(secs) / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": {"workload": "%s %s FP64" % ("x".join(map(str, shape)), solver),
                                             "solver": args.solver, "precond": args.precond,
                                             "lambda_max": oc.lmax or None},
            "iters_mean": statistics.mean(iters), "iters": iters,
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": oc.threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_batch(args):
    """Ensemble workload: `--batch` ragged cases (dims from {32..96}, random
    cube obstacle, Cs from [0.1, 0.2], inflow noise 0.02), mixed-precision
    Chebyshev(4)-PCG, every step one CUDA graph launch for all cases.  By
    default the cases' solves share kernels (one launch per inner pass over
    all cases); with --ens-batched 0 each case is its own graph branch, with
    strip shapes and chunk lengths from the ensemble autotuner."""
    import torch
    import les_cases
    import les_gb300 as G

    rank, world, local = dist_env()
    torch.cuda.set_device(local if world > 1 else 0)
    pg = None
    if world > 1:   # the cases are independent: each rank advances its share, no exchange
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
        pg = dist
    all_specs = les_cases.batch_cases(args.batch, args.seed)
    cells_all = sum(int(np.prod(s["shape"])) for s in all_specs)
    specs = [all_specs[i] for i in shard_cases([int(np.prod(s["shape"])) for s in all_specs], rank, world)]
    meshes = [G.Mesh(*s["shape"], s["h"], s["h"], s["h"]) for s in specs]
    ens = G.Ensemble(meshes)
    ens.set_batched(args.ens_batched)
    prm = []
    for c, s in zip(ens.cases, specs):
        shape = s["shape"]
        n = int(np.prod(shape))
        if args.pdl is not None:
            c.set_option(G.OPT_PDL, args.pdl)
        c.set_option(G.OPT_PHYS32, args.phys32)
        c.upload_mask(np.zeros(n, np.uint8))
        c.build_stencil()
        lmax = c.lambda_max(20)
        solid = les_cases.box_mask(shape, s["box"])
        f = les_cases.init_fields(shape, s["noise"], s["seed"])
        les_cases.velocity_bcs_np(shape, f, solid)
        c.upload_fields(f)
        c.upload_mask(solid)
        prm.append(G.step_params(nu=les_cases.NU, rho=les_cases.RHO, cs=s["cs"], cfl_conv=les_cases.CFL_CONV,
                                 solver=G.SOLVER_PCG, rel_tol=1e-8,
                                 pcg=G.pcg_opts(precond=G.PC_CHEBYSHEV, max_iter=5000, lambda_min=3 * np.pi ** 2,
                                                lambda_max=lmax, degree=4, precision=G.MIXED,
                                                inner_rtol=args.inner_rtol)))
    cells = sum(int(np.prod(s["shape"])) for s in specs)
    t0 = time.perf_counter()
    tune_us = ens.autotune(prm[0].pcg) if args.tune else None   # batched: the work split; else per case
    split = ens.batch_split()
    tune_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    for _ in range(args.warmup):
        ens.step(prm)
    ens.sync()
    warm_s = time.perf_counter() - t0
    launches0 = sum(c.launch_count() for c in ens.cases)
    clocks = Clocks(local if world > 1 else 0)
    if pg:
        pg.barrier()
    clocks.start()
    iters, worst = [], 0.0
    t0 = time.perf_counter()
    for _ in range(args.steps):
        st = ens.step(prm)
        iters.append(statistics.mean(x.iters for x in st))
        worst = max(worst, max(x.residual / x.b_norm for x in st if x.b_norm > 0))
        bad = [x.status for x in st if x.status != G.OK]
        if bad:
            raise RuntimeError("ensemble step: %d cases did not converge" % len(bad))
    wall = max_over_ranks(time.perf_counter() - t0, pg, "cuda" if torch.cuda.is_available() else "cpu")
    clk = clocks.stop()
    launches = sum(c.launch_count() for c in ens.cases) - launches0
    value = cells_all * args.steps / wall / 1e6   # every rank's cases over the slowest rank's time
    ens.close()
    if pg:
        pg.barrier()
        pg.destroy_process_group()
    if rank != 0:
        return 0
    line = {"metric": "Mcell-steps/s, ensemble of %d ragged cases, mixed FP32/FP64 at div<=1e-8" % args.batch,
            "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * wall / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 inner / f64 outer", "data": "synthetic",
            "config": {"workload": "batch: %d cases, dims from {32,48,64,80,96}, cube obstacle, Cs U[0.1,0.2], "
                                   "cheb(4)-PCG mixed, one graph launch per step" % args.batch,
                       "cells": cells_all, "cells_rank0": cells,
                       "parallelism": "cases sharded over %d ranks, no exchange" % world if world > 1 else "single",
                       "timing": "host wall clock around each step's launch + stats sync, max over ranks",
                       "l2": "inputs (~%.1f GB) larger than L2" % (cells * 120 / 1e9),
                       "pdl": 0 if args.pdl is None else args.pdl, "phys32": args.phys32,
                       "form": "batched solves" if args.ens_batched else "one branch per case",
                       "split": ("whole-length strips, then one more chunk for the longest march until the "
                                 "items reach %dx the resident warps (%s)" %
                                 (split, "chosen by the ensemble autotuner from 2, 3, 4, 6"
                                  if args.tune else "the default") if args.ens_batched else
                                 "per case from the ensemble autotuner"),
                       "autotune_us_per_iteration": tune_us, "autotune_s": tune_s,
                       "first_steps_with_capture_s": warm_s},
            "gpu_launches": launches, "iters_inner_mean": statistics.mean(iters), "rel_residual_max": worst,
            "clocks": clk}
    print(json.dumps(line), flush=True)
    return 0


def run_adjoint(args):
    """Adjoint workload: 128x64x64 (h = 1/64) with the centred cube, N steps
    of the mixed-precision Chebyshev(4) step at fixed dt, J = time average of
    the probe-box kinetic energy over [96,120)x[16,48)x[16,48); gradient with
    respect to the 64x64 inlet u-profile (at the uniform profile u = 1) and
    Cs, checkpoint every 10 steps; checked against central finite
    differences (step --fd-step) on 16 seeded profile entries and on Cs."""
    import torch
    import les_cases
    import les_gb300 as G

    rank, world, local = dist_env()
    if rank != 0:
        return 0
    torch.cuda.set_device(0)
    shape, h, solid, f = les_cases.case("adjoint", args.seed)
    n = int(np.prod(shape))
    box = (96, 120, 16, 48, 16, 48)
    nsteps = args.adj_steps
    prof0 = np.ones(shape[1] * shape[2])

    def setup(c, prof):
        c.upload_mask(np.zeros(n, np.uint8))
        c.build_stencil()
        lmax = c.lambda_max(20)
        c.upload_fields(f)
        c.upload_mask(solid)
        c.set_inlet(prof)
        c.velocity_bcs()
        dt = c.adaptive_dt(les_cases.NU, les_cases.CFL_CONV, les_cases.CFL_VISC, les_cases.DT_MAX)
        return lmax, dt

    def params(lmax, dt, cs):
        return G.step_params(nu=les_cases.NU, rho=les_cases.RHO, cs=cs, dt_fixed=dt, solver=G.SOLVER_PCG,
                             rel_tol=args.adj_tol,
                             pcg=G.pcg_opts(precond=G.PC_CHEBYSHEV, max_iter=50000, lambda_min=3 * np.pi ** 2,
                                            lambda_max=lmax, degree=4, precision=G.MIXED, inner_rtol=1e-4))

    mesh = G.Mesh(*shape, h, h, h)

    def J_of(prof, cs):
        with G.Context(mesh) as c:
            lmax, dt = setup(c, prof)
            return c.adjoint_forward(params(lmax, dt, cs), nsteps, 10, box, args.adj_tol)

    with G.Context(mesh) as c:
        lmax, dt = setup(c, prof0)
        prm = params(lmax, dt, les_cases.CS)
        c.sync()
        t0 = time.perf_counter()
        J = c.adjoint_forward(prm, nsteps, 10, box, args.adj_tol)
        t_fwd = time.perf_counter() - t0
        t0 = time.perf_counter()
        g, gcs = c.adjoint_backward()
        t_bwd = time.perf_counter() - t0
        # FP64 tangent-linear model along a seeded direction: the dot-product test
        rng_t = np.random.default_rng(args.seed + 1)
        d_in, d_cs = rng_t.standard_normal(g.size), 0.01
        t0 = time.perf_counter()
        dJ_tl = c.adjoint_tangent(d_in, d_cs)
        t_tl = time.perf_counter() - t0
        proj = float(np.dot(g, d_in) + gcs * d_cs)
        tl_err = abs(dJ_tl - proj) / max(abs(proj), 1e-300)
    rng = np.random.default_rng(args.seed)
    ny, nz = shape[1], shape[2]
    cand = [(j, k) for j in range(1, ny - 1) for k in range(1, nz - 1)]
    pick = [cand[i] for i in rng.choice(len(cand), 16, replace=False)]
    hs = args.fd_step
    # central differences with the configured step, and a noise check: J is
    # computed with solves to a relative residual of 1e-12 whose rounding
    # differs from run to run, so a difference quotient carries about
    # |dJ_noise| / step of noise; the Richardson combination of steps 10 and
    # 20 times larger, (4 D(10 h) - D(20 h)) / 3, removes the O(step^2)
    # truncation term at a tenth of that noise
    def cdiff(fn, h):
        return (fn(h) - fn(-h)) / (2 * h)

    def fds(fn):
        d1, d10, d20 = cdiff(fn, hs), cdiff(fn, 10 * hs), cdiff(fn, 20 * hs)
        return d1, (4 * d10 - d20) / 3

    rows = []
    for (j, k) in pick:
        idx = j * nz + k

        def Jp(h, idx=idx):
            p = prof0.copy()
            p[idx] += h
            return J_of(p, les_cases.CS)
        fd, fdr = fds(Jp)
        rows.append({"j": j, "k": k, "adjoint": float(g[idx]), "fd": fd, "fd_richardson": fdr,
                     "rel_err": abs(fd - g[idx]) / max(abs(g[idx]), 1e-300),
                     "rel_err_richardson": abs(fdr - g[idx]) / max(abs(g[idx]), 1e-300)})
    fdc, fdcr = fds(lambda h: J_of(prof0, les_cases.CS + h))
    cs_err = abs(fdc - gcs) / max(abs(gcs), 1e-300)
    cs_err_r = abs(fdcr - gcs) / max(abs(gcs), 1e-300)
    errs = [r["rel_err"] for r in rows] + [cs_err]
    errs_r = [r["rel_err_richardson"] for r in rows] + [cs_err_r]
    line = {"metric": "adjoint gradient of the probe-box kinetic energy vs central finite differences",
            "value": max(errs), "unit": "max relative error", "higher_is_better": False, "n_gpus": 1,
            "steps": nsteps, "warmup": 0, "dtype": "f32 inner / f64 outer (tol %g)" % args.adj_tol, "data": "synthetic",
            "config": {"workload": "adjoint 128x64x64 h=1/64 centred cube, %d steps, dt %.3g fixed, checkpoint "
                                   "every 10, probe [96,120)x[16,48)x[16,48), controls 64x64 inlet u + Cs" % (nsteps, dt),
                       "fd_step": hs, "fd_entries": 16},
            "J": J, "grad_cs": gcs, "fd_cs": fdc, "cs_rel_err": cs_err, "grad_inlet_max_abs": float(np.abs(g).max()),
            "median_rel_err": float(np.median(errs)),
            "richardson": {"steps": [10 * hs, 20 * hs], "max_rel_err": max(errs_r),
                           "median_rel_err": float(np.median(errs_r)), "cs_rel_err": cs_err_r},
            "entries": rows,
            "forward_s": t_fwd, "backward_s": t_bwd, "backward_over_forward": t_bwd / t_fwd,
            "tangent": {"dJ": dJ_tl, "adjoint_projection": proj, "rel_err": tl_err, "seconds": t_tl}}
    print(json.dumps(line), flush=True)
    return 0


# FP64 operations per cell of the FP64 PCG kernels (each multiply and add
# counted; the reference-order kernels run without FMA): the 7-point row is
# 7 multiplies + 6 adds
FP64_OPS_PER_CELL = {"spmv_f64": 15.0,     # row + p.q term
                     "update_f64": 6.0,    # x += a p, r -= a q, r.r term (Chebyshev/IC form)
                     "cheb_f64": 18.0}     # row + r - Az + beta p + z + alpha p


def rel_err(a, b, tmp=None):
    """max |a - b| / max |b|; `tmp` (an array like a) avoids allocating."""
    d = np.subtract(a, b, out=tmp)
    np.abs(d, out=d)
    num = float(d.max())
    np.abs(b, out=d)
    return num / max(float(d.max()), 1e-300)


def run_ours(args):
    import torch
    import les_cases
    import les_gb300 as G

    rank, world, local = dist_env()
    dev = local if world > 1 else 0
    torch.cuda.set_device(dev)
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
        pg = dist
    gs = args.solver == "gs"
    shape, h, solid, f = les_cases.case(args.workload, args.seed)
    n = int(np.prod(shape))
    ctx, lmax = make_ctx(G, les_cases, shape, h, solid, f, dev, args.precond)
    ctx.set_option(G.OPT_FUSED, args.fused)
    ctx.set_option(G.OPT_TMA, args.tma)
    ctx.set_option(G.OPT_GRAPH, args.graph)
    ctx.set_option(G.OPT_PDL, 1 if args.pdl is None else args.pdl)
    ctx.set_option(G.OPT_PHYS32, args.phys32)
    ra, rb = (int(x) for x in args.rows.split(","))
    ca, cb = (int(x) for x in args.chunks.split(","))
    for opt, v in ((G.OPT_ROWS_A, ra), (G.OPT_ROWS_B, rb), (G.OPT_CHUNK_A, ca), (G.OPT_CHUNK_B, cb)):
        ctx.set_option(opt, v)
    prm = step_params(G, les_cases, args.precond, lmax, G.FP64 if gs else G.MIXED, args.inner_rtol, args.solver)
    tune_us = None   # strip rows and chunk lengths from the autotuner (outside the timed region)
    if (not gs and args.tune and args.fused == 1 and args.rows == "0,0" and args.chunks == "0,0"
            and args.precond != "ic"):
        tune_us = ctx.autotune(prm.pcg)
    shape_used = {k: ctx.get_option(o) for k, o in (("rows_a", G.OPT_ROWS_A), ("rows_b", G.OPT_ROWS_B),
                                                    ("chunk_a", G.OPT_CHUNK_A), ("chunk_b", G.OPT_CHUNK_B))}
    ctx64 = ctxT = None
    if not gs and not args.no_fp64:   # the plain FP64 path on the same trajectory (the reference's arithmetic)
        ctx64, _ = make_ctx(G, les_cases, shape, h, solid, f, dev, args.precond)
        prm64 = step_params(G, les_cases, args.precond, lmax, G.FP64)
        if args.truth:   # converged solves: FP64 defect correction to relative residual 1e-12, FP64 physics
            ctxT, _ = make_ctx(G, les_cases, shape, h, solid, f, dev, args.precond)
            ctxT.set_option(G.OPT_PHYS32, 0)
            prmT = step_params(G, les_cases, args.precond, lmax, G.MIXED, args.inner_rtol)
            prmT.rel_tol = 1e-12
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")   # 256 MiB > L2

    def l2_flush():
        flush.fill_(1.0)
        torch.cuda.synchronize()

    # ---- warm-up; the first step of the FP64 path (or of GS-SOR) is kept for
    # the parity check against the CPU oracle's first step
    par = ctx64 if ctx64 else (ctx if gs else None)
    first = None
    for w in range(args.warmup):
        st = ctx.step(prm)
        s64 = ctx64.step(prm64) if ctx64 else None
        if ctxT:
            ctxT.step(prmT)
        if w == 0 and par is not None:
            first = {"iters": (s64 if ctx64 else st).iters,
                     "fields": par.download_fields(("u", "v", "w", "p", "nu_t"))}
    ctx.sync()

    # ---- timed steps.  Each step is one call of the public API with host
    # buffers, les_step_io: the step's inputs (the Field arrays) copied from
    # pinned host memory, the step, the step's outputs copied back.  `value`
    # is the device time of the step alone (CUDA events on the library's
    # stream, reported by the call); `e2e` is the host wall time of the same
    # calls.
    in_keys = ("u", "v", "w", "u_new", "v_new", "w_new", "p", "nu_t")
    out_keys = ("u", "v", "w", "u_new", "v_new", "w_new", "p", "p_rhs", "nu_t")
    host = {k: torch.empty(n, dtype=torch.float64).pin_memory() for k in set(in_keys) | set(out_keys)}
    for k in host:
        ctx.download_ptr(k, host[k].data_ptr())
    up = {k: host[k].data_ptr() for k in in_keys}
    down = {k: host[k].data_ptr() for k in out_keys}
    hview = {k: host[k].numpy() for k in host}

    rec = dict(ms=[], e2e_s=[], ms64=[], iters=[], outer=[], iters64=[], rres=[], rres64=[], err=[], errT=[])
    d64 = {k: np.empty(n) for k in ("u", "v", "w", "p")}
    pT, tmp = np.empty(n), np.empty(n)
    # this machine's host link, outside the timed region: the copies les_step_io makes
    link = {}
    for name, fn, nbytes in (("h2d", lambda: ctx.upload_many_ptr(up), 8 * n * len(in_keys)),
                             ("d2h", lambda: ctx.download_many_ptr(down), 8 * n * len(out_keys))):
        fn()
        t0 = time.perf_counter()
        for _ in range(3):
            fn()
        link[name] = 3 * nbytes / (time.perf_counter() - t0) / 1e9
    clocks = Clocks(dev)
    if pg:
        pg.barrier()
    torch.cuda.synchronize()
    clocks.start()
    launches0 = ctx.launch_count()
    wall0 = time.perf_counter()
    # the timed steps run back to back; each one's fields are kept (host
    # copies into buffers touched beforehand) for the comparison runs, which
    # step after the timed loop from the same initial state
    sv_keys = ("u", "v", "w", "p") if 4 * 8 * n * args.steps <= (16 << 30) else ("p",)
    saved = {k: np.zeros((args.steps, n)) for k in sv_keys} if ctx64 else {}
    for s in range(args.steps):
        l2_flush()
        t0 = time.perf_counter()
        st, step_ms = ctx.step_io(prm, up, down)
        rec["e2e_s"].append(time.perf_counter() - t0)
        rec["ms"].append(step_ms)
        rec["iters"].append(st.iters)
        rec["outer"].append(st.outer)
        rec["rres"].append(st.residual / st.b_norm if st.b_norm > 0 else 0.0)
        for k in saved:
            np.copyto(saved[k][s], hview[k])
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    launches = ctx.launch_count() - launches0
    clk = clocks.stop()
    for s in range(args.steps if ctx64 else 0):   # the FP64 and converged trajectories
        l2_flush()
        ctx64.mark(0)
        s64 = ctx64.step(prm64)
        ctx64.mark(1)
        rec["ms64"].append(ctx64.elapsed(0, 1))
        rec["iters64"].append(s64.iters)
        rec["rres64"].append(s64.residual / s64.b_norm if s64.b_norm > 0 else 0.0)
        for k in d64:   # the comparison runs' fields into buffers allocated once
            ctx64.download_ptr(k, d64[k].ctypes.data)
        rec["err"].append({k: rel_err(saved[k][s], d64[k], tmp) for k in saved})
        if ctxT:
            ctxT.step(prmT)
            ctxT.download_ptr("p", pT.ctypes.data)
            rec["errT"].append({"mixed": rel_err(saved["p"][s], pT, tmp), "fp64": rel_err(d64["p"], pT, tmp)})

    # ---- per-kernel CUDA-event timing on extra steps, launch by launch (event
    # records cannot sit inside the replayed graph); same kernels and shapes
    def profile_steps(c, p):
        c.profile(1)
        tot = 0.0
        for _ in range(args.prof_steps):
            l2_flush()
            c.mark(0)
            c.step(p)
            c.mark(1)
            tot += c.elapsed(0, 1)
        c.sync()
        out = c.profile_all()
        c.profile(0)
        return out, tot

    prof, prof_ms = profile_steps(ctx, prm)
    t_dev = max_over_ranks(sum(rec["ms"]) / 1e3, pg, "cuda" if torch.cuda.is_available() else "cpu")
    t_e2e = max_over_ranks(sum(rec["e2e_s"]), pg, "cuda" if torch.cuda.is_available() else "cpu")
    value = world * n * args.steps / t_dev / 1e6
    e2e = {"value": world * n * args.steps / t_e2e / 1e6, "unit": UNIT,
           "h2d_bytes_per_step": 8 * n * len(in_keys), "d2h_bytes_per_step": 8 * n * len(out_keys),
           "timing": "host wall clock of one les_step_io call per timed step (the same steps as value): "
                     "upload of the step's fields from pinned host memory, the step, and the downloads -- "
                     "those of u_new, v_new, w_new, nu_t and p_rhs overlapping the pressure solve",
           "ms_per_step": {"les_step_io": 1e3 * t_e2e / args.steps, "step_device": 1e3 * t_dev / args.steps},
           "steps_ms": [[round(1e3 * a, 2), round(b, 2)] for a, b in zip(rec["e2e_s"], rec["ms"])],
           "host_link_gbs": link}

    # ---- roofline of the dominant kernel (CUDA events during the profiled steps)
    peak, peak_kind = measured_peak()
    roof = None
    if prof:
        name, (cnt, ms) = max(prof.items(), key=lambda kv: kv[1][1])
        bpc = alg_bytes_per_cell(name, args.fused)
        traffic = None
        tp = os.path.join(ROOT, "profiles", "traffic.json")
        if os.path.exists(tp):
            try:
                traffic = json.load(open(tp)).get(name, {}).get("dram_bytes_per_cell")
                traffic = traffic * n if traffic else None
            except Exception:
                traffic = None
        if bpc:
            achieved = bpc * n * cnt / (ms / 1e3) / 1e9
            roof = {"bound": "hbm", "kernel": name, "achieved": achieved, "peak": peak, "unit": "GB/s",
                    "frac": achieved / peak, "peak_source": peak_kind, "traffic": traffic,
                    "alg_bytes_per_launch": bpc * n, "launches": cnt, "avg_launch_us": 1e3 * ms / cnt,
                    "share_of_step": ms / (prof_ms or 1.0), "profiled_steps": args.prof_steps,
                    "kernels": {k: {"launches": v[0], "ms": v[1], "us_per_launch": 1e3 * v[1] / max(v[0], 1),
                                    "gbs": (alg_bytes_per_cell(k, args.fused) or 0) * n * v[0] / max(v[1], 1e-9) / 1e6}
                                for k, v in prof.items()}}

    solver = "GS-SOR (omega 1.7) FP64" if gs else "%s(4)-PCG mixed FP32/FP64" % args.precond
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t_dev / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64" if gs else "f32 inner / f64 outer",
            "data": "synthetic",
            "config": {"workload": "%s %s obstacle, %s to %s" %
                                   (args.workload, "x".join(map(str, shape)), solver,
                                    "max |dp| < 1e-6" if gs else "rel residual 1e-8"),
                       "cells": n, "parallelism": "replicas" if world > 1 else "single",
                       "l2": "flushed (256 MiB write) before every timed step",
                       "inner_rtol": args.inner_rtol, "tma": args.tma, "fused": args.fused,
                       "rows": args.rows, "chunks": args.chunks, "graph": args.graph,
                       "pdl": 1 if args.pdl is None else args.pdl, "phys32": args.phys32,
                       "autotune_us": tune_us, "strip_shape": shape_used},
            "e2e": e2e, "gpu_launches": launches, "wall_s": wall,
            "iters_mean": statistics.mean(rec["iters"]), "outer_mean": statistics.mean(rec["outer"]),
            "roofline": roof, "clocks": clk}
    if not gs:
        line["rel_residual_max"] = max(rec["rres"])
    if ctx64:
        t64 = sum(rec["ms64"]) / 1e3
        prof64, prof64_ms = profile_steps(ctx64, prm64)
        fp64_rate = ctx64.fp64_rate()
        kern = {}
        for k, (cnt, ms) in prof64.items():
            ops = FP64_OPS_PER_CELL.get(k)
            bpc = alg_bytes_per_cell(k)
            if not ops or not cnt:
                continue
            rate = ops * n * cnt / (ms / 1e3)
            kern[k] = {"launches": cnt, "us_per_launch": 1e3 * ms / cnt, "fp64_ops_per_cell": ops,
                       "fp64_gops": rate / 1e9, "fp64_frac": rate / fp64_rate,
                       "hbm_gbs": (bpc or 0) * n * cnt / (ms / 1e3) / 1e9,
                       "hbm_frac": (bpc or 0) * n * cnt / (ms / 1e3) / 1e9 / peak,
                       "share_of_step": ms / (prof64_ms or 1.0)}
        line["fp64"] = {"value": n * args.steps / t64 / 1e6, "ms_per_step": 1e3 * t64 / args.steps,
                        "iters_mean": statistics.mean(rec["iters64"]), "rel_residual_max": max(rec["rres64"]),
                        "roofline": {"bound": "fp64 pipe", "peak_fp64_gops": fp64_rate / 1e9,
                                     "peak_source": "measured live (les_fp64_rate: DMUL+DADD chains)",
                                     "kernels": kern}}
        line["speedup_vs_fp64"] = value / line["fp64"]["value"]
        line["err_vs_fp64_max"] = {k: max(e[k] for e in rec["err"]) for k in rec["err"][0]}
        if rec["errT"]:
            line["p_err_vs_converged_max"] = {
                "mixed": max(e["mixed"] for e in rec["errT"]), "fp64": max(e["fp64"] for e in rec["errT"]),
                "note": "max |p - p_conv| / max |p_conv|, p_conv from the same trajectory with every solve converged "
                        "to relative residual 1e-12 (FP64 defect correction): each run's own solve error; the "
                        "mixed-vs-FP64 difference is bounded by their sum"}
            line["p_err_steps"] = [{"vs_fp64": e["p"], "mixed_vs_conv": t["mixed"], "fp64_vs_conv": t["fp64"]}
                                   for e, t in zip(rec["err"], rec["errT"])]
    if rank == 0 and world == 1 and not args.no_cpu:
        oc = OracleCase(shape, h, solid, f, args.precond, args.solver, os.cpu_count() or 1)
        secs, its = [], []
        for q in range(max(1, args.cpu_steps)):
            t, it = oc.step()
            secs.append(t)
            its.append(it)
            if q == 0 and first is not None:   # FP64 parity at this size: the GPU's first step vs the oracle's
                line["fp64_vs_oracle_step0"] = {
                    "rel_err": {k: rel_err(first["fields"][k], oc.f[k]) for k in ("u", "v", "w", "p", "nu_t")},
                    "iters_gpu": first["iters"], "iters_oracle": it}
        line["cpu_baseline"] = {"value": n * len(secs) / sum(secs) / 1e6, "unit": UNIT, "cores": oc.threads,
                                "kind": "port", "iters": its,
                                "sample": "%d full FP64 time step(s) of the CPU oracle (%s, computed lambda_max) "
                                          "from the initial state at %s, %.1f s" %
                                          (len(secs), "GS-SOR" if gs else args.precond + "-PCG",
                                           "x".join(map(str, shape)), sum(secs))}
    if rank == 0:
        print(json.dumps(line), flush=True)
    for c in (ctx, ctx64, ctxT):
        if c:
            c.close()
    if pg:
        pg.barrier()
        pg.destroy_process_group()
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "batch":
        return run_batch(args)
    if args.workload == "adjoint":
        return run_adjoint(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
