"""Benchmark of the fixed-source sweep / source-iteration hot path on GB300.

Workload (one step = one complete fixed-source solve, Gauss-Seidel over
groups wrapping source iteration wrapping 8-octant sweeps, from a zero flux
to the tolerance): a 64^3 mesh of 1 cm cells, 8 groups, Gauss-Chebyshev
8 polar x 16 azimuthal = 128 directions, theta-weighted diamond difference
with theta = 0.7, four materials in a seeded checkerboard of 8^3 blocks
(sigma_t lognormal, median 1/cm; c ~ U[0.5, 0.95]; lower-triangular
scattering plus upscatter between the last two groups), unit group-0 source
in one seeded 8^3 block, vacuum boundaries.  Synthetic inputs from the seeded
generator in doma_gb300.problems.

metric: cell * direction * group updates per second (Gupdates/s) over whole
solves; the sweep runs in FP32 with compensated angular sums, sources,
fluxes and every norm in FP64.

  value     device-resident: the solver is created once; each step re-zeroes
            the flux and solves.  CUDA events on the solver's stream around
            each step; L2 is flushed (a 512 MB write) between steps.
  e2e       through the C ABI with host buffers: create (H2D of the problem),
            solve, read the flux back (D2H), destroy -- wall clock per step.
  roofline  the sweep kernels alone (bare sweeps of group 0), achieved
            algorithmic bytes (6 s + 3 s / D_oct per update, s = 4) per second
            against the measured HBM copy bandwidth.
  roofline_all_groups  the same kernel with all 8 groups in flight in one
            launch (the multigroup iteration's sweep), same byte count.
  cpu_baseline  the CPU restatement of DOMA's OpenMP sweep (oracle/) on the
            host cores, a bounded sample of source iterations of group 0.

--impl reference runs DOMA's CPU algorithm (the oracle port, the reference's
own code cannot be compiled on this host) on the same workload and metric.
Replicas only: with --gpus N each rank solves its own replica (weak scaling).

`python bench.py profile [...]` runs a small fixed workload for ncu captures
instead (see profile_main).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "sweep Gupdates/s over full fixed-source solves (time to tolerance per step)"
UNIT = "Gupdates/s"


def workload(seed: int = 0, n: int = 64):
    from doma_gb300 import problems as P
    p = P.checkerboard(seed, n=n, groups=8, np_=4, na=4, block=8)
    return p


def options(precision: str = "fp32", tol: float = 1e-8):
    from doma_gb300 import problems as P
    return P.make_options(scheme="tw_dd", theta=0.7, precision=precision, fs_tol=tol,
                          fs_max_it=5000, mg_tol=tol, mg_max_it=500)


def config_dict(p, args, extra=None):
    d = {"workload": "checkerboard_64cube_8g_128dir_twdd_theta0.7",
         "cells": p.num_cells, "groups": p.num_groups, "directions": p.num_directions,
         "scheme": "tw_dd", "theta": 0.7, "tolerance": args.tol,
         "l2": "flushed between steps (512 MB write)", "parallelism": "replicas"}
    if extra:
        d.update(extra)
    return d


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def aggregate(total_ms: float, units: float, world: int, device=None) -> tuple[float, float]:
    """Whole-job figures of `world` replicas: the slowest rank's time and the
    units (updates) of all ranks -> (units per second / 1e9, max total ms).
    With world > 1 it needs an initialised process group (NCCL on GPUs, gloo
    on CPUs); every rank gets the same result."""
    if world > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([total_ms], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        u = torch.tensor([float(units)], dtype=torch.float64, device=device)
        dist.all_reduce(u)
        total_ms, units = float(t.item()), float(u.item())
    return float(units) / (total_ms / 1e3) / 1e9, total_ms


class ClockSampler:
    """nvidia-smi samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = Path(os.environ.get("TMPDIR", "/tmp")) / f"doma_clocks_{os.getpid()}.csv"

    def __enter__(self):
        self.fh = None
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
            if self.fh is not None:
                self.fh.close()
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        if self.proc is None or not self.path.exists():
            self.path.unlink(missing_ok=True)
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        self.path.unlink(missing_ok=True)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "reasons": sorted(reasons), "samples": len(sm)}


# DRAM traffic of one sweep launch on this workload (dram__bytes_read.sum +
# dram__bytes_write.sum from one ncu capture of sweep_persistent_kernel, FP32
# TW-DD, 64^3, 128 directions).  Far below the algorithmic bytes: the sweep's
# working set stays in L2.
SWEEP_DRAM_BYTES_PER_LAUNCH = 2_709_504 + 924_160
# the same kernel with all 8 groups in flight: mean of two captured launches
# (dram__bytes_read.sum + dram__bytes_write.sum)
ALL_GROUPS_DRAM_BYTES_PER_LAUNCH = 41_324_672 + 305_230_080


def measured_peak_hbm():
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        try:
            return float(json.loads(f.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


def cpu_sample(p, opts, threads: int, iters: int):
    """Time `iters` source iterations of group 0 with the CPU restatement."""
    sys.path.insert(0, str(ROOT / "tests"))
    import oracle_lib as ol
    ol.oracle()  # build/load before timing
    t0 = time.perf_counter()
    ol.oracle_source_iterations(p, opts, 0, iters, threads=threads)
    dt = time.perf_counter() - t0
    upd = iters * p.updates_per_sweep()
    return upd / dt / 1e9, dt, upd


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from doma_gb300 import problems as P  # noqa: F401
    p = workload(args.seed)
    opts = options("fp64", args.tol)
    threads = os.cpu_count() or 1
    for _ in range(args.warmup if args.warmup < 1 else 1):
        cpu_sample(p, opts, threads, 1)
    times, upds = [], []
    for _ in range(args.steps):
        rate, dt, upd = cpu_sample(p, opts, threads, args.ref_iters)
        times.append(dt)
        upds.append(upd)
    value = sum(upds) / sum(times) / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * sum(times) / len(times), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": config_dict(p, args, {"sample": f"{args.ref_iters} source iterations of group 0 per step"}),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{args.ref_iters} source iterations (sweep + residual + update) "
                                   f"of group 0 per step, {threads} OpenMP threads over the "
                                   f"ordinates of each octant (DOMA's parallel-in-angle scheme)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


WEIGHTS = ROOT / "doma_gb300" / "learned" / "weights" / "unet_c32.npz"


def drivers_leg(args):
    """The eigenvalue and transient drivers on one fissile problem: 48^3 cells,
    4 groups, 128 directions, FP32 DD sweeps (FP64 norms), fission in two of
    four materials, 3 and 2 delayed groups and a source step of each kind.
    Reports each driver's update rate and time, and the CPU restatement's
    update rate (all host threads) on a bounded sample of the same sweeps."""
    from doma_gb300 import problems as P
    from doma_gb300.solver import Solver
    p, tr = P.transient_problem(args.seed + 7, dims=3, nx=48, ny=48, nz=48, groups=4, np_=4,
                                na=4, materials=4, num_steps=4, t1=0.4)
    kw = dict(scheme="dd", precision="fp32", fs_tol=1e-6, fs_max_it=5000, mg_tol=1e-5,
              mg_max_it=500)
    out = {"workload": "48^3 cells, 4 groups, 8x16 directions, DD FP32, random materials "
                       "(2 fissile), 4 transient steps of dt = 0.1"}
    # power iteration to a shape residual of 1e-3 and |dk| <= 1e-4 (the kernels are
    # warm from the legs before; the host-driven loop has no graph to build)
    with Solver(p, P.make_options(**{**kw, "mg_tol": 1e-3, "mg_max_it": 1000})) as s:
        rep, k = s.solve_eigenvalue(1e-4)
    out["eigen"] = {"k": k, "converged": rep.converged, "power_iterations": rep.mg_iterations,
                    "mg_tol": 1e-3, "k_tol": 1e-4,
                    "sweeps": rep.si_iterations, "ms": rep.solve_ms,
                    "ms_per_power_iteration": rep.solve_ms / max(rep.mg_iterations, 1),
                    "gupdates": rep.updates / rep.solve_ms / 1e6}
    with Solver(p, P.make_options(**kw)) as s:
        s.solve_transient(tr)                            # warm
        rep = s.solve_transient(tr)
    out["transient"] = {"steps": tr.num_steps, "converged": rep.converged,
                        "sweeps": rep.si_iterations, "ms": rep.solve_ms,
                        "ms_per_step": rep.solve_ms / tr.num_steps,
                        "gupdates": rep.updates / rep.solve_ms / 1e6}
    if not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        rate, dt, upd = cpu_sample(p, P.make_options(**{**kw, "precision": "fp64"}), threads,
                                   args.driver_cpu_iters)
        out["cpu_rate"] = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
                           "sample": f"{args.driver_cpu_iters} source iterations of group 0 "
                                     f"({upd / 1e6:.1f} M updates, {dt:.1f} s)"}
    return out


def batch_leg(args):
    """The batched solve: `--batch-problems` independent problems drawn by
    batch_mix (n ~ U{16..96}, G in {1, 2, 4, 8, 16}, 2k x 4k directions with
    k ~ U{2..6}), FP32 DD multigroup iteration to 1e-6, every problem's sweep
    in one persistent launch per iteration.  The block shapes are tuned first;
    the solve is timed alone.  Each problem's error against an FP64 solution
    is reported for `--batch-error-problems` of them (the cheapest FP64 solve
    of each group count first, then by FP64 cost): the FP64 drop-in mode costs
    about 1000 s for all 256."""
    import torch

    from doma_gb300 import problems as P
    from doma_gb300.solver import Batch, Solver
    ps = P.batch_mix(args.seed, count=args.batch_problems)
    with Batch(ps, scheme="dd", precision="fp32", fs_tol=1e-6, fs_max_it=5000,
               iteration="multigroup") as b:
        t0 = time.perf_counter()
        tx = b.tune()
        tune_s = time.perf_counter() - t0
        tiles = b.tiles()
        tune = b.tune_report()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        reps = b.solve()
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        cost = [p.updates_per_sweep() * p.num_groups for p in ps]
        order = sorted(range(len(ps)), key=lambda i: cost[i])
        picked = []
        for g in sorted({p.num_groups for p in ps}):
            picked += [i for i in order if ps[i].num_groups == g][:1]
        picked += [i for i in order if i not in picked]
        picked = picked[:max(0, args.batch_error_problems)]
        errors = []
        for i in picked:
            p = ps[i]
            phi32 = b.scalar_flux(i)
            with Solver(p, P.make_options(scheme="dd", precision="fp64", fs_tol=1e-10,
                                          fs_max_it=20000, iteration="multigroup")) as s64:
                s64.solve_fixed_source()
                phi64 = s64.scalar_flux()
            errors.append({"problem": i, "name": p.name, "cells": p.num_cells,
                           "groups": p.num_groups, "directions": p.num_directions,
                           "iterations": reps[i].mg_iterations,
                           "error_vs_fp64_rel_l2": float(np.linalg.norm(phi32 - phi64)
                                                         / np.linalg.norm(phi64))})
    upd = sum(r.updates for r in reps)
    its = [r.mg_iterations for r in reps]
    return {"problems": len(ps), "tile_x": tx, "solve_s": dt, "gupdates": upd / dt / 1e9,
            "tune_s": tune_s, "tune": tune,
            "tiles_used": {str(k): tiles.count(k) for k in (8, 16, 32)},
            "converged": sum(r.converged for r in reps), "iterations_min": min(its),
            "iterations_max": max(its), "updates": upd,
            "errors_vs_fp64": errors,
            "error_max": max((e["error_vs_fp64_rel_l2"] for e in errors), default=None)}


def timed_solve(solver, stream, flush, warm: bool = True):
    """One fixed-source solve timed with CUDA events on the solver's stream,
    after a warm-up solve and an L2 flush."""
    import torch
    if warm:
        solver.solve_fixed_source()
    flush.fill_(1.0)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    rep = solver.solve_fixed_source()
    e1.record(stream)
    e1.synchronize()
    return rep, e0.elapsed_time(e1)


def timed_sweeps(solver, stream, group: int, count: int) -> float:
    """ms per bare sweep of `group` (CUDA events on the solver's stream)."""
    import torch
    solver.source_iterations(group, 1)
    solver.sweeps(group, 2)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    solver.sweeps(group, count)
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1) / count


def timed_source_iterations(solver, stream, group: int, count: int) -> float:
    """ms per source iteration (sweep + epilogue) of `group`, warm, CUDA events."""
    import torch
    solver.source_iterations(group, 2)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    solver.source_iterations(group, count)
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1) / count


def roofline_entry(ms: float, updates: float, d_oct: int, s_bytes: int, peak: float, peak_kind: str,
                   traffic=None, traffic_source=None):
    b_upd = 6 * s_bytes + 3 * s_bytes / d_oct
    achieved = b_upd * updates / (ms / 1e3) / 1e9
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "traffic": traffic, "traffic_source": traffic_source,
            "peak_source": peak_kind, "bytes_per_update": b_upd, "sweep_ms": ms,
            "updates_per_launch": updates}


# DRAM traffic of one sweep launch on the 100^3, 288-direction duct problem
# (dram__bytes_read.sum + dram__bytes_write.sum, one ncu capture).  The
# 320 MB of double partials (5 ordinate groups of 8 x 8 octants x 10^6 cells)
# do not fit in L2, so most of it is their write-back.
STREAMING_SWEEP_DRAM_BYTES = 30_568_960 + 346_246_912


def streaming_leg(args, stream, flush):
    """The streaming/shielding workload: 100^3 cells of 1 cm, one group,
    12 x 24 = 288 directions (36 ordinates per octant), DD, a 10 cm near-void
    duct (sigma_t = 1e-4, c = 0.5) on a seeded 3-segment path from a 10^3
    corner source through an absorber (sigma_t = 0.1, c = 0.5).  FP32 sweeps
    with FP64 norms to the FP32 floor (1e-6), the FP64 drop-in mode to DOMA's
    1e-8, the bare sweep's roofline, and the CPU restatement's rate."""
    import torch

    from doma_gb300 import problems as P
    from doma_gb300.solver import Solver
    p = P.streaming_duct(args.seed, n=100, np_=6, na=6)
    o32 = P.make_options(scheme="dd", precision="fp32", fs_tol=1e-6, fs_max_it=5000, mg_tol=1e-6)
    o64 = P.make_options(scheme="dd", precision="fp64", fs_tol=1e-8, fs_max_it=5000, mg_tol=1e-8)
    peak, peak_kind = measured_peak_hbm()
    with Solver(p, o32) as s:
        s.set_stream(stream.cuda_stream)
        rep, ms = timed_solve(s, stream, flush)
        phi32 = s.scalar_flux()
        sweep_ms = timed_sweeps(s, stream, 0, args.roofline_sweeps)
        desc = s.describe()
    with Solver(p, o64) as s64:
        s64.set_stream(stream.cuda_stream)
        rep64, ms64 = timed_solve(s64, stream, flush)
        phi64 = s64.scalar_flux()
    out = {"workload": "streaming_duct_100cube_1g_288dir_dd", "cells": p.num_cells,
           "directions": p.num_directions, "directions_per_octant": p.directions_per_octant,
           "fp32": {"time_to_tolerance_ms": ms, "tolerance": 1e-6, "sweeps": rep.si_iterations,
                    "converged": rep.converged, "gupdates": rep.updates / ms / 1e6,
                    "tile": list(desc["tile"])},
           "fp64_dropin": {"time_to_tolerance_ms": ms64, "tolerance": 1e-8,
                           "sweeps": rep64.si_iterations, "converged": rep64.converged,
                           "gupdates": rep64.updates / ms64 / 1e6},
           "error_fp32_vs_fp64_rel_l2": float(np.linalg.norm(phi32 - phi64) / np.linalg.norm(phi64)),
           "roofline": roofline_entry(sweep_ms, p.updates_per_sweep(), p.directions_per_octant, 4,
                                      peak, peak_kind, STREAMING_SWEEP_DRAM_BYTES,
                                      "ncu capture of one launch" if STREAMING_SWEEP_DRAM_BYTES
                                      else None)}
    out["roofline"]["gupdates"] = p.updates_per_sweep() / (sweep_ms / 1e3) / 1e9
    if not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        rate, dt, upd = cpu_sample(p, o64, threads, args.streaming_cpu_iters)
        out["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
                               "sample": f"{args.streaming_cpu_iters} source iterations of the "
                                         f"group ({upd / 1e6:.0f} M updates, {dt:.1f} s), "
                                         f"{threads} OpenMP threads over the 36 ordinates of "
                                         f"each octant"}
        out["cpu_time_to_tolerance_estimate_s"] = rep64.updates / (rate * 1e9)
    return out


def small_leg(args, stream, flush):
    """The small CPU-runnable workload: a 10 cm cube of 20^3 cells, 2 groups,
    4 x 8 = 32 directions, DD, downscatter, a central 5^3 unit source; the
    FP64 drop-in mode to DOMA's 1e-8 (time to tolerance, warm), and the CPU
    restatement's full solve on all host threads."""
    from doma_gb300 import problems as P
    from doma_gb300.solver import Solver
    sys.path.insert(0, str(ROOT / "tests"))
    p = P.small_cube(args.seed, n=20)
    o64 = P.make_options(scheme="dd", precision="fp64", fs_tol=1e-8, mg_tol=1e-8)
    with Solver(p, o64) as s:
        s.set_stream(stream.cuda_stream)
        rep, ms = timed_solve(s, stream, flush)
    out = {"workload": "small_cube_20cube_2g_32dir_dd", "cells": p.num_cells,
           "fp64_dropin": {"time_to_tolerance_ms": ms, "sweeps": rep.si_iterations,
                           "mg_iterations": rep.mg_iterations, "converged": rep.converged,
                           "gupdates": rep.updates / ms / 1e6}}
    if not args.no_cpu_baseline:
        import oracle_lib as ol
        threads = os.cpu_count() or 1
        ol.oracle()
        t0 = time.perf_counter()
        _, ok, si, mg, _ = ol.oracle_solve(p, o64, threads=threads)
        dt = time.perf_counter() - t0
        upd = int(sum(si)) * p.updates_per_sweep()
        out["cpu_baseline"] = {"time_to_tolerance_ms": dt * 1e3, "value": upd / dt / 1e9,
                               "unit": UNIT, "cores": threads, "kind": "port",
                               "sample": "one full solve to 1e-8 (the oracle's OpenMP "
                                         "parallel-in-angle sweep: 4 ordinates per octant)"}
    return out


def learned_leg(args):
    """Time to args.learned_target relative L2 error against the FP64 solution,
    plain multigroup FP32 source iteration vs the same with learned corrections,
    on held-out learned-accelerator problems (64^3, 8 groups, 6x12 directions,
    c ~ U[0.9, 0.999])."""
    from doma_gb300 import problems as P
    from doma_gb300.learned import evaluate as E
    from doma_gb300.learned.net import UNet

    if not WEIGHTS.exists():
        return {"unavailable": "no trained weights file"}
    net = UNet(seed=0)
    net.load(WEIGHTS)
    rows = []
    for i in range(args.learned_problems):
        p = P.learned_problem(1_000_001 + i, n=args.learned_n, groups=8)
        t0 = time.perf_counter()
        ref, info = E.reference_flux(p, tol=1e-9)
        ref_s = time.perf_counter() - t0
        plain = E.time_to_error(p, ref, args.learned_target, max_it=20000)
        lrn = E.time_to_error(p, ref, args.learned_target, net=net, first=args.accel_first,
                              interval=args.accel_interval, max_corrections=64, max_it=20000)
        gs = E.time_to_error_gs(p, ref, args.learned_target) if args.learned_gs else None
        rows.append({"problem": p.name, "fp64_reference_s": ref_s,
                     "gauss_seidel_ms": gs["ms"] if gs else None,
                     "gauss_seidel_tolerance": gs["tolerance"] if gs else None,
                     "gauss_seidel_error": gs["error"] if gs else None,
                     "gauss_seidel_sweeps": gs.get("sweeps") if gs else None,
                     "fp64_reference_iterations": info["iterations"],
                     "plain_ms": plain["ms"], "plain_iterations": plain["iterations"],
                     "plain_error": plain["error"],
                     "learned_ms": lrn["ms"], "learned_iterations": lrn["iterations"],
                     "learned_error": lrn["error"], "corrections_kept": lrn["accepted"],
                     "corrections_undone": lrn["rejected"]})
    net.close()
    plain_ms = sum(r["plain_ms"] for r in rows)
    learned_ms = sum(r["learned_ms"] for r in rows)
    per = [r["plain_ms"] / r["learned_ms"] for r in rows if r["learned_ms"]]
    per_gs = [r["gauss_seidel_ms"] / r["learned_ms"] for r in rows
              if r["learned_ms"] and r["gauss_seidel_ms"]]
    return {"target_rel_l2": args.learned_target,
            "speedup_mean": float(np.mean(per)) if per else None,
            "speedup_min": float(np.min(per)) if per else None,
            "speedup_vs_gauss_seidel_mean": float(np.mean(per_gs)) if per_gs else None,
            "speedup_vs_gauss_seidel_min": float(np.min(per_gs)) if per_gs else None,
            "workload": f"{args.learned_n}^3 cells, 8 groups, 6x12 directions, DD, sigma_t lognormal "
                        "field (log-sigma 0.8, correlation 4 cells), c ~ U[0.9, 0.999]",
            "plain_ms": plain_ms, "learned_ms": learned_ms,
            "speedup": plain_ms / learned_ms if learned_ms > 0 else None,
            "accel": {"first": args.accel_first, "interval": args.accel_interval, "guard": True},
            "problems": rows}


def run_ours(args):
    import torch
    import torch.distributed as dist

    from doma_gb300 import problems as P
    from doma_gb300.solver import Solver

    rank, world, local = dist_env()
    if world > 1:
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    p = workload(args.seed + rank)
    opts = options(args.precision, args.tol)
    # A dedicated (non-NULL) stream: the solver launches on it and the CUDA
    # events below are recorded on it, so they bracket exactly its kernels.
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    # -- device-resident leg ------------------------------------------------
    solver = Solver(p, opts)
    solver.set_stream(stream.cuda_stream)
    for _ in range(args.warmup):
        rep = solver.solve_fixed_source()
        assert rep.converged, "warm-up solve did not converge"
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    step_ms, updates, launches = [], 0, 0
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            flush.fill_(1.0)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            rep = solver.solve_fixed_source()
            e1.record(stream)
            e1.synchronize()
            step_ms.append(e0.elapsed_time(e1))
            updates += rep.updates
            launches += rep.kernel_launches
            assert rep.converged
    torch.cuda.synchronize()
    value, total_ms = aggregate(sum(step_ms), updates, world, dev)
    last_rep = rep
    phi32 = solver.scalar_flux()

    # -- roofline: the sweep kernels alone ------------------------------------
    solver.source_iterations(0, 1)
    nsw = args.roofline_sweeps
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    solver.sweeps(0, nsw)
    e1.record(stream)
    e1.synchronize()
    sweep_ms = e0.elapsed_time(e1) / nsw
    desc = solver.describe()
    s_bytes = 4 if args.precision == "fp32" else 8
    d_oct = p.directions_per_octant
    b_upd = 6 * s_bytes + 3 * s_bytes / d_oct
    upd_sweep = p.updates_per_sweep()
    achieved = b_upd * upd_sweep / (sweep_ms / 1e3) / 1e9
    peak, peak_kind = measured_peak_hbm()
    solver.close()

    # -- the same sweep kernel with every group of the problem in flight (the
    # multigroup iteration's sweep: one persistent launch over G groups) ----------
    roof_all = None
    if args.all_groups_roofline:
        mg_opts = P.make_options(scheme="tw_dd", theta=0.7, precision=args.precision, fs_tol=args.tol,
                                 fs_max_it=5000, iteration="multigroup")
        with Solver(p, mg_opts) as smg:
            smg.set_stream(stream.cuda_stream)
            smg.source_iterations(0, 1)
            smg.sweeps(0, 3)
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            smg.sweeps(0, nsw)
            e1.record(stream)
            e1.synchronize()
            mg_ms = e0.elapsed_time(e1) / nsw
        mg_achieved = b_upd * upd_sweep * p.num_groups / (mg_ms / 1e3) / 1e9
        roof_all = {"bound": "hbm", "achieved": mg_achieved, "peak": peak, "unit": "GB/s",
                    "frac": mg_achieved / peak,
                    "traffic": ALL_GROUPS_DRAM_BYTES_PER_LAUNCH if args.precision == "fp32" else None,
                    "traffic_source": "ncu capture of two launches (dram__bytes_read + dram__bytes_write)",
                    "sweep_ms": mg_ms, "groups_in_flight": p.num_groups,
                    "gupdates": upd_sweep * p.num_groups / (mg_ms / 1e3) / 1e9}

    # -- FP64 drop-in reference solution and its rate ----------------------------
    err = None
    fp64 = None
    if args.fp64_check:
        # the FP64 reference converged tightly (1e-8), independent of --tol; its
        # rate is then taken warm with CUDA events over source iterations of group 0
        with Solver(p, options("fp64", 1e-8)) as s64:
            s64.set_stream(stream.cuda_stream)
            t0 = time.perf_counter()
            r64 = s64.solve_fixed_source()
            torch.cuda.synchronize()
            dt64 = time.perf_counter() - t0
            phi64 = s64.scalar_flux()
            si_ms = timed_source_iterations(s64, stream, 0, args.fp64_iters)
            sw_ms = timed_sweeps(s64, stream, 0, max(3, args.fp64_iters // 2))
        err = float(np.linalg.norm(phi32 - phi64) / np.linalg.norm(phi64))
        upd_sweep = p.updates_per_sweep()
        fp64 = {"gupdates": upd_sweep / (si_ms / 1e3) / 1e9, "source_iteration_ms": si_ms,
                "sweep_ms": sw_ms, "sweep_gupdates": upd_sweep / (sw_ms / 1e3) / 1e9,
                "sample": f"{args.fp64_iters} warm source iterations of group 0, CUDA events",
                "reference_solve": {"tolerance": 1e-8, "sweeps": r64.si_iterations,
                                    "wall_s_first_solve": dt64}}

    # -- e2e through the C ABI with host buffers ---------------------------------
    h2d = (p.dx.nbytes + p.dy.nbytes + p.dz.nbytes + p.cell_material.nbytes + p.total.nbytes
           + p.scatter.nbytes + (p.source.nbytes if p.source is not None else 0))
    d2h = p.num_groups * p.num_cells * 8
    e2e_times, e2e_upd = [], 0
    for i in range(args.e2e_steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        with Solver(p, opts) as s:
            r = s.solve_fixed_source()
            _ = s.scalar_flux()
        torch.cuda.synchronize()
        e2e_times.append(time.perf_counter() - t0)
        e2e_upd += r.updates
    e2e_value = e2e_upd / sum(e2e_times) / 1e9 * world

    if rank != 0:
        if world > 1:
            dist.barrier()
            dist.destroy_process_group()
        return

    cpu = None
    if not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        rate, dt, upd = cpu_sample(p, options("fp64", args.tol), threads, args.cpu_iters)
        cpu = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{args.cpu_iters} source iterations of group 0 ({upd / 1e6:.1f} M updates, "
                         f"{dt:.1f} s), {threads} OpenMP threads over ordinates"}

    streaming = streaming_leg(args, stream, flush) if args.streaming else None
    small = small_leg(args, stream, flush) if args.small else None
    learned = learned_leg(args) if args.learned_problems > 0 else None
    drivers = drivers_leg(args) if args.drivers else None
    batch = batch_leg(args) if args.batch_problems > 0 else None

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f32" if args.precision == "fp32" else "f64", "data": "synthetic",
        "config": config_dict(p, args, {"precision": args.precision,
                                        "tile": list(desc["tile"]),
                                        "si_sweeps_per_solve": last_rep.si_iterations,
                                        "mg_iterations": last_rep.mg_iterations}),
        "time_to_tolerance_ms": total_ms / args.steps,
        "error_vs_fp64_rel_l2": err,
        "fp64_dropin": fp64,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak,
                     "traffic": SWEEP_DRAM_BYTES_PER_LAUNCH if args.precision == "fp32" else None,
                     "traffic_source": "ncu capture of one launch (dram__bytes_read + dram__bytes_write)",
                     "peak_source": peak_kind,
                     "bytes_per_update": b_upd, "sweep_ms": sweep_ms,
                     "sweep_launches": desc["launches_per_sweep"]},
        "roofline_all_groups": roof_all,
        "cpu_baseline": cpu,
        "streaming": streaming,
        "small": small,
        "learned": learned,
        "drivers": drivers,
        "batch": batch,
        "gpu_launches": launches,
        "clocks": clocks.summary(),
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()


def profile_main(argv) -> None:
    """`python bench.py profile ...`: a small, self-contained workload for ncu.

    Builds the seeded checkerboard problem on cuda:0, sets up group 0's source
    with one source iteration, then runs `--sweeps` bare sweeps (or, with
    --solve, one full fixed-source solve) and prints the solver's block shape
    and launch counts.  With --iteration multigroup every group is in flight in
    each sweep launch.  --streaming selects the 100^3, 288-direction DD duct
    problem instead.  With --unet-forward K it runs K forward passes of the
    learned accelerator's U-Net (the committed weights) on an n^3 volume of
    `--batch` samples.  Device memory stays well under a few GB."""
    ap = argparse.ArgumentParser(prog="bench.py profile")
    ap.add_argument("--n", type=int, default=64)
    ap.add_argument("--groups", type=int, default=8)
    ap.add_argument("--np", dest="np_", type=int, default=4)
    ap.add_argument("--na", type=int, default=4)
    ap.add_argument("--precision", choices=["fp32", "fp64"], default="fp32")
    ap.add_argument("--scheme", choices=["dd", "tw_dd"], default="tw_dd")
    ap.add_argument("--theta", type=float, default=0.7)
    ap.add_argument("--tile", type=int, default=0)
    ap.add_argument("--sweeps", type=int, default=3)
    ap.add_argument("--solve", action="store_true")
    ap.add_argument("--schedule", choices=["persistent", "levels"], default="persistent")
    ap.add_argument("--loop", choices=["graph", "host"], default="graph",
                    help="host: host-driven solve loop (kernels profilable one by one)")
    ap.add_argument("--iteration", choices=["gauss_seidel", "multigroup"], default="gauss_seidel")
    ap.add_argument("--unet-forward", type=int, default=0)
    ap.add_argument("--unet-backward", type=int, default=0,
                    help="K training steps (forward, loss, backward, Adam) of the U-Net")
    ap.add_argument("--batch", type=int, default=1)
    ap.add_argument("--streaming", action="store_true",
                    help="the 100^3 duct problem (one group, 12 x 24 directions, DD)")
    a = ap.parse_args(argv)
    if a.unet_forward > 0 or a.unet_backward > 0:
        profile_unet_forward(a)
        return
    if a.schedule == "levels":
        os.environ["DOMA_SWEEP_SCHEDULE"] = "levels"
    if a.loop == "host":
        os.environ["DOMA_SOLVE_LOOP"] = "host"

    import torch

    from doma_gb300 import problems as P
    from doma_gb300.solver import Solver

    torch.cuda.set_device(0)
    if a.streaming:
        p = P.streaming_duct(0, n=100, np_=6, na=6)
    else:
        p = P.checkerboard(0, n=a.n, groups=a.groups, np_=a.np_, na=a.na, block=8)
    o = P.make_options(scheme=a.scheme, theta=a.theta, precision=a.precision,
                       fs_tol=1e-6 if a.precision == "fp32" else 1e-8,
                       mg_tol=1e-6 if a.precision == "fp32" else 1e-8,
                       fs_max_it=5000, mg_max_it=500, tile=(a.tile, 0, 0),
                       iteration=a.iteration)
    with Solver(p, o) as s:
        t0 = time.perf_counter()
        if a.solve:
            r = s.solve_fixed_source()
            extra = {"converged": r.converged, "si_iterations": r.si_iterations,
                     "mg_iterations": r.mg_iterations}
        else:
            s.source_iterations(0, 1)
            s.sweeps(0, a.sweeps)
            extra = {"sweeps": a.sweeps}
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        print(json.dumps({"workload": p.name, "precision": a.precision, "scheme": a.scheme,
                          "seconds": round(dt, 4), **extra, **s.describe()}))


def profile_unet_forward(a) -> None:
    """K forward passes (--unet-forward K) or K training steps (--unet-backward
    K: forward, mean-square loss against a random target, backward, Adam) of
    the U-Net with the committed weights on an n^3 volume of --batch samples;
    prints the CUDA-event time per pass or step."""
    import torch

    from doma_gb300.learned.net import UNet

    torch.cuda.set_device(0)
    weights = str(WEIGHTS)
    with UNet(seed=0) as net:
        net.load(weights)
        net.set_stream(torch.cuda.current_stream().cuda_stream)
        g = torch.Generator(device="cuda").manual_seed(0)
        x = torch.randn((a.batch, a.n, a.n, a.n, 16), generator=g, device="cuda").to(torch.bfloat16)
        y = torch.empty((a.batch, a.n, a.n, a.n), dtype=torch.float32, device="cuda")
        t = torch.randn((a.batch, a.n, a.n, a.n), generator=g, device="cuda")
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        count = a.unet_backward if a.unet_backward > 0 else a.unet_forward
        torch.cuda.synchronize()
        e0.record()
        for _ in range(count):
            if a.unet_backward > 0:
                net.backward(x, t)
                net.adam(1e-6)
            else:
                net.forward(x, y)
        e1.record()
        torch.cuda.synchronize()
        kind = "training_step" if a.unet_backward > 0 else "forward"
        print(json.dumps({"workload": f"unet_{kind}_{a.n}cube_batch{a.batch}", "count": count,
                          f"ms_per_{kind}": e0.elapsed_time(e1) / count}))


def main():
    if len(sys.argv) > 1 and sys.argv[1] == "profile":
        profile_main(sys.argv[2:])
        return
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--precision", choices=["fp32", "fp64"], default="fp32")
    ap.add_argument("--tol", type=float, default=1e-6)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--roofline-sweeps", type=int, default=50)
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--ref-iters", type=int, default=30,
                    help="source iterations of group 0 per --impl reference step")
    ap.add_argument("--cpu-iters", type=int, default=300,
                    help="source iterations of group 0 in the cpu_baseline sample (about 10 s)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--fp64-check", type=int, default=1)
    ap.add_argument("--all-groups-roofline", type=int, default=1,
                    help="also time the sweep with every group in flight (multigroup mode)")
    ap.add_argument("--fp64-iters", type=int, default=20,
                    help="warm FP64 source iterations timed for the drop-in rate")
    ap.add_argument("--streaming", type=int, default=1,
                    help="also time the 100^3, 288-direction duct problem (0: skip)")
    ap.add_argument("--streaming-cpu-iters", type=int, default=6)
    ap.add_argument("--small", type=int, default=1,
                    help="also time the 20^3, 2-group, 32-direction problem (0: skip)")
    ap.add_argument("--batch-error-problems", type=int, default=10,
                    help="batched problems whose error against FP64 is measured")
    ap.add_argument("--learned-problems", type=int, default=3)
    ap.add_argument("--drivers", type=int, default=1,
                    help="also time the eigenvalue and transient drivers (0: skip)")
    ap.add_argument("--driver-cpu-iters", type=int, default=20)
    ap.add_argument("--batch-problems", type=int, default=256,
                    help="also time the batched solve of this many problems (0: skip)")
    ap.add_argument("--learned-n", type=int, default=64)
    ap.add_argument("--learned-gs", type=int, default=1,
                    help="also time DOMA's Gauss-Seidel order (FP32) to the same error")
    ap.add_argument("--learned-target", type=float, default=1e-5)
    ap.add_argument("--accel-first", type=int, default=10)
    ap.add_argument("--accel-interval", type=int, default=10)
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
