"""A small, self-contained sweep workload for profilers (ncu) and timing.

    python -m doma_gb300.profile_case [--n 64] [--groups 8] [--np 4] [--na 4]
        [--precision fp32|fp64] [--scheme dd|tw_dd] [--tile 8] [--sweeps 3]
        [--solve] [--schedule persistent|levels] [--loop graph|host]
        [--iteration gauss_seidel|multigroup]
    python -m doma_gb300.profile_case --unet-forward 3 [--n 64] [--batch 1]

Builds the seeded checkerboard problem (doma_gb300.problems.checkerboard) on
cuda:0, sets up group 0's source with one source iteration, then runs
`--sweeps` bare sweeps (or, with --solve, one full fixed-source solve) and
prints the solver's block shape and launch counts.  With --iteration
multigroup every group is in flight in each sweep launch.  Device memory stays
well under 1 GB at the default size.

With --unet-forward K it instead runs K forward passes of the learned
accelerator's U-Net (the committed weights) on an n^3 volume of `--batch`
samples, one per group of a correction, and prints their CUDA-event time.
"""
from __future__ import annotations

import argparse
import json
import os
import time


def main() -> None:
    ap = argparse.ArgumentParser()
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
    ap.add_argument("--batch", type=int, default=1)
    a = ap.parse_args()
    if a.unet_forward > 0:
        unet_forward(a)
        return
    if a.schedule == "levels":
        os.environ["DOMA_SWEEP_SCHEDULE"] = "levels"
    if a.loop == "host":
        os.environ["DOMA_SOLVE_LOOP"] = "host"

    import torch

    from . import problems as P
    from .solver import Solver

    torch.cuda.set_device(0)
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


def unet_forward(a) -> None:
    import torch

    from .learned.net import UNet

    torch.cuda.set_device(0)
    weights = os.path.join(os.path.dirname(__file__), "learned", "weights", "unet_c32.npz")
    with UNet(seed=0) as net:
        net.load(weights)
        net.set_stream(torch.cuda.current_stream().cuda_stream)
        g = torch.Generator(device="cuda").manual_seed(0)
        x = torch.randn((a.batch, a.n, a.n, a.n, 16), generator=g, device="cuda").to(torch.bfloat16)
        y = torch.empty((a.batch, a.n, a.n, a.n), dtype=torch.float32, device="cuda")
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(a.unet_forward):
            net.forward(x, y)
        e1.record()
        torch.cuda.synchronize()
        print(json.dumps({"workload": f"unet_forward_{a.n}cube_batch{a.batch}",
                          "forwards": a.unet_forward,
                          "ms_per_forward": e0.elapsed_time(e1) / a.unet_forward}))


if __name__ == "__main__":
    main()
