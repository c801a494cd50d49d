"""Time to a target error: plain multigroup source iteration against the same
iteration with learned corrections, both stopped on the relative L2 error of
the scalar flux against an FP64 solution of the same problem."""
from __future__ import annotations

import numpy as np

from .. import problems as P
from ..solver import Solver


def reference_flux(p: P.Problem, tol: float = 1e-11, max_it: int = 100000) -> tuple[np.ndarray, dict]:
    """FP64 multigroup solve (plain source iteration, DD) to a tight increment tolerance."""
    with Solver(p, P.make_options(scheme="dd", precision="fp64", fs_tol=tol, fs_max_it=max_it,
                                  iteration="multigroup")) as s:
        rep = s.solve_fixed_source()
        if not rep.converged:
            raise RuntimeError(f"FP64 reference of {p.name} did not converge")
        return s.scalar_flux(), {"iterations": rep.mg_iterations, "ms": rep.solve_ms}


def time_to_error(p: P.Problem, ref: np.ndarray, target: float = 1e-5, net=None,
                  first: int = 3, interval: int = 3, max_corrections: int = 32,
                  guard: bool = True, max_it: int = 100000, warm: bool = True) -> dict:
    """FP32 multigroup DD solve stopped at relative L2 error <= target.
    A first, untimed solve warms the network's workspace and the kernels."""
    opts = P.make_options(scheme="dd", precision="fp32", fs_tol=0.0, fs_max_it=max_it,
                          iteration="multigroup")
    with Solver(p, opts) as s:
        s.set_reference(ref, target)
        if net is not None:
            s.set_accelerator(net, first=first, interval=interval,
                              max_corrections=max_corrections, guard=guard)
        if warm:
            s.solve_fixed_source()
        rep = s.solve_fixed_source()
        st = s.accel_stats()
        phi = s.scalar_flux()
    err = float(np.linalg.norm(phi - ref) / np.linalg.norm(ref))
    return {"ms": rep.solve_ms, "iterations": rep.mg_iterations, "converged": rep.converged,
            "accepted": st["accepted"], "rejected": st["rejected"], "error": err,
            "reported_error": st["error"], "updates": rep.updates}


def time_to_error_gs(p: P.Problem, ref: np.ndarray, target: float = 1e-5,
                     tolerances=(1e-4, 3e-5, 1e-5, 3e-6, 1e-6, 3e-7), max_it: int = 100000) -> dict:
    """DOMA's own iteration order in FP32: Gauss-Seidel over groups wrapping
    within-group source iteration, stopped by its increment tolerance
    (fs_tol = mg_tol).  It has no error-based stop, so the tolerances are
    tried from loose to tight and the first solve whose relative L2 error
    against ref is <= target gives the time (each solve warm, timed on the
    device).  Returns the tried solves as well."""
    tried = []
    for tol in tolerances:
        opts = P.make_options(scheme="dd", precision="fp32", fs_tol=tol, fs_max_it=max_it,
                              mg_tol=tol, mg_max_it=max_it)
        with Solver(p, opts) as s:
            s.solve_fixed_source()
            rep = s.solve_fixed_source()
            phi = s.scalar_flux()
        err = float(np.linalg.norm(phi - ref) / np.linalg.norm(ref))
        tried.append({"tolerance": tol, "ms": rep.solve_ms, "sweeps": rep.si_iterations,
                      "mg_iterations": rep.mg_iterations, "error": err,
                      "converged": rep.converged})
        if err <= target:
            return {"ms": rep.solve_ms, "tolerance": tol, "error": err,
                    "sweeps": rep.si_iterations, "tried": tried}
    return {"ms": None, "tolerance": None, "error": tried[-1]["error"], "tried": tried}
