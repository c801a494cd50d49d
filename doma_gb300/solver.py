"""Python host interface of the GB300 fixed-source solver (binds the C ABI).

Mirrors DOMA's solver interface for this path: a solver is built from a
problem and options (TransportSolver3D<T>(mesh, params, verbose, threads),
src/TransportSolver3D.cpp:5-27) and ``solve_fixed_source()`` runs the
Gauss-Seidel / source-iteration solve (TransportSolver3D::solveFixedSource,
src/TransportSolver3D.cpp:262-316).  As in DOMA, non-convergence is a
``False`` result, not an exception; invalid input and CUDA failures raise.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import abi
from .problems import Problem, make_options


@dataclass
class Report:
    converged: bool
    status: int
    mg_iterations: int
    si_iterations: int
    updates: int
    kernel_launches: int
    mg_residual: float
    si_residual: float
    solve_ms: float
    si_counts: np.ndarray


class Solver:
    """One problem resident on the current CUDA device."""

    def __init__(self, problem: Problem, options: abi.DomaOptions | None = None, **kw):
        self.lib = abi.load_library()
        self.problem = problem
        self.options = options if options is not None else make_options(**kw)
        self._cp = problem.to_c()
        h = ctypes.c_void_p()
        st = self.lib.doma_solver_create(ctypes.byref(self._cp), ctypes.byref(self.options),
                                         ctypes.byref(h))
        abi.check(st, "doma_solver_create", self.lib)
        self._h = h

    # -- lifecycle ----------------------------------------------------------
    def close(self) -> None:
        if getattr(self, "_h", None):
            self.lib.doma_solver_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- calls --------------------------------------------------------------
    def set_stream(self, stream_ptr: int | None) -> None:
        abi.check(self.lib.doma_solver_set_stream(self._h, ctypes.c_void_p(stream_ptr or 0)),
                  "doma_solver_set_stream", self.lib)

    def solve_fixed_source(self, si_capacity: int = 1 << 16) -> Report:
        counts = np.zeros(si_capacity, dtype=np.uint32)
        rep = abi.DomaReport()
        rep.si_counts = counts.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))
        rep.si_counts_capacity = si_capacity
        st = self.lib.doma_solver_solve_fixed_source(self._h, ctypes.byref(rep))
        abi.check(st, "doma_solver_solve_fixed_source", self.lib,
                  allow=(abi.DOMA_OK, abi.DOMA_NOT_CONVERGED))
        n = min(rep.si_counts_len, si_capacity)
        return Report(converged=st == abi.DOMA_OK, status=st, mg_iterations=rep.mg_iterations,
                      si_iterations=rep.si_iterations, updates=rep.updates,
                      kernel_launches=rep.kernel_launches, mg_residual=rep.mg_residual,
                      si_residual=rep.si_residual, solve_ms=rep.solve_ms,
                      si_counts=counts[:n].copy())

    def solve_eigenvalue(self, k_tol: float = 1e-5, si_capacity: int = 1 << 16) -> tuple[Report, float]:
        """k-eigenvalue power iteration (DOMA's solveEigenvalue) -> (report, k).
        report.mg_iterations counts power iterations."""
        counts = np.zeros(si_capacity, dtype=np.uint32)
        rep = abi.DomaReport()
        rep.si_counts = counts.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))
        rep.si_counts_capacity = si_capacity
        k = ctypes.c_double(0.0)
        st = self.lib.doma_solver_solve_eigenvalue(self._h, k_tol, ctypes.byref(rep), ctypes.byref(k))
        abi.check(st, "doma_solver_solve_eigenvalue", self.lib,
                  allow=(abi.DOMA_OK, abi.DOMA_NOT_CONVERGED))
        n = min(rep.si_counts_len, si_capacity)
        return (Report(converged=st == abi.DOMA_OK, status=st, mg_iterations=rep.mg_iterations,
                       si_iterations=rep.si_iterations, updates=rep.updates,
                       kernel_launches=rep.kernel_launches, mg_residual=rep.mg_residual,
                       si_residual=rep.si_residual, solve_ms=rep.solve_ms,
                       si_counts=counts[:n].copy()), float(k.value))

    def solve_transient(self, transient, on_step=None, si_capacity: int = 1 << 16) -> Report:
        """Transient solve from a zero initial condition (DOMA's solveTransient).
        transient: problems.Transient.  on_step(step, t, phi[G][N], dnps[D][N])
        is called after each step with copies of that step's flux and
        precursors; a truthy return stops the solve.  -> report (si_counts over
        every step; mg_iterations of the last step)."""
        p = self.problem
        G, N, D = p.num_groups, p.num_cells, transient.num_d_groups
        counts = np.zeros(si_capacity, dtype=np.uint32)
        rep = abi.DomaReport()
        rep.si_counts = counts.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))
        rep.si_counts_capacity = si_capacity
        ct = transient.to_c()
        errors = []

        def _cb(user, step, t, phi, dnps):
            if on_step is None:
                return 0
            try:
                f = np.ctypeslib.as_array(phi, shape=(G * N,)).reshape(G, N).copy()
                d = (np.ctypeslib.as_array(dnps, shape=(D * N,)).reshape(D, N).copy()
                     if D else np.zeros((0, N)))
                return 1 if on_step(int(step), float(t), f, d) else 0
            except Exception as e:  # surfaced after the call returns
                errors.append(e)
                return 1

        cb = abi.StepCallback(_cb)
        st = self.lib.doma_solver_solve_transient(self._h, ctypes.byref(ct), cb, None,
                                                  ctypes.byref(rep))
        if errors:
            raise errors[0]
        abi.check(st, "doma_solver_solve_transient", self.lib,
                  allow=(abi.DOMA_OK, abi.DOMA_NOT_CONVERGED))
        n = min(rep.si_counts_len, si_capacity)
        return Report(converged=st == abi.DOMA_OK, status=st, mg_iterations=rep.mg_iterations,
                      si_iterations=rep.si_iterations, updates=rep.updates,
                      kernel_launches=rep.kernel_launches, mg_residual=rep.mg_residual,
                      si_residual=rep.si_residual, solve_ms=rep.solve_ms,
                      si_counts=counts[:n].copy())

    def scalar_flux(self) -> np.ndarray:
        p = self.problem
        out = np.empty((p.num_groups, p.num_cells), dtype=np.float64)
        abi.check(self.lib.doma_solver_get_scalar_flux(
            self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), out.size),
            "doma_solver_get_scalar_flux", self.lib)
        return out

    def source_iterations(self, group: int, count: int) -> None:
        abi.check(self.lib.doma_solver_source_iterations(self._h, group, count),
                  "doma_solver_source_iterations", self.lib)

    def sweeps(self, group: int, count: int) -> None:
        abi.check(self.lib.doma_solver_sweeps(self._h, group, count), "doma_solver_sweeps",
                  self.lib)

    def set_accelerator(self, net, first: int = 3, interval: int = 3, max_corrections: int = 32,
                        guard: bool = True) -> None:
        """Learned corrections (net: doma_gb300.learned.net.UNet, or None to detach)."""
        o = abi.DomaAccelOptions(first=first, interval=interval, max_corrections=max_corrections,
                                 guard=1 if guard else 0)
        self._net = net
        abi.check(self.lib.doma_solver_set_accelerator(self._h, net.handle if net else None,
                                                       ctypes.byref(o)),
                  "doma_solver_set_accelerator", self.lib)

    def set_reference(self, phi_ref: np.ndarray | None, target: float = 1e-5) -> None:
        """Stop on relative L2 error <= target against phi_ref ([G][N])."""
        if phi_ref is None:
            abi.check(self.lib.doma_solver_set_reference(self._h, None, 0, 0.0),
                      "doma_solver_set_reference", self.lib)
            return
        ref = np.ascontiguousarray(phi_ref, dtype=np.float64).reshape(-1)
        abi.check(self.lib.doma_solver_set_reference(
            self._h, ref.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), ref.size, target),
            "doma_solver_set_reference", self.lib)

    def accel_stats(self) -> dict:
        st = abi.DomaAccelStats()
        abi.check(self.lib.doma_solver_accel_stats(self._h, ctypes.byref(st)),
                  "doma_solver_accel_stats", self.lib)
        return {"iterations": st.iterations, "accepted": st.corrections_accepted,
                "rejected": st.corrections_rejected, "error": st.error, "solve_ms": st.solve_ms}

    def describe(self) -> dict:
        tile = (ctypes.c_uint32 * 3)()
        lps = ctypes.c_uint32()
        launches = ctypes.c_uint64()
        abi.check(self.lib.doma_solver_describe(self._h, tile, ctypes.byref(lps),
                                                ctypes.byref(launches)),
                  "doma_solver_describe", self.lib)
        return {"tile": tuple(tile), "launches_per_sweep": lps.value,
                "kernel_launches": launches.value}


class Batch:
    """Many independent problems solved together (doma_batch_*): every group of
    every unconverged problem is swept in one persistent launch per iteration.
    Multigroup iteration in FP32 with FP64 norms; problems share dims/scheme."""

    def __init__(self, problems: list[Problem], options: abi.DomaOptions | None = None, **kw):
        self.lib = abi.load_library()
        self.problems = list(problems)
        kw.setdefault("precision", "fp32")
        kw.setdefault("iteration", "multigroup")
        self.options = options if options is not None else make_options(**kw)
        self._cps = (abi.DomaProblem * len(self.problems))(*[p.to_c() for p in self.problems])
        h = ctypes.c_void_p()
        st = self.lib.doma_batch_create(self._cps, len(self.problems), ctypes.byref(self.options),
                                        ctypes.byref(h))
        abi.check(st, "doma_batch_create", self.lib)
        self._h = h

    def close(self) -> None:
        if getattr(self, "_h", None):
            self.lib.doma_batch_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream_ptr: int | None) -> None:
        abi.check(self.lib.doma_batch_set_stream(self._h, ctypes.c_void_p(stream_ptr or 0)),
                  "doma_batch_set_stream", self.lib)

    def tune(self) -> int:
        """Per-class block lengths (see doma_batch_tune); returns the most common."""
        tx = ctypes.c_uint32(0)
        abi.check(self.lib.doma_batch_tune(self._h, ctypes.byref(tx)), "doma_batch_tune", self.lib)
        return tx.value

    def tiles(self) -> list[int]:
        out = (ctypes.c_uint32 * len(self.problems))()
        abi.check(self.lib.doma_batch_tiles(self._h, out, len(self.problems)), "doma_batch_tiles",
                  self.lib)
        return list(out)

    def tune_report(self) -> dict:
        u = (ctypes.c_float * 3)()
        m = ctypes.c_float()
        c = ctypes.c_uint32()
        abi.check(self.lib.doma_batch_tune_report(self._h, u, ctypes.byref(m), ctypes.byref(c)),
                  "doma_batch_tune_report", self.lib)
        return {"uniform_ms": {8: u[0], 16: u[1], 32: u[2]}, "per_class_ms": m.value,
                "classes": c.value}

    def solve(self) -> list[Report]:
        n = len(self.problems)
        reps = (abi.DomaReport * n)()
        st = self.lib.doma_batch_solve(self._h, reps, n)
        abi.check(st, "doma_batch_solve", self.lib, allow=(abi.DOMA_OK, abi.DOMA_NOT_CONVERGED))
        return [Report(converged=r.status == abi.DOMA_OK, status=r.status,
                       mg_iterations=r.mg_iterations, si_iterations=r.si_iterations,
                       updates=r.updates, kernel_launches=r.kernel_launches,
                       mg_residual=r.mg_residual, si_residual=r.si_residual, solve_ms=r.solve_ms,
                       si_counts=np.array([r.mg_iterations], dtype=np.uint32)) for r in reps]

    def begin(self) -> None:
        abi.check(self.lib.doma_batch_begin(self._h), "doma_batch_begin", self.lib)

    def iterate(self, iterations: int) -> int:
        """Run up to `iterations` batched iterations; returns problems still active."""
        active = ctypes.c_uint32()
        abi.check(self.lib.doma_batch_iterate(self._h, iterations, ctypes.byref(active)),
                  "doma_batch_iterate", self.lib)
        return active.value

    def state_pointers(self, index: int) -> tuple[int, int]:
        """Device addresses of problem `index`'s flux and last increment ([G][N] doubles)."""
        phi, inc = ctypes.c_void_p(), ctypes.c_void_p()
        abi.check(self.lib.doma_batch_state(self._h, index, ctypes.byref(phi), ctypes.byref(inc)),
                  "doma_batch_state", self.lib)
        return phi.value, inc.value

    def set_increment(self, index: int, ptr: int) -> None:
        """Sweep the device field at `ptr` ([G][N] doubles) in the next iteration."""
        abi.check(self.lib.doma_batch_set_increment(self._h, index, ctypes.c_void_p(ptr)),
                  "doma_batch_set_increment", self.lib)

    def reports(self) -> list[Report]:
        n = len(self.problems)
        reps = (abi.DomaReport * n)()
        st = self.lib.doma_batch_reports(self._h, reps, n)
        abi.check(st, "doma_batch_reports", self.lib, allow=(abi.DOMA_OK, abi.DOMA_NOT_CONVERGED))
        return [Report(converged=r.status == abi.DOMA_OK, status=r.status,
                       mg_iterations=r.mg_iterations, si_iterations=r.si_iterations,
                       updates=r.updates, kernel_launches=r.kernel_launches,
                       mg_residual=r.mg_residual, si_residual=r.si_residual, solve_ms=r.solve_ms,
                       si_counts=np.array([r.mg_iterations], dtype=np.uint32)) for r in reps]

    def scalar_flux(self, index: int) -> np.ndarray:
        p = self.problems[index]
        out = np.empty((p.num_groups, p.num_cells), dtype=np.float64)
        abi.check(self.lib.doma_batch_get_scalar_flux(
            self._h, index, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), out.size),
            "doma_batch_get_scalar_flux", self.lib)
        return out


def quadrature(num_polar: int, num_azimuthal: int, dims: int = 3):
    """(mu, eta, xi, w, counts) from the library's host quadrature (no GPU needed)."""
    lib = abi.load_library()
    D = (8 if dims == 3 else 4) * num_polar * num_azimuthal
    arrs = [np.zeros(D) for _ in range(4)]
    counts = np.zeros(8, dtype=np.uint32)
    dp = ctypes.POINTER(ctypes.c_double)
    abi.check(lib.doma_quadrature(num_polar, num_azimuthal, dims,
                                  *[a.ctypes.data_as(dp) for a in arrs],
                                  counts.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))),
              "doma_quadrature", lib)
    return (*arrs, counts)


def solve(problem: Problem, **kw):
    """Convenience: build, solve, read back.  -> (phi [G][N], Report)"""
    with Solver(problem, **kw) as s:
        rep = s.solve_fixed_source()
        return s.scalar_flux(), rep
