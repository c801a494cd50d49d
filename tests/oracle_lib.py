"""Test-side bindings of the CPU oracles (never imported by the product).

* liboracle.so   -- the project's C restatement of DOMA's fixed-source path
                    (oracle/doma_oracle.c), built by oracle/Makefile.
* libdoma_ref.so -- DOMA itself, compiled from its own sources with
                    oracle/ref_harness.cpp (only where the DOMA tree exists).
"""
from __future__ import annotations

import ctypes
import os
import re
import subprocess
from pathlib import Path

import numpy as np

from doma_gb300 import abi
from doma_gb300.problems import Problem

ROOT = Path(__file__).resolve().parents[1]
ORACLE_DIR = ROOT / "oracle"
ORACLE_LIB = ORACLE_DIR / "_build" / "liboracle.so"
REF_LIB = ORACLE_DIR / "_ref" / "libdoma_ref.so"

_dp = ctypes.POINTER(ctypes.c_double)
_u32p = ctypes.POINTER(ctypes.c_uint32)


def build_oracle() -> Path:
    if not ORACLE_LIB.exists():
        subprocess.run(["make", "-s", "-C", str(ORACLE_DIR), "oracle"], check=True)
    return ORACLE_LIB


_oracle = None
_ref = None


def oracle() -> ctypes.CDLL:
    global _oracle
    if _oracle is None:
        lib = ctypes.CDLL(str(build_oracle()))
        lib.oracle_quadrature.restype = ctypes.c_int
        lib.oracle_quadrature.argtypes = [ctypes.c_uint32] * 3 + [_dp] * 4 + [_u32p]
        lib.oracle_solve.restype = ctypes.c_int
        lib.oracle_solve.argtypes = [
            ctypes.POINTER(abi.DomaProblem), ctypes.POINTER(abi.DomaOptions), ctypes.c_uint32,
            _dp, _u32p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t), _u32p, _dp,
        ]
        lib.oracle_source_iterations.restype = ctypes.c_int
        lib.oracle_source_iterations.argtypes = [
            ctypes.POINTER(abi.DomaProblem), ctypes.POINTER(abi.DomaOptions), ctypes.c_uint32,
            ctypes.c_uint32, ctypes.c_uint32, _dp, _dp,
        ]
        lib.oracle_solve_eigen.restype = ctypes.c_int
        lib.oracle_solve_eigen.argtypes = [
            ctypes.POINTER(abi.DomaProblem), ctypes.POINTER(abi.DomaOptions), ctypes.c_double,
            ctypes.c_uint32, _dp, _dp, _u32p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t),
            _u32p, _dp, _dp,
        ]
        lib.oracle_solve_transient.restype = ctypes.c_int
        lib.oracle_solve_transient.argtypes = [
            ctypes.POINTER(abi.DomaProblem), ctypes.POINTER(abi.DomaOptions),
            ctypes.POINTER(abi.DomaTransient), ctypes.c_uint32, _dp, _dp, _u32p, _u32p,
            ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t),
        ]
        lib.oracle_set_single_thread_order.restype = None
        lib.oracle_set_single_thread_order.argtypes = [ctypes.c_int]
        lib.oracle_multigroup_solve.restype = ctypes.c_int
        lib.oracle_multigroup_solve.argtypes = [
            ctypes.POINTER(abi.DomaProblem), ctypes.POINTER(abi.DomaOptions), ctypes.c_uint32,
            _dp, _u32p, _dp,
        ]
        _oracle = lib
    return _oracle


def ref_available() -> bool:
    return REF_LIB.exists()


def ref() -> ctypes.CDLL:
    global _ref
    if _ref is None:
        lib = ctypes.CDLL(str(REF_LIB))
        lib.ref_solve.restype = ctypes.c_int
        lib.ref_solve.argtypes = [
            ctypes.POINTER(abi.DomaProblem), ctypes.POINTER(abi.DomaOptions), ctypes.c_uint32,
            _dp, ctypes.c_char_p, ctypes.c_size_t, ctypes.c_char_p,
        ]
        lib.ref_solve_eigen.restype = ctypes.c_int
        lib.ref_solve_eigen.argtypes = [
            ctypes.POINTER(abi.DomaProblem), ctypes.POINTER(abi.DomaOptions), ctypes.c_double,
            ctypes.c_uint32, ctypes.c_int, _dp, ctypes.c_char_p, ctypes.c_size_t,
        ]
        lib.ref_solve_transient.restype = ctypes.c_int
        lib.ref_solve_transient.argtypes = [
            ctypes.POINTER(abi.DomaProblem), ctypes.POINTER(abi.DomaOptions),
            ctypes.POINTER(abi.DomaTransient), ctypes.c_double, ctypes.c_uint32, _dp, _dp,
            ctypes.c_char_p, ctypes.c_size_t, ctypes.c_char_p,
        ]
        lib.ref_quadrature.restype = ctypes.c_int
        lib.ref_quadrature.argtypes = [ctypes.c_uint32] * 3 + [_dp] * 4 + [_u32p]
        _ref = lib
    return _ref


def _quad(fn, np_, na, dims):
    D = (8 if dims == 3 else 4) * np_ * na
    out = [np.zeros(D) for _ in range(4)]
    counts = np.zeros(8, dtype=np.uint32)
    n = fn(np_, na, dims, *[a.ctypes.data_as(_dp) for a in out], counts.ctypes.data_as(_u32p))
    if n != D:
        raise RuntimeError(f"quadrature returned {n}, expected {D}")
    return (*out, counts)


def oracle_quadrature(np_, na, dims):
    return _quad(oracle().oracle_quadrature, np_, na, dims)


def ref_quadrature(np_, na, dims):
    return _quad(ref().ref_quadrature, np_, na, dims)


def oracle_solve(p: Problem, opts: abi.DomaOptions, threads: int = 1, ordered: bool = False):
    """-> (phi[G][N], converged, si_counts, mg_iterations, mg_residual)

    ordered: sum in the one-thread order with any thread count (bit-equal to
    threads=1, which DOMA's single-thread results and the GPU's exact mode
    follow); otherwise threads > 1 sum as DOMA does with that many threads."""
    phi = np.zeros((p.num_groups, p.num_cells))
    cap = 1 << 16
    si = np.zeros(cap, dtype=np.uint32)
    n_si = ctypes.c_size_t(0)
    mg = ctypes.c_uint32(0)
    res = ctypes.c_double(0)
    cp = p.to_c()
    lib = oracle()
    lib.oracle_set_single_thread_order(1 if ordered else 0)
    try:
        rc = lib.oracle_solve(ctypes.byref(cp), ctypes.byref(opts), threads,
                              phi.ctypes.data_as(_dp), si.ctypes.data_as(_u32p), cap,
                              ctypes.byref(n_si), ctypes.byref(mg), ctypes.byref(res))
    finally:
        lib.oracle_set_single_thread_order(0)
    if rc < 0:
        raise ValueError("oracle rejected the problem")
    return phi, bool(rc), si[: min(n_si.value, cap)].copy(), int(mg.value), float(res.value)


def oracle_source_iterations(p: Problem, opts: abi.DomaOptions, group: int, count: int,
                             threads: int = 1):
    phi = np.zeros((p.num_groups, p.num_cells))
    res = np.zeros(max(count, 1))
    cp = p.to_c()
    rc = oracle().oracle_source_iterations(ctypes.byref(cp), ctypes.byref(opts), threads, group,
                                           count, phi.ctypes.data_as(_dp),
                                           res.ctypes.data_as(_dp))
    if rc < 0:
        raise ValueError("oracle rejected the problem")
    return phi, res[:count]


def oracle_multigroup_solve(p: Problem, opts: abi.DomaOptions, threads: int = 1):
    """-> (phi[G][N], converged, iterations, residual)"""
    phi = np.zeros((p.num_groups, p.num_cells))
    it = ctypes.c_uint32(0)
    res = ctypes.c_double(0)
    cp = p.to_c()
    rc = oracle().oracle_multigroup_solve(ctypes.byref(cp), ctypes.byref(opts), threads,
                                          phi.ctypes.data_as(_dp), ctypes.byref(it),
                                          ctypes.byref(res))
    if rc < 0:
        raise ValueError("oracle rejected the problem")
    return phi, bool(rc), int(it.value), float(res.value)


_SI_RE = re.compile(r"SI (?:converged|failed to converge) after (\d+) iterations")
_MG_RE = re.compile(r"MGI (?:converged|failed to converge) after (\d+) iterations")


def ref_solve(p: Problem, opts: abi.DomaOptions, threads: int = 1, out_base: str | None = None):
    """Run DOMA itself.  -> (phi[G][N], converged, si_counts, mg_iterations or None, log)"""
    phi = np.zeros((p.num_groups, p.num_cells))
    cap = 1 << 22
    buf = ctypes.create_string_buffer(cap)
    cp = p.to_c()
    rc = ref().ref_solve(ctypes.byref(cp), ctypes.byref(opts), threads, phi.ctypes.data_as(_dp),
                         buf, cap, out_base.encode() if out_base else None)
    log = buf.value.decode()
    si = np.array([int(m) for m in _SI_RE.findall(log)], dtype=np.uint32)
    mg = _MG_RE.findall(log)
    return phi, bool(rc), si, (int(mg[-1]) if mg else None), log


def oracle_solve_eigen(p: Problem, opts: abi.DomaOptions, k_tol: float, threads: int = 1):
    """-> (phi[G][N], k, converged, si_counts, pi_iterations, shape_residual, k_residual)"""
    phi = np.zeros((p.num_groups, p.num_cells))
    k = ctypes.c_double(0)
    cap = 1 << 16
    si = np.zeros(cap, dtype=np.uint32)
    n_si = ctypes.c_size_t(0)
    pi = ctypes.c_uint32(0)
    shape = ctypes.c_double(0)
    kres = ctypes.c_double(0)
    cp = p.to_c()
    rc = oracle().oracle_solve_eigen(ctypes.byref(cp), ctypes.byref(opts), k_tol, threads,
                                     phi.ctypes.data_as(_dp), ctypes.byref(k),
                                     si.ctypes.data_as(_u32p), cap, ctypes.byref(n_si),
                                     ctypes.byref(pi), ctypes.byref(shape), ctypes.byref(kres))
    if rc < 0:
        raise ValueError("oracle rejected the problem")
    return (phi, float(k.value), bool(rc), si[: min(n_si.value, cap)].copy(), int(pi.value),
            float(shape.value), float(kres.value))


_PI_RE = re.compile(r"PI (?:converged|failed to converge) after (\d+) iterations")
_K_RE = re.compile(r"Converged value of k = (\S+)")


def ref_solve_eigen(p: Problem, opts: abi.DomaOptions, k_tol: float, threads: int = 1,
                    precision: int = 0):
    """Run DOMA's solveEigenvalue.  -> (phi[G][N], converged, si_counts, pi_iterations or
    None, k or None, log).  With precision=17 the printed k is exact."""
    phi = np.zeros((p.num_groups, p.num_cells))
    cap = 1 << 22
    buf = ctypes.create_string_buffer(cap)
    cp = p.to_c()
    rc = ref().ref_solve_eigen(ctypes.byref(cp), ctypes.byref(opts), k_tol, threads, precision,
                               phi.ctypes.data_as(_dp), buf, cap)
    log = buf.value.decode()
    si = np.array([int(m) for m in _SI_RE.findall(log)], dtype=np.uint32)
    pi = _PI_RE.findall(log)
    k = _K_RE.findall(log)
    return (phi, bool(rc), si, (int(pi[-1]) if pi else None), (float(k[-1]) if k else None), log)


def oracle_solve_transient(p: Problem, tr, opts: abi.DomaOptions, threads: int = 1):
    """-> (phi_steps[S][G][N], dnps[D][N], converged, steps_done, si_counts)"""
    S, G, N, D = tr.num_steps, p.num_groups, p.num_cells, tr.num_d_groups
    phis = np.zeros((S, G, N))
    dnps = np.zeros((max(D, 1), N))
    done = ctypes.c_uint32(0)
    cap = 1 << 16
    si = np.zeros(cap, dtype=np.uint32)
    n_si = ctypes.c_size_t(0)
    cp, ct = p.to_c(), tr.to_c()
    rc = oracle().oracle_solve_transient(ctypes.byref(cp), ctypes.byref(opts), ctypes.byref(ct),
                                         threads, phis.ctypes.data_as(_dp),
                                         dnps.ctypes.data_as(_dp), ctypes.byref(done),
                                         si.ctypes.data_as(_u32p), cap, ctypes.byref(n_si))
    if rc < 0:
        raise ValueError("oracle rejected the problem")
    return phis, dnps[:D], bool(rc), int(done.value), si[: min(n_si.value, cap)].copy()


def ref_solve_transient(p: Problem, tr, opts: abi.DomaOptions, threads: int = 1,
                        out_base: str | None = None):
    """Run DOMA's solveTransient (zero initial condition).  -> (phi[G][N] of the
    last step, dnps[D][N], converged, si_counts, log).  Without out_base the
    reference's per-step text files go to a temporary directory."""
    import tempfile
    G, N, D = p.num_groups, p.num_cells, tr.num_d_groups
    phi = np.zeros((G, N))
    dnps = np.zeros((max(D, 1), N))
    cap = 1 << 22
    buf = ctypes.create_string_buffer(cap)
    cp, ct = p.to_c(), tr.to_c()
    with tempfile.TemporaryDirectory() as tmp:
        base = out_base or os.path.join(tmp, "ref")
        rc = ref().ref_solve_transient(ctypes.byref(cp), ctypes.byref(opts), ctypes.byref(ct),
                                       tr.t1, threads, phi.ctypes.data_as(_dp),
                                       dnps.ctypes.data_as(_dp), buf, cap, base.encode())
    log = buf.value.decode()
    si = np.array([int(m) for m in _SI_RE.findall(log)], dtype=np.uint32)
    return phi, dnps[:D], bool(rc), si, log
