"""Pin the CPU restatement (oracle/doma_oracle.c) to DOMA itself.

The golden fixtures were produced by running DOMA's own solver on seeded
synthetic problems (tests/golden/make_golden.py).  The restatement must
reproduce them bit for bit: scalar flux, return value and every
source-iteration count.
"""
import numpy as np
import pytest

import oracle_lib as ol
from doma_gb300 import problems as P
from golden_cases import (case_names, eigen_case_names, load_case, load_eigen_case,
                          load_transient_case, quadrature_sets, transient_case_names)


@pytest.mark.parametrize("dims,np_,na,mu,eta,xi,w,counts", quadrature_sets())
def test_quadrature_matches_reference(dims, np_, na, mu, eta, xi, w, counts):
    m, e, x, ww, c = ol.oracle_quadrature(np_, na, dims)
    assert np.array_equal(c, counts)
    for a, b in ((m, mu), (e, eta), (x, xi), (ww, w)):
        assert np.array_equal(a, b)
    assert abs(w.sum() - (4 * np.pi if dims == 3 else 2 * np.pi)) < 1e-12


@pytest.mark.parametrize("name", case_names())
def test_oracle_bitwise_equals_reference(name):
    p, opts, exp = load_case(name)
    phi, ok, si, mg, _ = ol.oracle_solve(p, opts, threads=1)
    assert ok == exp["converged"]
    assert list(si) == list(exp["si_counts"])
    if exp["mg_iterations"] is not None:
        assert mg == exp["mg_iterations"]
    assert np.array_equal(phi, exp["phi"]), np.abs(phi - exp["phi"]).max()


def test_oracle_threads_agree():
    """The OpenMP split over ordinates changes only the summation order."""
    p, opts, exp = load_case("small_cube_twdd")
    phi, ok, si, _, _ = ol.oracle_solve(p, opts, threads=3)
    assert ok and list(si) == list(exp["si_counts"])
    rel = np.abs(phi - exp["phi"]).max() / np.abs(exp["phi"]).max()
    assert rel < 1e-13


@pytest.mark.parametrize("scheme", ["dd", "tw_dd"])
@pytest.mark.parametrize("dims", [2, 3])
def test_oracle_single_thread_order_with_threads(scheme, dims):
    """Ordinates in parallel, sums in the one-thread order: the same bits as a
    single-thread run (and therefore as DOMA's single-thread run)."""
    p = P.random_problem(41, dims, 9, 8, 6, groups=3, np_=3, na=2, materials=4, fission=True)
    opts = P.make_options(scheme=scheme, theta=0.8, fs_tol=1e-9, mg_tol=1e-9)
    a, ok_a, si_a, mg_a, _ = ol.oracle_solve(p, opts, threads=1)
    b, ok_b, si_b, mg_b, _ = ol.oracle_solve(p, opts, threads=4, ordered=True)
    assert np.array_equal(a, b)
    assert (ok_a, list(si_a), mg_a) == (ok_b, list(si_b), mg_b)


def test_oracle_rejects_bad_input():
    from doma_gb300 import problems as P
    p = P.random_problem(0, 3, 3, 3, 3, groups=2)
    p.cell_material[0] = 99
    with pytest.raises(ValueError):
        ol.oracle_solve(p, P.make_options())


@pytest.mark.parametrize("name", eigen_case_names())
def test_oracle_eigenvalue_bitwise_equals_reference(name):
    """k-eigenvalue power iteration: flux, k, power-iteration and SI counts
    exactly as DOMA's solveEigenvalue produced them."""
    p, opts, k_tol, exp = load_eigen_case(name)
    phi, k, ok, si, pi, _, _ = ol.oracle_solve_eigen(p, opts, k_tol, threads=1)
    assert ok == exp["converged"]
    assert pi == exp["pi_iterations"]
    assert list(si) == list(exp["si_counts"])
    if exp["k_is_final"]:
        assert k == exp["k"]
    assert np.array_equal(phi, exp["phi"]), np.abs(phi - exp["phi"]).max()


@pytest.mark.parametrize("name", transient_case_names())
def test_oracle_transient_bitwise_equals_reference(name):
    """Transient from a zero initial condition: every step's flux, the
    precursors and the SI counts exactly as DOMA's solveTransient produced
    them, including a solve that fails part-way."""
    p, tr, opts, exp = load_transient_case(name)
    phis, dnps, ok, done, si = ol.oracle_solve_transient(p, tr, opts, threads=1)
    assert ok == exp["converged"]
    assert done == exp["steps_done"]
    assert list(si) == list(exp["si_counts"])
    n = len(exp["phi_steps"])
    assert np.array_equal(phis[:n], exp["phi_steps"])
    assert np.array_equal(dnps, exp["dnps"])


def test_oracle_transient_threads_agree():
    """Threads only split cells: the parallel oracle matches the serial one."""
    p, tr, opts, exp = load_transient_case("transient3d_twdd")
    a = ol.oracle_solve_transient(p, tr, opts, threads=1)
    b = ol.oracle_solve_transient(p, tr, opts, threads=4)
    assert np.abs(a[0] - b[0]).max() <= 1e-12 * np.abs(a[0]).max()
    assert a[2] == b[2] and a[3] == b[3]


def test_oracle_transient_rejects_bad_input():
    from doma_gb300 import problems as P
    p, tr = P.transient_problem(0, num_steps=2)
    import dataclasses
    bad = dataclasses.replace(tr, t1=0.0)
    with pytest.raises(ValueError):
        ol.oracle_solve_transient(p, bad, P.make_options())
