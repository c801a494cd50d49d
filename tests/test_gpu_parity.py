"""Parity of the GPU library (called through the C ABI) with DOMA.

* FP64 drop-in mode against DOMA's own results (the golden fixtures, made by
  running DOMA) and against the CPU oracle on fresh seeded problems: same
  return value, same source-iteration count for every (MG iteration, group),
  scalar flux within 1e-12 relative L-infinity (and, in practice, bit-equal).
* FP32 sweep mode against the same references: relative L2 error <= 1e-5.
* Determinism, block-shape independence and the failure paths.
"""
import numpy as np
import pytest

import oracle_lib as ol
from doma_gb300 import problems as P
from doma_gb300.solver import Solver, quadrature
from golden_cases import (case_names, eigen_case_names, load_case, load_eigen_case,
                          load_transient_case, quadrature_sets, transient_case_names)

pytestmark = pytest.mark.gpu

FP64_RTOL = 1e-12   # relative L-infinity, FP64 drop-in mode
FP32_RTOL = 1e-5    # relative L2, FP32 sweep vs FP64


def rel_linf(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def run(p, opts):
    with Solver(p, opts) as s:
        rep = s.solve_fixed_source()
        return s.scalar_flux(), rep


@pytest.mark.parametrize("dims,np_,na,mu,eta,xi,w,counts", quadrature_sets())
def test_quadrature_bitwise_on_this_host(dims, np_, na, mu, eta, xi, w, counts):
    m, e, x, ww, c = quadrature(np_, na, dims)
    assert np.array_equal(c, counts)
    for a, b in ((m, mu), (e, eta), (x, xi), (ww, w)):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("name", case_names())
def test_fp64_matches_reference_golden(name):
    p, opts, exp = load_case(name)
    phi, rep = run(p, opts)
    assert rep.converged == exp["converged"]
    assert list(rep.si_counts) == list(exp["si_counts"])
    if exp["mg_iterations"] is not None:
        assert rep.mg_iterations == exp["mg_iterations"]
    assert rel_linf(phi, exp["phi"]) <= FP64_RTOL


def test_fp64_bit_equal_to_reference_golden():
    """Stronger than the contract: with matching iteration counts, the
    exact-order FP64 path reproduces DOMA's scalar flux bit for bit."""
    unequal = []
    for name in case_names():
        p, opts, exp = load_case(name)
        phi, rep = run(p, opts)
        if not np.array_equal(phi, exp["phi"]):
            unequal.append((name, rel_linf(phi, exp["phi"])))
    assert not unequal, unequal


@pytest.mark.parametrize("seed", [21, 22, 23])
@pytest.mark.parametrize("scheme", ["dd", "tw_dd"])
@pytest.mark.parametrize("dims", [2, 3])
def test_fp64_matches_oracle_random(seed, scheme, dims):
    p = P.random_problem(seed, dims, 9, 7, 6, groups=3, np_=2, na=3, materials=4,
                         fission=seed % 2 == 1)
    opts = P.make_options(scheme=scheme, theta=0.8, fs_tol=1e-10, mg_tol=1e-10)
    phi, rep = run(p, opts)
    o_phi, ok, si, mg, _ = ol.oracle_solve(p, opts)
    assert rep.converged == ok
    assert list(rep.si_counts) == list(si)
    assert rep.mg_iterations == mg
    assert rel_linf(phi, o_phi) <= FP64_RTOL


@pytest.mark.parametrize("tile", [(8, 0, 0), (16, 0, 0), (32, 0, 0)])
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("dims", [2, 3])
@pytest.mark.parametrize("scheme", ["tw_dd", "dd"])
def test_block_shape_does_not_change_results(tile, precision, dims, scheme):
    """Every block length, with ragged edge blocks in every axis and a
    partial ordinate group (9 ordinates per octant: in FP32 a full group of 8
    and a partial one, in FP64 one partial group of 16), gives the same bits."""
    p = P.random_problem(31, dims, 37, 19, 7, groups=2, np_=3, na=3, materials=3)
    base = P.make_options(scheme=scheme, precision=precision, fs_tol=1e-9, mg_tol=1e-9)
    ref_phi, _ = run(p, base)
    opts = P.make_options(scheme=scheme, precision=precision, fs_tol=1e-9, mg_tol=1e-9,
                          tile=tile)
    phi, _ = run(p, opts)
    assert np.array_equal(phi, ref_phi)


@pytest.mark.parametrize("scheme", ["dd", "tw_dd"])
@pytest.mark.parametrize("dims", [2, 3])
def test_both_register_bodies_give_the_same_bits(monkeypatch, dims, scheme):
    """Each FP32 scheme is compiled twice, for fewer and for more CTAs per SM
    (DD 8 and 12, TW-DD 5 and 6); the solver picks one by the tasks a
    wavefront level holds.  Both run the same arithmetic, so a solve gives the
    same bits and counts."""
    p = P.random_problem(17, dims, 21, 12, 8, groups=2, np_=3, na=3, materials=3)
    opts = P.make_options(scheme=scheme, precision="fp32", fs_tol=1e-6, mg_tol=1e-6)
    out = []
    for many in ("0", "1"):
        monkeypatch.setenv("DOMA_SWEEP_MANY", many)
        out.append(run(p, opts))
    (phi0, rep0), (phi1, rep1) = out
    assert list(rep0.si_counts) == list(rep1.si_counts)
    assert np.array_equal(phi0, phi1)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_deterministic(precision):
    p = P.small_cube(3, n=14)
    opts = P.make_options(scheme="tw_dd", precision=precision)
    a, ra = run(p, opts)
    b, rb = run(p, opts)
    assert np.array_equal(a, b) and list(ra.si_counts) == list(rb.si_counts)


@pytest.mark.parametrize("name", [n for n in case_names() if not n.startswith("capped")])
def test_fp32_error_against_reference(name):
    """FP32 sweeps recompute each group's flux from zero at every Gauss-Seidel
    iteration, so the Gauss-Seidel residual cannot fall much below the FP32
    rounding of the flux (~1e-7): FP32 solves run at tolerances >= 1e-6."""
    p, opts, exp = load_case(name)
    opts.precision = 1
    opts.fs_tol = max(opts.fs_tol, 1e-6)
    opts.mg_tol = max(opts.mg_tol, 1e-6)
    phi, rep = run(p, opts)
    assert rep.converged
    assert rel_l2(phi, exp["phi"]) <= FP32_RTOL, rel_l2(phi, exp["phi"])


def test_2d_twdd_keeps_bare_xi_term():
    """DOMA's 2D TW-DD b weight carries a bare |xi| term; removing it would
    change the answer, so matching the oracle pins it."""
    p = P.square_2d(4, n=12, groups=1)
    opts = P.make_options(scheme="tw_dd", theta=0.9)
    phi, _ = run(p, opts)
    o_phi, *_ = ol.oracle_solve(p, opts)
    assert rel_linf(phi, o_phi) <= FP64_RTOL


def test_not_converged_keeps_last_iterate():
    p, opts, exp = load_case("capped_si_twdd")
    phi, rep = run(p, opts)
    assert not rep.converged and rep.status == 1
    assert np.array_equal(phi, exp["phi"])


def test_source_iterations_match_oracle():
    p = P.checkerboard(0, n=16, groups=4, np_=2, na=2, block=4)
    opts = P.make_options(scheme="tw_dd", theta=0.7)
    with Solver(p, opts) as s:
        s.source_iterations(0, 5)
        phi = s.scalar_flux()
    o_phi, _ = ol.oracle_source_iterations(p, opts, 0, 5)
    assert rel_linf(phi, o_phi) <= FP64_RTOL


def test_empty_source_gives_zero_flux():
    p = P.random_problem(2, 3, 4, 4, 4, groups=2)
    p.source[:] = 0.0
    phi, rep = run(p, P.make_options())
    assert rep.converged and not phi.any()


def test_single_cell_and_single_ordinate():
    p = P.random_problem(9, 3, 1, 1, 1, groups=1, np_=1, na=1, materials=1)
    opts = P.make_options(scheme="tw_dd")
    phi, rep = run(p, opts)
    o_phi, ok, si, _, _ = ol.oracle_solve(p, opts)
    assert list(rep.si_counts) == list(si)
    assert rel_linf(phi, o_phi) <= FP64_RTOL


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("dims", [2, 3])
def test_persistent_and_level_schedules_agree(monkeypatch, precision, dims):
    """The dataflow sweep and the one-launch-per-level sweep run the same task
    body; their results must be bit-identical."""
    p = P.random_problem(41, dims, 13, 11, 9, groups=2, np_=2, na=3, materials=3)
    opts = P.make_options(scheme="tw_dd", precision=precision, fs_tol=1e-8, mg_tol=1e-8,
                          tile=(4, 3, 2))
    a, ra = run(p, opts)
    monkeypatch.setenv("DOMA_SWEEP_SCHEDULE", "levels")
    b, rb = run(p, opts)
    assert np.array_equal(a, b) and list(ra.si_counts) == list(rb.si_counts)


@pytest.mark.parametrize("tile", [8, 16, 32])
@pytest.mark.parametrize("np_,na", [(2, 3), (3, 3), (5, 5)])
@pytest.mark.parametrize("scheme", ["dd", "tw_dd"])
@pytest.mark.parametrize("dims", [2, 3])
def test_schedules_agree_across_shapes(monkeypatch, tile, np_, na, scheme, dims):
    """The dataflow sweep and the one-launch-per-level sweep give the same
    bits in single precision for every block length and scheme, with an odd
    number of ordinates per octant (the last warp half used) and with more
    ordinates per octant than one task holds (25 = 16 + 9)."""
    p = P.random_problem(43, dims, 21, 13, 6, groups=2, np_=np_, na=na, materials=3)
    opts = P.make_options(scheme=scheme, theta=0.8, precision="fp32", fs_tol=1e-6, mg_tol=1e-6,
                          tile=(tile, 0, 0))
    a, ra = run(p, opts)
    monkeypatch.setenv("DOMA_SWEEP_SCHEDULE", "levels")
    b, rb = run(p, opts)
    assert list(ra.si_counts) == list(rb.si_counts)
    assert np.array_equal(a, b), rel_linf(a, b)


def test_wait_timeout_is_reported_and_context_survives(monkeypatch):
    """A dependency wait that can never be satisfied gives up after a bounded
    number of polls; the host sees DOMA_DEVICE_WAIT_TIMEOUT and the CUDA
    context stays usable."""
    from doma_gb300 import abi
    p = P.random_problem(42, 3, 10, 9, 8, groups=1, np_=1, na=2, materials=2)
    opts = P.make_options(tile=(4, 4, 4))
    monkeypatch.setenv("DOMA_SWEEP_WAIT_TEST", "1")
    with pytest.raises(abi.DomaError) as ei:
        run(p, opts)
    assert ei.value.status == abi.DOMA_DEVICE_WAIT_TIMEOUT
    monkeypatch.delenv("DOMA_SWEEP_WAIT_TEST")
    phi, rep = run(p, opts)
    o_phi, ok, si, _, _ = ol.oracle_solve(p, opts)
    assert rep.converged and rel_linf(phi, o_phi) <= FP64_RTOL


@pytest.mark.parametrize("name", ["random3d_fission_twdd", "capped_si_twdd", "capped_mg_dd",
                                  "square2d_dd"])
def test_graph_loop_equals_host_loop(monkeypatch, name):
    """The solve captured as one CUDA graph (device-side loop tests through
    conditional WHILE nodes) and the host-driven loop give the same bits,
    iteration counts and status."""
    p, opts, exp = load_case(name)
    a, ra = run(p, opts)
    monkeypatch.setenv("DOMA_SOLVE_LOOP", "host")
    b, rb = run(p, opts)
    assert np.array_equal(a, b)
    assert list(ra.si_counts) == list(rb.si_counts)
    assert (ra.status, ra.mg_iterations, ra.si_iterations) == (rb.status, rb.mg_iterations,
                                                               rb.si_iterations)
    assert np.array_equal(a, exp["phi"])


@pytest.mark.parametrize("loop", ["graph", "host"])
@pytest.mark.parametrize("name", case_names())
def test_progress_lines_match_reference(monkeypatch, capfd, loop, name):
    """DOMA's stdout (MGI / SI lines) is reproduced line for line."""
    p, opts, exp = load_case(name)
    if loop == "host":
        monkeypatch.setenv("DOMA_SOLVE_LOOP", "host")
    opts.verbose = 1
    capfd.readouterr()
    run(p, opts)
    out = capfd.readouterr().out
    assert out == exp["log"]
    if exp["log_verbose"] is not None:
        opts.verbose = 2
        run(p, opts)
        assert capfd.readouterr().out == exp["log_verbose"]


# ---- multigroup mode (every group in flight) -----------------------------------

@pytest.mark.parametrize("dims", [2, 3])
@pytest.mark.parametrize("scheme", ["dd", "tw_dd"])
def test_multigroup_matches_oracle_iteration(dims, scheme):
    """FP64 multigroup mode against the CPU restatement of the same iteration:
    same iteration count, same flux (1e-12), and FP32 within 1e-5 of it."""
    p = P.random_problem(51, dims, 9, 8, 6, groups=4, np_=2, na=2, materials=3, fission=True)
    o64 = P.make_options(scheme=scheme, theta=0.8, fs_tol=1e-11, fs_max_it=5000,
                         iteration="multigroup")
    o_phi, ok, o_it, _ = ol.oracle_multigroup_solve(p, o64)
    phi, rep = run(p, o64)
    assert rep.converged == ok and rep.mg_iterations == o_it
    assert rel_linf(phi, o_phi) <= FP64_RTOL
    o32 = P.make_options(scheme=scheme, theta=0.8, precision="fp32", fs_tol=1e-7,
                         fs_max_it=5000, iteration="multigroup")
    phi32, rep32 = run(p, o32)
    assert rep32.converged and rel_l2(phi32, o_phi) <= FP32_RTOL, rel_l2(phi32, o_phi)


@pytest.mark.parametrize("dims", [2, 3])
def test_multigroup_dd_has_the_reference_fixed_point(dims):
    """DD is linear, so multigroup iteration converges to DOMA's own solution.
    (TW-DD is not: its weights act on increments, so each iteration path has
    its own fixed point; DOMA's is reached only by the Gauss-Seidel mode.)"""
    p = P.random_problem(53, dims, 9, 8, 6, groups=4, np_=2, na=2, materials=3, fission=True)
    ref_opts = P.make_options(scheme="dd", fs_tol=1e-13, mg_tol=1e-13, fs_max_it=5000,
                              mg_max_it=2000)
    o_phi, ok, *_ = ol.oracle_solve(p, ref_opts)
    assert ok
    phi, rep = run(p, P.make_options(scheme="dd", fs_tol=1e-13, fs_max_it=5000,
                                     iteration="multigroup"))
    assert rep.converged and rel_l2(phi, o_phi) <= 1e-10, rel_l2(phi, o_phi)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_multigroup_graph_equals_host_loop_and_levels(monkeypatch, precision):
    p = P.checkerboard(2, n=12, groups=3, np_=2, na=2, block=4)
    opts = P.make_options(scheme="tw_dd", theta=0.7, precision=precision, fs_tol=1e-7,
                          fs_max_it=2000, iteration="multigroup")
    a, ra = run(p, opts)
    monkeypatch.setenv("DOMA_SOLVE_LOOP", "host")
    b, rb = run(p, opts)
    monkeypatch.setenv("DOMA_SWEEP_SCHEDULE", "levels")
    c, rc = run(p, opts)
    assert np.array_equal(a, b) and np.array_equal(a, c)
    assert ra.mg_iterations == rb.mg_iterations == rc.mg_iterations
    assert ra.si_iterations == ra.mg_iterations * p.num_groups


def test_multigroup_cap_is_reported():
    p = P.random_problem(52, 3, 6, 5, 4, groups=3, np_=1, na=2, materials=2)
    opts = P.make_options(fs_tol=1e-14, fs_max_it=4, iteration="multigroup")
    phi, rep = run(p, opts)
    assert not rep.converged and rep.status == 1 and rep.mg_iterations == 4


# ---- k-eigenvalue power iteration ------------------------------------------------

def run_eigen(p, opts, k_tol):
    with Solver(p, opts) as s:
        rep, k = s.solve_eigenvalue(k_tol)
        return s.scalar_flux(), rep, k


@pytest.mark.parametrize("name", eigen_case_names())
def test_fp64_eigenvalue_matches_reference_golden(name):
    """DOMA's solveEigenvalue: same return value, power-iteration and SI
    counts, k and flux (the contract is 1e-12 relative; the host-side k update
    sums in DOMA's order, so both come out bit-equal)."""
    p, opts, k_tol, exp = load_eigen_case(name)
    phi, rep, k = run_eigen(p, opts, k_tol)
    assert rep.converged == exp["converged"]
    assert rep.mg_iterations == exp["pi_iterations"]
    assert list(rep.si_counts) == list(exp["si_counts"])
    if exp["k_is_final"]:
        assert abs(k - exp["k"]) <= 1e-12 * abs(exp["k"])
    assert rel_linf(phi, exp["phi"]) <= FP64_RTOL


@pytest.mark.parametrize("loop", ["graph", "host"])
@pytest.mark.parametrize("name", eigen_case_names())
def test_eigenvalue_progress_lines_match_reference(monkeypatch, capfd, loop, name):
    """The PI / SI progress lines of solveEigenvalue, line for line, with each
    power iteration's group loop as a graph launch and as the host loop."""
    p, opts, k_tol, exp = load_eigen_case(name)
    if loop == "host":
        monkeypatch.setenv("DOMA_SOLVE_LOOP", "host")
    opts.verbose = 1
    capfd.readouterr()
    run_eigen(p, opts, k_tol)
    assert capfd.readouterr().out == exp["log"]
    if exp["log_verbose"] is not None:
        opts.verbose = 2
        run_eigen(p, opts, k_tol)
        assert capfd.readouterr().out == exp["log_verbose"]


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("name", ["eigen3d_twdd", "eigen2d_dd", "eigen_capped_dd"])
def test_eigenvalue_graph_equals_host_loop(monkeypatch, precision, name):
    """The group loop captured as a graph (k read from device memory) and the
    host-driven loop give the same bits, k, counts and status."""
    p, opts, k_tol, exp = load_eigen_case(name)
    opts.precision = 0 if precision == "fp64" else 1
    a, ra, ka = run_eigen(p, opts, k_tol)
    monkeypatch.setenv("DOMA_SOLVE_LOOP", "host")
    b, rb, kb = run_eigen(p, opts, k_tol)
    assert np.array_equal(a, b) and ka == kb
    assert list(ra.si_counts) == list(rb.si_counts)
    assert (ra.status, ra.mg_iterations, ra.si_iterations) == (rb.status, rb.mg_iterations,
                                                               rb.si_iterations)


@pytest.mark.parametrize("scheme", ["dd", "tw_dd"])
def test_fp32_eigenvalue_against_fp64(scheme):
    """The FP32 sweep in the power iteration: k within 1e-5 and the flux within
    1e-4 (relative L2) of the FP64 mode's."""
    p, _, k_tol, _ = load_eigen_case("eigen3d_dd")
    kw = dict(scheme=scheme, theta=0.9, fs_tol=1e-7, mg_tol=1e-6, mg_max_it=400)
    phi64, rep64, k64 = run_eigen(p, P.make_options(precision="fp64", **kw), 1e-7)
    phi32, rep32, k32 = run_eigen(p, P.make_options(precision="fp32", **kw), 1e-7)
    assert rep64.converged and rep32.converged
    assert abs(k32 - k64) <= 1e-5 * k64
    assert np.linalg.norm(phi32 - phi64) / np.linalg.norm(phi64) <= 1e-4


def test_eigenvalue_needs_fission_and_gauss_seidel():
    """Input errors come back as DOMA_BAD_INPUT (checked before any GPU work)."""
    from doma_gb300 import abi
    p = P.random_problem(3, 3, 4, 4, 4, groups=2)  # no fissile material
    with Solver(p, P.make_options()) as s:
        with pytest.raises(abi.DomaError, match="fissile"):
            s.solve_eigenvalue(1e-6)


# ---- transient (zero initial condition) -------------------------------------------

def run_transient(p, tr, opts, stop_after=None):
    """-> (per-step fluxes, per-step precursors, final flux, report)."""
    phis, dnps = [], []

    def on_step(step, t, phi, dn):
        phis.append(phi)
        dnps.append(dn)
        return stop_after is not None and step >= stop_after

    with Solver(p, opts) as s:
        rep = s.solve_transient(tr, on_step)
        return phis, dnps, s.scalar_flux(), rep


@pytest.mark.parametrize("name", transient_case_names())
def test_fp64_transient_matches_reference_golden(name):
    """DOMA's solveTransient: same return value and SI counts, every step's
    flux and the precursors within 1e-12 (relative L-infinity), including a
    solve that stops part-way (its partial flux is the one DOMA keeps)."""
    p, tr, opts, exp = load_transient_case(name)
    phis, dnps, last, rep = run_transient(p, tr, opts)
    assert rep.converged == exp["converged"]
    assert len(phis) == exp["steps_done"]
    assert list(rep.si_counts) == list(exp["si_counts"])
    ref = exp["phi_steps"]
    for k, phi in enumerate(phis):
        assert rel_linf(phi, ref[k]) <= FP64_RTOL, k
    assert rel_linf(last, ref[-1]) <= FP64_RTOL
    if tr.num_d_groups and phis:
        assert rel_linf(dnps[-1], exp["dnps"]) <= FP64_RTOL


def test_fp64_transient_bit_equal_to_reference_golden():
    """As for fixed source: the exact-order FP64 path gives DOMA's bits."""
    unequal = []
    for name in transient_case_names():
        p, tr, opts, exp = load_transient_case(name)
        phis, dnps, last, rep = run_transient(p, tr, opts)
        for k, phi in enumerate(phis):
            if not np.array_equal(phi, exp["phi_steps"][k]):
                unequal.append((name, k, rel_linf(phi, exp["phi_steps"][k])))
        if not np.array_equal(last, exp["phi_steps"][-1]):
            unequal.append((name, "last", rel_linf(last, exp["phi_steps"][-1])))
    assert not unequal, unequal


@pytest.mark.parametrize("name", ["transient3d_twdd", "transient2d_dd",
                                  "transient3d_capped_mid_dd", "transient2d_capped_si_dd"])
def test_transient_graph_equals_host_loop(monkeypatch, name):
    p, tr, opts, exp = load_transient_case(name)
    a = run_transient(p, tr, opts)
    monkeypatch.setenv("DOMA_SOLVE_LOOP", "host")
    b = run_transient(p, tr, opts)
    assert len(a[0]) == len(b[0])
    assert all(np.array_equal(x, y) for x, y in zip(a[0], b[0]))
    assert all(np.array_equal(x, y) for x, y in zip(a[1], b[1]))
    assert np.array_equal(a[2], b[2])
    ra, rb = a[3], b[3]
    assert list(ra.si_counts) == list(rb.si_counts)
    assert (ra.status, ra.mg_iterations, ra.si_iterations) == (rb.status, rb.mg_iterations,
                                                               rb.si_iterations)


@pytest.mark.parametrize("loop", ["graph", "host"])
@pytest.mark.parametrize("name", transient_case_names())
def test_transient_progress_lines_match_reference(monkeypatch, capfd, loop, name):
    """solveTransient's stdout (initial conditions, time steps, MGI / SI lines)."""
    p, tr, opts, exp = load_transient_case(name)
    if loop == "host":
        monkeypatch.setenv("DOMA_SOLVE_LOOP", "host")
    opts.verbose = 1
    capfd.readouterr()
    with Solver(p, opts) as s:
        s.solve_transient(tr)
    assert capfd.readouterr().out == exp["log"]
    if exp["log_verbose"] is not None:
        opts.verbose = 2
        with Solver(p, opts) as s:
            s.solve_transient(tr)
        assert capfd.readouterr().out == exp["log_verbose"]


@pytest.mark.parametrize("seed", [31, 32])
@pytest.mark.parametrize("scheme", ["dd", "tw_dd"])
@pytest.mark.parametrize("dims", [2, 3])
def test_fp64_transient_matches_oracle_random(seed, scheme, dims):
    p, tr = P.transient_problem(seed, dims=dims, nx=7, ny=6, nz=5, np_=2, na=2, num_steps=3,
                                t1=0.6)
    opts = P.make_options(scheme=scheme, theta=0.9, fs_tol=1e-10, mg_tol=1e-10)
    phis, dnps, _, rep = run_transient(p, tr, opts)
    o_phis, o_dnps, ok, done, si = ol.oracle_solve_transient(p, tr, opts)
    assert rep.converged and ok and len(phis) == done == 3
    assert list(rep.si_counts) == list(si)
    for k in range(3):
        assert rel_linf(phis[k], o_phis[k]) <= FP64_RTOL
    assert rel_linf(dnps[-1], o_dnps) <= FP64_RTOL


@pytest.mark.parametrize("scheme", ["dd", "tw_dd"])
def test_fp32_transient_against_fp64(scheme):
    """The FP32 sweep in a transient: each step's flux within 1e-5 (relative
    L2) of the FP64 mode's."""
    p, tr = P.transient_problem(41, dims=3, nx=12, ny=10, nz=8, np_=2, na=2, num_steps=3)
    kw = dict(scheme=scheme, theta=0.9, fs_tol=1e-8, mg_tol=1e-8)
    a = run_transient(p, tr, P.make_options(precision="fp64", **kw))
    b = run_transient(p, tr, P.make_options(precision="fp32", **kw))
    assert a[3].converged and b[3].converged
    for x, y in zip(b[0], a[0]):
        assert rel_l2(x, y) <= FP32_RTOL


def test_transient_callback_stops_and_solver_is_reused():
    """A nonzero callback return stops after that step (DOMA_BAD_INPUT with a
    message); the same solver then runs a transient with more delayed groups
    (tables regrown, step graph rebuilt) and a fixed-source solve, each
    matching a fresh solver's bits."""
    from doma_gb300 import abi
    p, tr = P.transient_problem(5, dims=3, num_steps=4, delayed=2)
    _, tr3 = P.transient_problem(5, dims=3, num_steps=4, delayed=3)
    opts = P.make_options(fs_tol=1e-9, mg_tol=1e-9)
    seen = []
    with Solver(p, opts) as s:
        with pytest.raises(abi.DomaError, match="callback stopped"):
            s.solve_transient(tr, lambda k, t, phi, d: seen.append(k) or k == 1)
        assert seen == [0, 1]
        out = []
        s.solve_transient(tr3, lambda k, t, phi, d: out.append((t, phi, d)) and False)
        fixed = s.solve_fixed_source()
        fixed_phi = s.scalar_flux()
    fresh = run_transient(p, tr3, opts)
    assert [t for t, _, _ in out] == tr3.times()
    assert all(np.array_equal(x, y) for (_, x, _), y in zip(out, fresh[0]))
    assert np.array_equal(out[-1][2], fresh[1][-1]) and out[-1][2].shape[0] == 3
    phi, rep = run(p, opts)
    assert np.array_equal(fixed_phi, phi) and fixed.si_counts.tolist() == rep.si_counts.tolist()


def test_transient_rejects_bad_input():
    """Transient input errors come back as DOMA_BAD_INPUT before any GPU work."""
    import dataclasses

    from doma_gb300 import abi
    p, tr = P.transient_problem(6, dims=3, num_steps=2)
    bad = [
        dataclasses.replace(tr, t1=0.0),
        dataclasses.replace(tr, step_remove=np.where(tr.step_type == 1, 0.0, tr.step_remove)),
        dataclasses.replace(tr, d_groups=np.array([3, 2, 1, 0], dtype=np.uint32)),  # no fission in 2
        dataclasses.replace(tr, lambda_=np.zeros_like(tr.lambda_)),
    ]
    with Solver(p, P.make_options()) as s:
        for b in bad:
            with pytest.raises(abi.DomaError) as e:
                s.solve_transient(b)
            assert e.value.status == abi.DOMA_BAD_INPUT
    with Solver(p, P.make_options(iteration="multigroup")) as s:
        with pytest.raises(abi.DomaError, match="Gauss-Seidel"):
            s.solve_transient(tr)
