/*
 * doma_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C, CPU restatement of DOMA's 2D/3D fixed-source path, used as the
 * checker for the GPU library (tests, the smoke check and the CPU-baseline leg
 * of the benchmark).  The product never links it.  Parity of this restatement
 * with DOMA itself is pinned two ways: bit-for-bit against the committed
 * golden fixtures (tests/golden/, produced by running DOMA's own code through
 * oracle/ref_harness.cpp), and live against oracle/_ref/libdoma_ref.so where
 * the DOMA sources are present.
 */
#ifndef DOMA_ORACLE_H
#define DOMA_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#include "../include/doma_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Quadrature binned by octant; returns the total order, or -1 on bad input. */
int oracle_quadrature(uint32_t np, uint32_t na, uint32_t dims, double *mu, double *eta,
                      double *xi, double *w, uint32_t counts[8]);

/* Full fixed-source solve.  phi_out: [G][N].  si_counts receives the SI count
 * of each (MG iteration, group) pair (up to si_cap entries; *si_len gets the
 * total).  Returns 1 converged, 0 cap reached, -1 bad input. */
int oracle_solve(const doma_problem *p, const doma_options *o, uint32_t num_threads,
                 double *phi_out, uint32_t *si_counts, size_t si_cap, size_t *si_len,
                 uint32_t *mg_iterations, double *mg_residual);

/* k-eigenvalue power iteration (DOMA's solveEigenvalue): Gauss-Seidel over
 * groups with source iteration, fission source / k, k from the production
 * ratio; stops when mg_max_it is reached or both the flux-shape residual
 * (<= mg_tol) and |k - k_prev| (<= k_tol) have converged.  phi_out: [G][N];
 * *k_out the last k.  Returns 1 converged, 0 a cap reached, -1 bad input. */
int oracle_solve_eigen(const doma_problem *p, const doma_options *o, double k_tol,
                       uint32_t num_threads, double *phi_out, double *k_out,
                       uint32_t *si_counts, size_t si_cap, size_t *si_len,
                       uint32_t *pi_iterations, double *shape_res_out, double *k_res_out);

/* Transient fixed source from a zero initial condition (DOMA's
 * solveTransient with TransientIC::Zero).  phi_steps ([num_steps][G][N], may
 * be NULL) receives each step's flux, and for a step whose solve failed the
 * partial flux it stopped with; dnps_out ([D][N], may be NULL) the precursor
 * concentrations after the last step done; *steps_done the steps completed.  Returns 1 when every step converged, 0 when a step's solve
 * reached a cap (the reference then returns false at once), -1 on bad input. */
int oracle_solve_transient(const doma_problem *p, const doma_options *o, const doma_transient *tr,
                           uint32_t num_threads, double *phi_steps, double *dnps_out,
                           uint32_t *steps_done, uint32_t *si_counts, size_t si_cap,
                           size_t *si_len);

/* From a zero flux: set up group g's source, then run `count` source
 * iterations (sweep, residual, update) with no convergence test.  phi_out
 * ([G][N]) gets the flux afterwards; residuals ([count]) the SI residuals.
 * This is the bounded CPU-baseline sample.  Returns 0, or -1 on bad input. */
int oracle_source_iterations(const doma_problem *p, const doma_options *o,
                             uint32_t num_threads, uint32_t group, uint32_t count,
                             double *phi_out, double *residuals);

/* Multigroup source iteration (the GPU library's DOMA_ITER_MULTIGROUP mode,
 * which DOMA itself does not have): increment form over all groups at once,
 * delta_q_h = s/pi * sum_g (S[h][g] + chi_h nu_sigma_f_g) delta_phi_g.  Same
 * sweep as oracle_solve; returns 1 converged, 0 cap reached, -1 bad input. */
int oracle_multigroup_solve(const doma_problem *p, const doma_options *o, uint32_t num_threads,
                            double *phi_out, uint32_t *iterations, double *residual);

/* Single-thread summation order with any thread count (on != 0): the
 * ordinates of an octant still sweep in parallel, but every cell's angular
 * sum and the residual norms follow the one-thread order, so results are
 * bit-equal to num_threads = 1.  Off (the default) the threads keep private
 * sums added in thread order, as DOMA does with T threads. */
void oracle_set_single_thread_order(int on);

#ifdef __cplusplus
}
#endif

#endif
