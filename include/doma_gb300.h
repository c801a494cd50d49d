/*
 * doma_gb300.h -- C ABI of the GB300 fixed-source discrete-ordinates solver.
 *
 * The library replaces DOMA's fixed-source hot path: the Gauss-Seidel loop
 * over energy groups, the within-group scattering-source iteration (increment
 * form) and the octant-by-octant transport sweep with diamond-difference (DD)
 * or theta-weighted diamond-difference (TW-DD) cell solves.  Everything
 * crosses this boundary as plain C: pointers, sizes and status codes.  No C++
 * or torch types appear here, so a C++ shim, ctypes or any other FFI can bind
 * it directly.
 *
 * Reference interfaces replaced (paths inside the DOMA source tree):
 *   doma_solver_create                 TransportSolver3D<T>::TransportSolver3D
 *                                      (src/TransportSolver3D.cpp:5-27) and
 *                                      TransportSolver2D<T>::TransportSolver2D
 *                                      (src/TransportSolver2D.cpp:5-27), plus the
 *                                      mesh set-up of BrickMesh3D/2D
 *                                      (src/BrickMesh3D.cpp:8-184)
 *   doma_solver_solve_fixed_source     TransportSolver3D<T>::solveFixedSource
 *                                      (src/TransportSolver3D.cpp:262-316) and the
 *                                      2D twin (src/TransportSolver2D.cpp:264-316)
 *   doma_solver_solve_eigenvalue       TransportSolver3D<T>::solveEigenvalue
 *                                      (src/TransportSolver3D.cpp:29-86, with
 *                                      updateMultigroupSourceEigen / updateEigenvalue
 *                                      :404-456) and the 2D twin
 *                                      (src/TransportSolver2D.cpp:31-88, :406-456)
 *   doma_solver_solve_transient        TransportSolver3D<T>::solveTransient with a zero
 *                                      initial condition (src/TransportSolver3D.cpp:88-140,
 *                                      initZeroIC / updateStepFluxes / stepDNPs :142-260,
 *                                      the transient terms of updateMultigroupSource
 *                                      :339-402) and the 2D twin
 *   doma_solver_get_scalar_flux        read-back of CartesianCell3D::_total_scalar_flux
 *                                      (include/CartesianCell3D.h:99), as used by
 *                                      BrickMesh3D::dumpToTextFile / fluxAtPoint
 *   doma_quadrature                    GCAngularQuadrature::GCAngularQuadrature,
 *                                      order/direction/weight
 *                                      (src/GCAngularQuadrature.cpp:9-75)
 *   doma_solver_source_iterations,     single steps of TransportSolver3D::sourceIteration
 *   doma_solver_sweeps                 (src/TransportSolver3D.cpp:458-497) and ::sweep
 *                                      (src/TransportSolver3D.cpp:565-622), exposed so a
 *                                      caller can time the hot loop on resident data
 *
 * Status codes replace the reference's std::exit(1) on bad input and its
 * `false` return on non-convergence; the library never exits the process.
 */
#ifndef DOMA_GB300_H
#define DOMA_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DOMA_ABI_VERSION 2u

/* Status codes returned by every entry point. */
typedef enum doma_status {
  DOMA_OK = 0,
  DOMA_NOT_CONVERGED = 1,        /* iteration cap reached (reference returns false) */
  DOMA_BAD_INPUT = 2,            /* invalid problem or options (reference exits) */
  DOMA_CUDA_ERROR = 3,           /* a CUDA runtime call failed */
  DOMA_DEVICE_WAIT_TIMEOUT = 4,  /* a bounded device-side wait gave up */
  DOMA_NO_DEVICE = 5,            /* no CUDA device is visible */
  DOMA_NUMERIC_ERROR = 6         /* a residual norm became NaN or Inf */
} doma_status;

/* Cell-balance scheme: EquationType DD / TW_DD (include/TransportBase.h:45-49). */
enum { DOMA_SCHEME_DD = 0, DOMA_SCHEME_TW_DD = 1 };

/* Arithmetic of the sweep.
 *   DOMA_PREC_FP64: reference drop-in.  Every cell solve uses the reference's
 *     operation order with round-to-nearest IEEE double and no fused
 *     multiply-add; the scalar flux is accumulated over directions in the
 *     reference's single-thread order (octant PPP..MMM, then ordinate).
 *   DOMA_PREC_FP32: single-precision sweep with compensated angular sums;
 *     sources, scalar flux, residual and convergence norms stay double. */
enum { DOMA_PREC_FP64 = 0, DOMA_PREC_FP32 = 1 };

/* Iteration structure.
 *   DOMA_ITER_GAUSS_SEIDEL: DOMA's own (solveFixedSource): groups in order,
 *     each with a within-group source iteration; fs_* and mg_* apply.
 *   DOMA_ITER_MULTIGROUP: every group in flight.  Source iteration on the
 *     whole multigroup scattering + fission operator in increment form: each
 *     iteration sweeps all groups in one launch, then forms the next
 *     increment's source for every group from all groups' increments.
 *     Converges to the same solution; fs_tol (relative L2 of the increment
 *     over all groups) and fs_max_it apply, mg_* are unused. */
enum { DOMA_ITER_GAUSS_SEIDEL = 0, DOMA_ITER_MULTIGROUP = 1 };

/* A fixed-source problem on a tensor-product Cartesian mesh.
 * Cells are numbered x fastest, then y, then z (src/BrickMesh3D.cpp:83-102).
 * Materials play the role of DOMA's block ids (include/InputParameters.h:24-48). */
typedef struct doma_problem {
  uint32_t num_dims;              /* 2 or 3 */
  uint32_t nx, ny, nz;            /* cells per axis; nz must be 1 when num_dims == 2 */
  const double *dx;               /* [nx] cell widths along x (cm) */
  const double *dy;               /* [ny] cell widths along y (cm) */
  const double *dz;               /* [nz] cell widths along z (cm); ignored in 2D */
  uint32_t num_groups;            /* G */
  uint32_t num_materials;         /* M */
  const uint32_t *cell_material;  /* [nx*ny*nz] material index of every cell */
  const double *total;            /* [M][G] total cross section */
  const double *scatter;          /* [M][G][G] row-major [to*G + from] */
  const double *source;           /* [M][G] isotropic external source, or NULL */
  const uint8_t *has_fission;     /* [M] nonzero: material carries a prompt
                                     fission spectrum, or NULL for none */
  const double *chi_p;            /* [M][G] prompt fission spectrum, or NULL */
  const double *nu_sigma_f;       /* [M][G] fission production, or NULL */
  uint32_t num_polar;             /* np of <angular_quad>: 2*np Legendre roots */
  uint32_t num_azimuthal;         /* na of <angular_quad>: 2*na Chebyshev roots */
} doma_problem;

/* Time-dependent data of a transient solve (DOMA's RunMode::Transient):
 * the per-block fields of MaterialProps that only transients read
 * (include/InputParameters.h:24-48) and the <source_step> blocks
 * (SourceStep, include/InputParameters.h:9-22), indexed by material.  The
 * delayed-group arrays are padded to num_d_groups; material m uses the first
 * d_groups[m] of them (DOMA's _num_d_groups, which may differ per block). */
typedef enum doma_step_type {
  DOMA_STEP_NONE = 0,    /* no source step in this material */
  DOMA_STEP_BOTH = 1,    /* on for insert_time <= t <= remove_time */
  DOMA_STEP_INSERT = 2,  /* on for insert_time <= t */
  DOMA_STEP_REMOVE = 3   /* on for t <= remove_time */
} doma_step_type;

typedef struct doma_transient {
  double dt;                   /* step length; DOMA: (t1 - t0) / num_steps */
  uint32_t num_steps;          /* time steps; the steps run at t = 0, dt, 2 dt, ... */
  uint32_t num_d_groups;       /* D: delayed-neutron groups (the most of any material) */
  const double *inv_v;         /* [M][G] inverse velocities */
  const uint32_t *d_groups;    /* [M] delayed groups of each material (<= D), or NULL: none */
  const double *chi_d;         /* [M][G][D] delayed spectra (DOMA's _n_g_chi_d, g*D_m + d) */
  const double *beta;          /* [M][G][D] delayed fractions (DOMA's _g_n_beta, g*D_m + d) */
  const double *lambda;        /* [M][D] decay constants */
  const uint32_t *step_type;   /* [M] doma_step_type, or NULL: no source steps */
  const double *step_insert;   /* [M] insertion times */
  const double *step_remove;   /* [M] removal times */
  const double *step_source;   /* [M][G] the stepped source */
} doma_transient;

/* Called after each time step of doma_solver_solve_transient with the step's
 * scalar flux phi[g*N + cell] and precursor concentrations dnps[d*N + cell]
 * (NULL when D = 0), both host memory valid during the call.  A nonzero
 * return stops the solve (DOMA_BAD_INPUT with that message). */
typedef int (*doma_step_callback)(void *user, uint32_t step, double t, const double *phi,
                                  const double *dnps);

/* Solver options (the <solver> block of a DOMA deck plus GPU choices). */
typedef struct doma_options {
  uint32_t scheme;      /* DOMA_SCHEME_DD or DOMA_SCHEME_TW_DD */
  double theta;         /* TW-DD theta (= theta_s); DOMA uses 0.9 */
  uint32_t precision;   /* DOMA_PREC_FP64 or DOMA_PREC_FP32 */
  double fs_tol;        /* source-iteration tolerance (relative L2 of the increment) */
  uint32_t fs_max_it;   /* source-iteration cap */
  double mg_tol;        /* Gauss-Seidel tolerance (relative L2 of the group change) */
  uint32_t mg_max_it;   /* Gauss-Seidel cap */
  uint32_t verbose;     /* 0: silent, 1: the reference's progress lines on stdout,
                           2: also every SI residual (the reference's --verbose) */
  uint32_t tile_x, tile_y, tile_z;   /* sweep block shape in cells; 0 = pick */
  uint32_t iteration;   /* DOMA_ITER_GAUSS_SEIDEL (default) or DOMA_ITER_MULTIGROUP */
} doma_options;

/* Filled by doma_solver_solve_fixed_source. */
typedef struct doma_report {
  uint32_t status;            /* doma_status of the solve */
  uint32_t mg_iterations;     /* Gauss-Seidel iterations performed */
  uint64_t si_iterations;     /* source iterations (= sweeps) over all groups */
  uint64_t updates;           /* cell * direction * group updates swept */
  uint64_t kernel_launches;   /* CUDA kernel launches issued by the solve */
  double mg_residual;         /* last Gauss-Seidel residual */
  double si_residual;         /* last source-iteration residual */
  double solve_ms;            /* host wall time of the solve */
  uint32_t *si_counts;        /* optional caller buffer: SI count of every
                                 (MG iteration, group) pair, in solve order */
  size_t si_counts_capacity;  /* entries available in si_counts */
  size_t si_counts_len;       /* entries written (may exceed capacity: the
                                 rest were dropped) */
} doma_report;

typedef struct doma_solver doma_solver;

/* Default options: DD, theta 0.9, FP64, tolerances 1e-8, caps 1000/100. */
void doma_default_options(doma_options *opts);

/* Last error message of the calling thread ("" if none). */
const char *doma_last_error(void);

/* ABI version of the loaded library (DOMA_ABI_VERSION). */
uint32_t doma_abi_version(void);

/* Gauss-Chebyshev product quadrature binned by octant, exactly as
 * GCAngularQuadrature(2*na, 2*np, num_dims) builds it.  Outputs are sized
 * 8*np*na (3D) or 4*np*na (2D) and ordered octant-major (PPP, PPM, PMP, PMM,
 * MPP, MPM, MMP, MMM), then by ordinate; counts[8] gets the per-octant sizes.
 * Host-only: needs no GPU. */
doma_status doma_quadrature(uint32_t num_polar, uint32_t num_azimuthal, uint32_t num_dims,
                            double *mu, double *eta, double *xi, double *weight,
                            uint32_t counts[8]);

/* Validate the problem, build the quadrature and upload everything to the
 * current CUDA device.  The problem arrays are copied; the caller may free
 * them after this returns. */
doma_status doma_solver_create(const doma_problem *problem, const doma_options *opts,
                               doma_solver **out);

/* Launch all work of this solver on `stream` (a cudaStream_t; NULL = the
 * solver's own stream). */
doma_status doma_solver_set_stream(doma_solver *solver, void *stream);

/* Zero the scalar flux and run the Gauss-Seidel / source-iteration solve.
 * Returns DOMA_OK, or DOMA_NOT_CONVERGED when an iteration cap was hit (the
 * flux of the last iterate is kept, as in the reference). */
doma_status doma_solver_solve_fixed_source(doma_solver *solver, doma_report *report);

/* k-eigenvalue power iteration.  Gauss-Seidel over groups with a source
 * iteration per group, as in the fixed-source solve, but the group source is
 * in-scatter plus fission divided by k (no external source), the flux starts
 * at 1 everywhere, and after each pass k is updated from the ratio of
 * volume-weighted production sums.  Stops when opts.mg_max_it passes are done,
 * or when both the flux-shape residual <= opts.mg_tol and |k - k_prev| <= k_tol.
 * report->mg_iterations counts the passes (power iterations) and
 * report->mg_residual is the last shape residual; *k gets the last k.
 * Returns DOMA_OK, or DOMA_NOT_CONVERGED when a cap was reached (DOMA's
 * false).  Gauss-Seidel iteration mode only. */
doma_status doma_solver_solve_eigenvalue(doma_solver *solver, double k_tol, doma_report *report,
                                         double *k);

/* Time-dependent fixed-source solve from a zero initial condition: at each
 * step the Gauss-Seidel / source-iteration solve of doma_solver_solve_fixed_source
 * with the transient source terms (source steps, prompt fission scaled by
 * 1 - beta, delayed neutrons, the previous step's flux times inv_v / dt), then
 * the precursor update, then `callback` (may be NULL), then the previous-step
 * flux := this step's.  Returns DOMA_OK, or DOMA_NOT_CONVERGED as soon as a
 * step's solve reaches a cap (DOMA's false).  report covers the last step.
 * Gauss-Seidel iteration mode only.  DOMA's steady-state initial condition is
 * not offered: the reference's version reads the precursor and previous-step
 * arrays before it sizes them. */
doma_status doma_solver_solve_transient(doma_solver *solver, const doma_transient *tr,
                                        doma_step_callback callback, void *user,
                                        doma_report *report);

/* Copy the scalar flux to host memory: out[g*N + cell], N = nx*ny*nz. */
doma_status doma_solver_get_scalar_flux(doma_solver *solver, double *out, size_t count);

/* Set up the group-g source (external + in-scatter + fission) from the
 * current flux, then run `count` source iterations (sweep, residual, source
 * update) without a convergence test.  Stream-ordered; does not synchronise. */
doma_status doma_solver_source_iterations(doma_solver *solver, uint32_t group, uint32_t count);

/* Run `count` bare sweeps of group g on the current iteration source (no
 * residual, no update).  Stream-ordered; for timing the sweep kernels. */
doma_status doma_solver_sweeps(doma_solver *solver, uint32_t group, uint32_t count);

/* Sweep block shape and launch counts actually in use (for reports). */
doma_status doma_solver_describe(const doma_solver *solver, uint32_t tile[3],
                                 uint32_t *launches_per_sweep, uint64_t *kernel_launches);

void doma_solver_destroy(doma_solver *solver);

/* ---- Batched solve: many independent problems, one persistent sweep ----
 * No counterpart in DOMA (it solves one deck per process).  Every problem is
 * solved with DOMA_ITER_MULTIGROUP in FP32; each batch iteration sweeps every
 * group of every unconverged problem in ONE persistent launch (the problems'
 * tasks merged level by level), then updates all of them in one batched
 * epilogue; a problem stops when its own relative increment norm is <=
 * fs_tol (or at fs_max_it).  All problems share dims and scheme. */
typedef struct doma_batch doma_batch;

doma_status doma_batch_create(const doma_problem *problems, size_t count,
                              const doma_options *opts, doma_batch **out);
doma_status doma_batch_set_stream(doma_batch *batch, void *stream);
/* Autotune the block length (8, 16 or 32 cells along x) per class of
 * problems -- (16-cell bucket of the longest axis, ordinates per octant,
 * groups) -- by timing batched sweeps with each class alone active, then
 * keep the per-class lengths if the whole batch sweeps faster with them than
 * with the best single length.  *tile_x gets the most common length;
 * doma_batch_tiles gives each problem's.  Results do not depend on it. */
doma_status doma_batch_tune(doma_batch *batch, uint32_t *tile_x);
doma_status doma_batch_tiles(doma_batch *batch, uint32_t *tiles, size_t count);
/* What the last doma_batch_tune measured: ms of two batched sweeps with each
 * uniform length (uniform_ms[3]: 8, 16, 32) and with the per-class lengths. */
doma_status doma_batch_tune_report(doma_batch *batch, float *uniform_ms, float *mixed_ms,
                                   uint32_t *classes);
/* Solve every problem; reports[i] (count entries, may be NULL) get each
 * problem's status, iterations (mg_iterations) and updates.  Returns DOMA_OK
 * when all converged, else the first failing status. */
doma_status doma_batch_solve(doma_batch *batch, doma_report *reports, size_t count);
doma_status doma_batch_get_scalar_flux(doma_batch *batch, size_t index, double *out,
                                       size_t count);
/* Stepping (what doma_batch_solve does, in parts): begin sets every problem
 * to a zero flux with its external source; iterate runs up to `iterations`
 * batched iterations (fewer once no problem is active; *active gets the count
 * still iterating); state returns DEVICE pointers to a problem's scalar flux
 * and last increment ([G][N] doubles each, valid until the next call that
 * iterates); reports fills per-problem reports as doma_batch_solve does. */
doma_status doma_batch_begin(doma_batch *batch);
doma_status doma_batch_iterate(doma_batch *batch, uint32_t iterations, uint32_t *active);
doma_status doma_batch_state(doma_batch *batch, size_t index, const double **phi,
                             const double **increment);
doma_status doma_batch_reports(doma_batch *batch, doma_report *reports, size_t count);
/* Replace problem `index`'s last increment by `increment` (DEVICE [G][N]
 * doubles) and form the next sweep's source from it: the following
 * iteration then sweeps that field (the transport operator applied to an
 * arbitrary error field; used to generate training pairs). */
doma_status doma_batch_set_increment(doma_batch *batch, size_t index, const double *increment);
void doma_batch_destroy(doma_batch *batch);

/* One FP32 sweep that allocates no memory -- no counterpart in DOMA.
 * For callers that cannot call cudaMalloc (code inside another framework's
 * memory pool or allocator budget, or that must keep its device footprint
 * fixed after start-up): one transport sweep of one group over all octants
 * and ordinates, the solver's FP32 kernel, with every piece of device scratch
 * in a fixed static device array of DOMA_NOALLOC_SCRATCH_BYTES (64 MiB, held
 * by every GPU that loads the library) and host staging in static buffers.
 * Inputs: the mesh and quadrature of `problem` (dims, nx/ny/nz, dx/dy/dz,
 * num_polar, num_azimuthal <= 8; materials are not read), the scheme and
 * theta, and device arrays q[N] (isotropic source per steradian) and
 * sigma_t[N] of the group, N = nx*ny*nz, x fastest.  Output: the swept scalar
 * flux phi_out[N] (device, double) -- what one source iteration from a zero
 * flux gives.  Problems that need more scratch are rejected with
 * DOMA_BAD_INPUT.  All calls share the array: calls that overlap on the GPU
 * race.  Every call looks up the array's device address on the current
 * device (cudaGetSymbolAddress), copies small tables from host memory and
 * synchronises `stream` before returning, so it cannot be called on a stream
 * that is being captured into a CUDA graph (it returns DOMA_BAD_INPUT). */
#define DOMA_NOALLOC_SCRATCH_BYTES (64u << 20)
doma_status doma_sweep_noalloc(const doma_problem *problem, uint32_t scheme, double theta,
                               const float *q, const float *sigma_t, double *phi_out,
                               void *stream);

/* ---- Learned source-iteration accelerator -- no counterpart in DOMA ------
 * doma_unet: a 3D convolutional U-Net (4 levels, 32/64/128/256 channels,
 * 3x3x3 convolutions, average pooling down, nearest upsampling with additive
 * skips up, a linear 1-channel FP32 head) with BF16 weights and activations
 * and FP32 accumulation, run and trained by this library's kernels.
 * Tensors are device memory, channels-last: input [batch][nz][ny][nx][16]
 * bf16 (channels beyond those used must be zero), output and target
 * [batch][nz][ny][nx] float.  nz, ny, nx must be multiples of 8.
 * Parameters are one flat FP32 array: per convolution (14, encoder then
 * decoder) weights [27][cout][cin] then biases [cout]; then the head's
 * weights [32] and bias [1].  Tap index = (dz+1)*9 + (dy+1)*3 + (dx+1). */
typedef struct doma_unet doma_unet;
#define DOMA_UNET_IN_CHANNELS 16u
doma_status doma_unet_create(uint64_t seed, doma_unet **out);
void doma_unet_destroy(doma_unet *net);
doma_status doma_unet_set_stream(doma_unet *net, void *stream);
size_t doma_unet_num_params(const doma_unet *net);
doma_status doma_unet_get_params(doma_unet *net, float *out, size_t count);
doma_status doma_unet_set_params(doma_unet *net, const float *in, size_t count);
doma_status doma_unet_get_grads(doma_unet *net, float *out, size_t count);
doma_status doma_unet_forward(doma_unet *net, const void *input, float *output, uint32_t batch,
                              uint32_t nz, uint32_t ny, uint32_t nx);
/* Forward pass, mean-square loss against target, and the gradient of that
 * loss for every parameter (read with doma_unet_get_grads). */
doma_status doma_unet_backward(doma_unet *net, const void *input, const float *target,
                               uint32_t batch, uint32_t nz, uint32_t ny, uint32_t nx);
/* The same with a weight per sample (device, batch floats): each sample's
 * squared error, and so its share of every gradient, is scaled by its
 * weight; the reported loss is the weighted mean.  Used to train on targets
 * of very different sizes without the largest dominating. */
doma_status doma_unet_backward_weighted(doma_unet *net, const void *input, const float *target,
                                        const float *sample_weight, uint32_t batch, uint32_t nz,
                                        uint32_t ny, uint32_t nx);
doma_status doma_unet_last_loss(doma_unet *net, double *loss);
/* One Adam step (bias-corrected) with the last gradients. */
doma_status doma_unet_adam(doma_unet *net, float lr, float beta1, float beta2, float eps);
/* One 3x3x3 convolution of the network's kind (zero padding, stride 1):
 * y = act(conv(x, w) + bias), x [batch][nz][ny][nx][cin] bf16, w
 * [27][cout][cin] bf16, bias [cout] float or NULL, y [..][cout] bf16, all
 * device memory; cin in {16,32,64,128,256}, cout in {32,64,128,256}.  path
 * selects the kernel: DOMA_CONV_AUTO (tensor-memory kernel where the shape
 * tiles into 128-voxel boxes, else the warp-MMA kernel), DOMA_CONV_MMA or
 * DOMA_CONV_TENSOR_MEMORY (tcgen05 + TMA; BAD_INPUT for shapes it does not
 * tile).  On shapes with fewer 128-voxel tiles than SMs the tensor-memory
 * kernel splits its reduction over the taps and adds the FP32 partials in a
 * fixed order, in scratch allocated and freed on `stream`.  Asynchronous on
 * `stream`.  doma_conv_wait_error reads the flag the tensor-memory kernel
 * sets if one of its bounded waits gave up. */
enum { DOMA_CONV_AUTO = 0, DOMA_CONV_MMA = 1, DOMA_CONV_TENSOR_MEMORY = 2 };
doma_status doma_conv3_forward(const void *x, uint32_t batch, uint32_t nz, uint32_t ny,
                               uint32_t nx, uint32_t cin, const void *w, const float *bias,
                               uint32_t cout, uint32_t relu, void *y, uint32_t path, void *stream);
doma_status doma_conv_wait_error(int *flag);
/* The weight gradient of one such convolution: dw[27][cout][cin] (FP32,
 * device) = sum over voxels of x[voxel + tap offset][cin] * dz[voxel][cout],
 * x [batch][nz][ny][nx][cin] and dz [...][cout] bf16 channels-last, reduced
 * in a fixed order.  path as above: the tensor-memory kernel stacks taps
 * along the MMA's 128 rows; DOMA_CONV_MMA is the warp-MMA kernel.  Scratch
 * for the partial sums is allocated on `stream` and freed there. */
doma_status doma_conv3_wgrad(const void *x, uint32_t batch, uint32_t nz, uint32_t ny, uint32_t nx,
                             uint32_t cin, const void *dz, uint32_t cout, float *dw,
                             uint32_t path, void *stream);

/* Learned corrections inside a multigroup solve (3D, DD, extents multiples
 * of 8).  After `first` iterations, and then every `interval` iterations,
 * the network proposes a correction of the flux from the last increment,
 * group by group; the next iteration sweeps from the corrected iterate.  With
 * `guard` set, a correction after which the relative increment norm rose is
 * undone (the flux, increment and source of the iterate before it come back;
 * that sweep is spent), so the plain iteration stays the fallback and the
 * fixed point is the plain solver's.  The network must outlive the solver's
 * solves (net NULL detaches it). */
typedef struct {
  uint32_t first;            /* iterations before the first correction (>= 1) */
  uint32_t interval;         /* plain iterations between corrections */
  uint32_t max_corrections;  /* corrections tried at most */
  uint32_t guard;            /* 1: undo corrections that raise the residual */
} doma_accel_options;
doma_status doma_solver_set_accelerator(doma_solver *solver, doma_unet *net,
                                        const doma_accel_options *opts);
/* Stop a multigroup solve once the relative L2 error of the flux against
 * phi_ref ([G][N] host values) is <= target_error, instead of on the
 * increment norm (time-to-accuracy measurements).  phi_ref NULL removes it. */
doma_status doma_solver_set_reference(doma_solver *solver, const double *phi_ref, size_t count,
                                      double target_error);
typedef struct {
  uint32_t iterations;
  uint32_t corrections_accepted;
  uint32_t corrections_rejected;
  uint32_t reserved;
  double error;     /* last relative L2 error against the reference, or -1 */
  double solve_ms;  /* wall time of the last guided solve */
} doma_accel_stats;
doma_status doma_solver_accel_stats(const doma_solver *solver, doma_accel_stats *out);

#ifdef __cplusplus
}  /* extern "C" */
#endif

#endif /* DOMA_GB300_H */
