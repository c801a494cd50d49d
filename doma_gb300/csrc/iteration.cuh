// iteration.cuh -- per-cell iteration kernels (iteration.cu) and the device
// state that lets them drive the solve's loops inside a CUDA graph.
#pragma once

#include "common.cuh"

namespace doma {

struct IterArgs {
  size_t N = 0;               // cells
  int G = 0;                  // groups
  int D = 0;                  // ordinates (exact-mode row length of wpsi)
  int grid = 0;               // fixed grid of every per-cell kernel
  int epi_grid = 0;           // fixed grid of the FP32 source-iteration epilogue
  unsigned oct_mask = 0;      // octants that carry ordinates
  int ngroups = 1;            // fp32: ordinate groups per octant (partials per octant)
  bool exact = false;         // FP64 exact mode: the sweep wrote wpsi, not octphi
  double src_scale = 0.25;    // 1/(4 pi) prefactor numerator: 0.25 (3D), 0.5 (2D)
  const double * vol = nullptr;       // [N]
  const uint32_t * mat = nullptr;     // [N]
  const double * total = nullptr;     // [M][G]
  const double * scatter = nullptr;   // [M][G][G] [to][from]
  const double * source = nullptr;    // [M][G] or null
  const uint8_t * fis = nullptr;      // [M] or null
  const double * chi = nullptr;       // [M][G]
  const double * nsf = nullptr;       // [M][G]
  const double * qcoef = nullptr;     // [M][G] src_scale * S_gg / pi (FP32 epilogue)
  // FP32 mode's group source: [M][G][G] s (S[g][g'] (g' != g) + chi_g nu_sigma_f_g') / pi
  // and [M][G] s Q_g / pi
  const double * mgcoef = nullptr;
  const double * srcq = nullptr;
  double * phi = nullptr;             // [G][N]
  double * prev = nullptr;            // [G][N]
  const double * wpsi = nullptr;      // exact: [groups in flight][N][D]
  const float2 * octphi = nullptr;    // fp32: [8 * ngroups][N] partials (hi, lo), see PartialSum
  double * partials = nullptr;        // [grid][2]
  unsigned * ticket = nullptr;        // last-block ticket (kept at 0 between launches)
  // Multigroup mode, the iteration after a learned correction Delta ([G][N]):
  // the sweep's result minus Delta is the increment from the corrected
  // iterate (the flux itself takes the full sweep result).  Null otherwise.
  const float * corr = nullptr;
};

// Transient mode (doma_transient on the device).  clock[0] is the step's
// time t, clock[1] the step length dt: device memory, so that one captured
// graph serves every step.  Delayed-group arrays are padded to D.
struct TransientArgs {
  int D = 0;                          // delayed groups (padded)
  bool dims2 = false;                 // 2D: the cell solves see sigma_t + inv_v / dt
  double * clock = nullptr;           // [2] t, dt
  const double * inv_v = nullptr;     // [M][G]
  const uint32_t * dg = nullptr;      // [M] delayed groups per material, or null
  const double * chi_d = nullptr;     // [M][G][D]
  const double * beta = nullptr;      // [M][G][D]
  const double * lambda = nullptr;    // [M][D]
  const double * decay = nullptr;     // [M][D] exp(-lambda dt), formed on the host
  const uint32_t * step_type = nullptr;   // [M] or null
  const double * step_insert = nullptr;   // [M]
  const double * step_remove = nullptr;   // [M]
  const double * step_source = nullptr;   // [M][G]
  double * last = nullptr;            // [G][N] previous step's flux
  double * dnps = nullptr;            // [D][N] precursor concentrations
};

// Device-side solve state (one per solver, in device memory; mirrored in
// pinned host memory for read-back).
struct LoopCtl {
  double norms[4];          // SI (diff, total), MG (diff, total)
  int error;                // a sweep wait timed out (DOMA_DEVICE_WAIT_TIMEOUT) or 0
  unsigned ticket;          // persistent sweep: next task
  unsigned exit_count;      // persistent sweep: CTAs that have left
  unsigned epoch;           // persistent sweep: sweeps completed
  // graph-driven loops
  unsigned si_it;           // source iterations of the group being solved
  unsigned mg_it;           // Gauss-Seidel iterations completed
  unsigned failed;          // 0, or the doma_status that stopped the solve
  unsigned pairs;           // (MG iteration, group) pairs completed
  unsigned long long sweeps;    // source iterations over the whole solve
  unsigned long long hist_len;  // SI residuals recorded
  double si_res;            // last SI residual
  double mg_res;            // last Gauss-Seidel residual
};

// Kernel argument for the graph-driven loops.  With graph == 0 the kernels
// only compute (the host drives the loops and reads the norms).
struct LoopParams {
  LoopCtl * ctl = nullptr;
  unsigned * pair_counts = nullptr;   // [pair_cap] SI count per (MG iteration, group)
  double * pair_res = nullptr;        // [pair_cap] last SI residual per pair
  unsigned pair_cap = 0;
  double * si_hist = nullptr;         // [hist_cap] every SI residual (verbose runs)
  unsigned long long hist_cap = 0;
  double * mg_hist = nullptr;         // [mg_cap] every Gauss-Seidel residual
  unsigned mg_cap = 0;
  double fs_tol = 0.0, mg_tol = 0.0;
  unsigned fs_max_it = 0, mg_max_it = 0;
  int G = 0;
  unsigned long long si_handle = 0;   // cudaGraphConditionalHandle of the SI loop
  unsigned long long mg_handle = 0;   // cudaGraphConditionalHandle of the MG loop
  int graph = 0;
};

doma_status launch_mg_source(const IterArgs & a, int g, int precision, void * q, void * sigt,
                             const LoopParams & L, cudaStream_t st);
doma_status launch_si_epilogue(const IterArgs & a, int g, int precision, void * q,
                               double * norms, const LoopParams & L, cudaStream_t st);
// k-eigenvalue mode: group g's source added to the current one (in-scatter +
// fission / k), and the starting flux (1 everywhere).  k comes from *k_dev
// when that is not null (a captured graph), else from k; graph-aware like
// launch_mg_source.
doma_status launch_mg_source_eigen(const IterArgs & a, int g, int precision, double k,
                                   const double * k_dev, void * q, void * sigt,
                                   const LoopParams & L, cudaStream_t st);
doma_status launch_eigen_init(const IterArgs & a, cudaStream_t st);
// Transient mode: group g's source at the clock's t (external, source steps,
// in-scatter, prompt fission (1 - beta), delayed neutrons, previous-step
// flux inv_v / dt); graph-aware like launch_mg_source.
doma_status launch_mg_source_transient(const IterArgs & a, const TransientArgs & x, int g,
                                       int precision, void * q, void * sigt,
                                       const LoopParams & L, cudaStream_t st);
// Precursor step: C_d = (production / lambda_d) (1 - decay) + C_d decay.
doma_status launch_step_dnps(const IterArgs & a, const TransientArgs & x, cudaStream_t st);
// Next step: last := phi, phi := 0, t := t + dt.
doma_status launch_step_rollover(const IterArgs & a, const TransientArgs & x, cudaStream_t st);
doma_status launch_mg_residual(const IterArgs & a, double * norms, const LoopParams & L,
                               cudaStream_t st);
// Batched multigroup solve: per-problem data of the batched epilogue.
struct BatchSlot {
  IterArgs it;            // the problem's cell data (partials sized >= blocks)
  void * q;               // [G][N] next increment's source, sweep precision
  double * dscratch;      // [G][N]
  int block0;             // first block of this problem in the batched grid
  int blocks;             // blocks of this problem
};

doma_status launch_batch_epilogue(const BatchSlot * slots, const int * block_prob, int blocks,
                                  const BatchLoop * loops, int precision, cudaStream_t st);
// Graph-driven batched loop: counts the iteration, resets *still_active and
// sets the WHILE node's condition (handle) to go on while any problem is
// active, no sweep wait failed and fewer than max_iters iterations ran.
doma_status launch_batch_continue(unsigned * still_active, const int * error, unsigned * iters,
                                  unsigned max_iters, unsigned long long handle, cudaStream_t st);
doma_status launch_batch_finalize(const BatchSlot * slots, BatchLoop * loops, int count,
                                  double tol, unsigned max_it, unsigned * still_active,
                                  cudaStream_t st);

// Multigroup mode (every group in flight).
doma_status launch_mgi_init(const IterArgs & a, int precision, void * q, void * sigt,
                            cudaStream_t st);
doma_status launch_mgi_epilogue(const IterArgs & a, int precision, void * q, double * dscratch,
                                double * norms, const LoopParams & L, cudaStream_t st);
int iteration_block();

}  // namespace doma
