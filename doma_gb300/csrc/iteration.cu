// iteration.cu -- per-cell kernels around the sweep: the multigroup source,
// the source-iteration epilogue (angular reduction, residual, increment
// update) and the Gauss-Seidel residual.
//
// Replaces updateMultigroupSource (src/TransportSolver3D.cpp:339-402, fixed-
// source terms), the thread reduction at the end of sweep (:610-621),
// computeScatteringResidual (:547-563), updateScatteringSource (:531-545) and
// computeMGFluxResidual (:318-337), with their 2D twins.  Sources and fluxes
// are double in every mode and use DOMA's association with unfused,
// correctly rounded operations.
//
// Norms are reduced deterministically without floating-point atomics: each
// thread owns a fixed set of cells (fixed grid, grid-stride), blocks reduce
// with a fixed shuffle tree, block partials go to a buffer, and the last block
// to finish (one integer ticket) sums the partials in block order.
#include <type_traits>

#include "common.cuh"
#include "iteration.cuh"
#include "loop_control.cuh"

namespace doma {
namespace {

__device__ __forceinline__ double dA(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dS(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dM(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dD(double a, double b) { return __ddiv_rn(a, b); }

constexpr int kBlock = 256;

// Fixed-order block sum of two values; the result is valid in thread 0.
__device__ __forceinline__ void block_sum2(double & a, double & b)
{
  __shared__ double sh[2][kBlock / 32];
  for (int off = 16; off > 0; off >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, off);
    b += __shfl_down_sync(0xffffffffu, b, off);
  }
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  if (lane == 0) {
    sh[0][warp] = a;
    sh[1][warp] = b;
  }
  __syncthreads();
  if (warp == 0) {
    a = lane < kBlock / 32 ? sh[0][lane] : 0.0;
    b = lane < kBlock / 32 ? sh[1][lane] : 0.0;
    for (int off = 16; off > 0; off >>= 1) {
      a += __shfl_down_sync(0xffffffffu, a, off);
      b += __shfl_down_sync(0xffffffffu, b, off);
    }
  }
  __syncthreads();
}

// Store this block's partial pair; the last block sums all pairs in block
// order into out[0..1] and re-arms the ticket.  Returns true in exactly one
// thread (thread 0 of the last block), after out[] is written.
__device__ __forceinline__ bool finish_norms(double a, double b, double * partials,
                                             unsigned * ticket, double * out)
{
  __shared__ bool last;
  block_sum2(a, b);
  if (threadIdx.x == 0) {
    partials[2 * blockIdx.x] = a;
    partials[2 * blockIdx.x + 1] = b;
    __threadfence();
    last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  double sa = 0.0, sb = 0.0;
  for (unsigned k = threadIdx.x; k < gridDim.x; k += blockDim.x) {
    sa += __ldcg(partials + 2 * k);
    sb += __ldcg(partials + 2 * k + 1);
  }
  block_sum2(sa, sb);
  if (threadIdx.x == 0) {
    out[0] = sa;
    out[1] = sb;
    *ticket = 0u;
    return true;
  }
  return false;
}

// updateMultigroupSource for group g (fixed source: external, in-scatter and
// prompt fission); also saves the previous iterate, zeroes phi_g and stages
// the sweep inputs (q and sigma_t of group g in the sweep's precision).
template <typename T>
__global__ void __launch_bounds__(kBlock) mg_source_kernel(const IterArgs A, int g, T * q_out,
                                                          T * sigt_out, const LoopParams L)
{
  if (L.graph) {
    // a failed group ends the solve: leave the flux of the last iterate alone
    const bool stop = L.ctl->failed != 0u;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      if (!stop) L.ctl->si_it = 0u;
      cudaGraphSetConditional(L.si_handle, stop ? 0u : 1u);
    }
    if (stop) return;
  }
  const size_t N = A.N;
  const int G = A.G;
  const double s = A.src_scale;
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < N;
       c += (size_t)gridDim.x * blockDim.x) {
    const unsigned m = A.mat[c];
    double q;
    if constexpr (std::is_same<T, float>::value) {
      // FP32 sweeps: one fused multiply-add per source group against the
      // per-material table (GB300's FP64 pipe makes DOMA's divisions costly)
      const double * cf = A.mgcoef + ((size_t)m * G + g) * G;
      q = A.srcq[(size_t)m * G + g];
      for (int gp = 0; gp < G; ++gp) q = __fma_rn(cf[gp], A.phi[(size_t)gp * N + c], q);
    } else {
      // DOMA's association (src/TransportSolver3D.cpp:350-380)
      q = A.source ? dD(dM(s, A.source[(size_t)m * G + g]), kPi) : 0.0;
      const bool fis = A.fis && A.fis[m];
      for (int gp = 0; gp < G; ++gp) {
        const double pg = A.phi[(size_t)gp * N + c];
        if (gp != g) q = dA(q, dD(dM(dM(s, A.scatter[((size_t)m * G + g) * G + gp]), pg), kPi));
        if (fis)
          q = dA(q, dD(dM(dM(dM(s, A.chi[(size_t)m * G + g]), A.nsf[(size_t)m * G + gp]), pg), kPi));
      }
    }
    q_out[c] = (T)q;
    sigt_out[c] = (T)A.total[(size_t)m * G + g];
    A.prev[(size_t)g * N + c] = A.phi[(size_t)g * N + c];
    A.phi[(size_t)g * N + c] = 0.0;
  }
}

// k-eigenvalue mode, updateMultigroupSourceEigen (src/TransportSolver3D.cpp:404-430):
// the in-scatter and fission / k terms are *added* to the current source,
// which still holds the previous group's last increment source (DOMA does not
// reset it there); the external source does not enter.  Same association as
// DOMA: ((s S) phi) / pi and ((((s chi) nu_sigma_f) phi) / pi) / k.
template <typename T>
__global__ void __launch_bounds__(kBlock) mg_source_eigen_kernel(const IterArgs A, int g, double k_arg,
                                                                 const double * k_dev, T * q,
                                                                 T * sigt_out, const LoopParams L)
{
  if (L.graph) {
    // a failed group ends the power iteration: leave the flux alone
    const bool stop = L.ctl->failed != 0u;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      if (!stop) L.ctl->si_it = 0u;
      cudaGraphSetConditional(L.si_handle, stop ? 0u : 1u);
    }
    if (stop) return;
  }
  const double k = k_dev ? *k_dev : k_arg;   // a captured graph reads k from the device
  const size_t N = A.N;
  const int G = A.G;
  const double s = A.src_scale;
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < N;
       c += (size_t)gridDim.x * blockDim.x) {
    const unsigned m = A.mat[c];
    double acc = (double)q[c];
    const bool fis = A.fis && A.fis[m];
    for (int gp = 0; gp < G; ++gp) {
      const double pg = A.phi[(size_t)gp * N + c];
      if (gp != g) acc = dA(acc, dD(dM(dM(s, A.scatter[((size_t)m * G + g) * G + gp]), pg), kPi));
      if (fis)
        acc = dA(acc, dD(dD(dM(dM(dM(s, A.chi[(size_t)m * G + g]), A.nsf[(size_t)m * G + gp]), pg),
                            kPi), k));
    }
    q[c] = (T)acc;
    sigt_out[c] = (T)A.total[(size_t)m * G + g];
    A.prev[(size_t)g * N + c] = A.phi[(size_t)g * N + c];
    A.phi[(size_t)g * N + c] = 0.0;
  }
}

// k-eigenvalue mode, initializeSolve (src/TransportSolver3D.cpp:512-518): the
// flux starts at 1 in every group, the previous iterate at 0.
__global__ void __launch_bounds__(kBlock) eigen_init_kernel(const IterArgs A)
{
  const size_t n = A.N * (size_t)A.G;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    A.phi[i] = 1.0;
    A.prev[i] = 0.0;
  }
}

// Transient mode, updateMultigroupSource with RunMode::Transient
// (src/TransportSolver3D.cpp:339-402; 2D: src/TransportSolver2D.cpp): the
// external source plus a source step that is on at t, then per source group
// g': in-scatter, prompt fission (scaled by 1 - sum_d beta when the material
// has delayed groups), the delayed-neutron source and the previous step's
// flux term.  The last two sit inside the g' loop in DOMA, so each is added G
// times; that is kept.  DOMA's association: (((s chi_d) C_d) lambda_d) / pi
// and ((((s phi_last) inv_v) / dt) / pi).  In 2D the cell solves use
// sigma_t + inv_v / dt (DiamondDifference2D.h:22-25); the 3D ones do not.
template <typename T>
__global__ void __launch_bounds__(kBlock) mg_source_transient_kernel(const IterArgs A,
                                                                     const TransientArgs X, int g,
                                                                     T * q_out, T * sigt_out,
                                                                     const LoopParams L)
{
  if (L.graph) {
    const bool stop = L.ctl->failed != 0u;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      if (!stop) L.ctl->si_it = 0u;
      cudaGraphSetConditional(L.si_handle, stop ? 0u : 1u);
    }
    if (stop) return;
  }
  const size_t N = A.N;
  const int G = A.G, D = X.D;
  const double s = A.src_scale;
  const double t = X.clock[0], dt = X.clock[1];
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < N;
       c += (size_t)gridDim.x * blockDim.x) {
    const unsigned m = A.mat[c];
    const size_t mg = (size_t)m * G + g;
    double q = A.source ? dD(dM(s, A.source[mg]), kPi) : 0.0;
    const unsigned st = X.step_type ? X.step_type[m] : 0u;
    if (st != 0u) {
      const double ins = X.step_insert[m], rem = X.step_remove[m];
      const bool on = st == 1u ? (ins <= t && t <= rem) : (st == 2u ? ins <= t : t <= rem);
      q = dA(q, on ? dD(dM(s, X.step_source[mg]), kPi) : 0.0);
    }
    const bool fis = A.fis && A.fis[m];
    const unsigned Dm = X.dg ? X.dg[m] : 0u;
    const double inv_v = X.inv_v[mg];
    const double last = X.last[(size_t)g * N + c];
    for (int gp = 0; gp < G; ++gp) {
      const double pg = A.phi[(size_t)gp * N + c];
      const size_t mgp = (size_t)m * G + gp;
      if (gp != g) q = dA(q, dD(dM(dM(s, A.scatter[mg * G + gp]), pg), kPi));
      if (fis && Dm == 0u) {
        q = dA(q, dD(dM(dM(dM(s, A.chi[mg]), A.nsf[mgp]), pg), kPi));
      } else if (fis) {
        double gb = 0.0;
        for (unsigned d = 0; d < Dm; ++d) gb = dA(gb, X.beta[mgp * D + d]);
        q = dA(q, dD(dM(dM(dM(dM(s, dS(1.0, gb)), A.chi[mg]), A.nsf[mgp]), pg), kPi));
      }
      for (unsigned d = 0; d < Dm; ++d)
        q = dA(q, dD(dM(dM(dM(s, X.chi_d[mg * D + d]), X.dnps[(size_t)d * N + c]),
                        X.lambda[(size_t)m * D + d]), kPi));
      q = dA(q, dD(dD(dM(dM(s, last), inv_v), dt), kPi));
    }
    q_out[c] = (T)q;
    sigt_out[c] = (T)(X.dims2 ? dA(A.total[mg], dD(inv_v, dt)) : A.total[mg]);
    A.prev[(size_t)g * N + c] = A.phi[(size_t)g * N + c];
    A.phi[(size_t)g * N + c] = 0.0;
  }
}

// stepDNPs (src/TransportSolver3D.cpp:236-260): production summed over groups
// in order, ((nu_sigma_f phi) beta); then (P / lambda) (1 - decay) + C decay.
__global__ void __launch_bounds__(kBlock) step_dnps_kernel(const IterArgs A, const TransientArgs X)
{
  const size_t N = A.N;
  const int G = A.G, D = X.D;
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < N;
       c += (size_t)gridDim.x * blockDim.x) {
    const unsigned m = A.mat[c];
    const unsigned Dm = X.dg ? X.dg[m] : 0u;
    for (unsigned d = 0; d < Dm; ++d) {
      double p = 0.0;
      for (int g = 0; g < G; ++g) {
        const size_t mg = (size_t)m * G + g;
        p = dA(p, dM(dM(A.nsf[mg], A.phi[(size_t)g * N + c]), X.beta[mg * D + d]));
      }
      const double lam = X.lambda[(size_t)m * D + d], dec = X.decay[(size_t)m * D + d];
      double & C = X.dnps[(size_t)d * N + c];
      C = dA(dM(dD(p, lam), dS(1.0, dec)), dM(C, dec));
    }
  }
}

// updateStepFluxes (src/TransportSolver3D.cpp:199-222) and t += dt.
__global__ void __launch_bounds__(kBlock) step_rollover_kernel(const IterArgs A, const TransientArgs X)
{
  const size_t n = A.N * (size_t)A.G;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    X.last[i] = A.phi[i];
    A.phi[i] = 0.0;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) X.clock[0] = dA(X.clock[0], X.clock[1]);
}

// The source-iteration epilogue for group g:
//   dphi = sum of the swept angular flux (exact: all ordinates in DOMA's
//          single-thread order; fp32: the (octant, ordinate group) partials in order)
//   diff += dphi^2 V, total += (phi + dphi)^2 V   (residual, before the update)
//   phi += dphi;  q = s * S_gg * dphi / pi       (the next increment's source)
template <typename T, bool EXACT>
__global__ void __launch_bounds__(kBlock) si_epilogue_kernel(const IterArgs A, int g, T * q_out,
                                                            double * norms, const LoopParams L)
{
  const size_t N = A.N;
  const int G = A.G;
  double diff = 0.0, tot = 0.0;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  // One cell's update after its increment d: phi, the norms (accumulated in
  // the thread's cell order), the next source.
  auto finish = [&](size_t c, double d) {
    const double V = A.vol[c];
    double * ph = A.phi + (size_t)g * N + c;
    const double t = dA(*ph, d);
    *ph = t;
    const unsigned m = A.mat[c];
    if (EXACT) {
      // DOMA's association (src/TransportSolver3D.cpp:537-539, :553-556)
      diff = dA(diff, dM(dM(d, d), V));
      tot = dA(tot, dM(dM(t, t), V));
      q_out[c] = (T)dD(dM(dM(A.src_scale, A.scatter[((size_t)m * G + g) * G + g]), d), kPi);
    } else {
      // FP32 sweeps: the FP64 pipe is the limit here (GB300 issues about two
      // FP64 operations per SM per clock), so fused norms and one multiply
      // by s * S_gg / pi replace DOMA's mul-mul-divide
      diff = __fma_rn(dM(d, d), V, diff);
      tot = __fma_rn(dM(t, t), V, tot);
      q_out[c] = (T)dM(d, A.qcoef[(size_t)m * G + g]);
    }
  };
  if constexpr (EXACT) {
    for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < N; c += stride) {
      double d = 0.0;
      const double * w = A.wpsi + c * (size_t)A.D;
      for (int k = 0; k < A.D; ++k) d = dA(d, w[k]);
      finish(c, d);
    }
  } else {
    // two of the thread's cells per pass: their slot sums are independent
    // chains, interleaved; the cells still finish in order
    for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < N; c += 2 * stride) {
      const size_t c2 = c + stride;
      const bool two = c2 < N;
      PartialSum sa, sb;
      for (int o = 0; o < 8; ++o)
        if (A.oct_mask & (1 << o))
          for (int og = 0; og < A.ngroups; ++og) {
            const float2 * part = A.octphi + ((size_t)o * A.ngroups + og) * N;
            sa.add(part[c]);
            if (two) sb.add(part[c2]);
          }
      finish(c, sa.value());
      if (two) finish(c2, sb.value());
    }
  }
  if (finish_norms(diff, tot, A.partials, A.ticket, norms) && L.graph) {
    // sourceIteration's loop test (src/TransportSolver3D.cpp:481), on the device
    si_loop_control(L, norms);
  }
}

// computeMGFluxResidual: sums over cells and groups of (phi - prev)^2 V and phi^2 V.
__global__ void __launch_bounds__(kBlock) mg_residual_kernel(const IterArgs A, double * norms,
                                                            const LoopParams L)
{
  if (L.graph && L.ctl->failed != 0u) {
    if (blockIdx.x == 0 && threadIdx.x == 0) cudaGraphSetConditional(L.mg_handle, 0u);
    return;
  }
  const size_t N = A.N;
  double diff = 0.0, tot = 0.0;
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < N;
       c += (size_t)gridDim.x * blockDim.x) {
    const double V = A.vol[c];
    for (int g = 0; g < A.G; ++g) {
      const double a = A.phi[(size_t)g * N + c];
      const double d = dS(a, A.prev[(size_t)g * N + c]);
      diff = dA(diff, dM(dM(d, d), V));
      tot = dA(tot, dM(dM(a, a), V));
    }
  }
  if (finish_norms(diff, tot, A.partials, A.ticket, norms) && L.graph) {
    // solveFixedSource's loop test (src/TransportSolver3D.cpp:295), on the device
    LoopCtl * C = L.ctl;
    const double res = norm_ratio(norms[0], norms[1]);
    if (C->mg_it < L.mg_cap) L.mg_hist[C->mg_it] = res;
    const unsigned mg = ++C->mg_it;
    C->mg_res = res;
    const bool ok = finite2(norms[0], norms[1]);
    if (!ok) C->failed = DOMA_NUMERIC_ERROR;
    const bool more = ok && mg < L.mg_max_it && L.mg_tol < res && L.G > 1;
    cudaGraphSetConditional(L.mg_handle, more ? 1u : 0u);
  }
}

// Multigroup mode, start of the solve: phi = 0, the first increment's source
// is the external source of every group, and sigma_t of every group is staged.
template <typename T>
__global__ void __launch_bounds__(kBlock) mgi_init_kernel(const IterArgs A, T * q, T * sigt)
{
  const size_t N = A.N;
  const int G = A.G;
  const double s = A.src_scale;
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < N;
       c += (size_t)gridDim.x * blockDim.x) {
    const unsigned m = A.mat[c];
    for (int g = 0; g < G; ++g) {
      q[(size_t)g * N + c] = (T)(A.source ? dD(dM(s, A.source[(size_t)m * G + g]), kPi) : 0.0);
      sigt[(size_t)g * N + c] = (T)A.total[(size_t)m * G + g];
      A.phi[(size_t)g * N + c] = 0.0;
    }
  }
}

// Multigroup mode, after an all-group sweep:
//   d_g  = sum of group g's (octant, ordinate group) partials, in slot order
//   diff += d_g^2 V, total += (phi_g + d_g)^2 V over all groups
//   phi_g += d_g
//   q_h  = s / pi * sum_g (S[h][g] + chi[h] nu_sigma_f[g]) d_g   (next increment)
// The G x G contraction per cell is small (G <= 16 in every workload here)
// and memory-bound, so it stays on the CUDA cores.
// One cell of the multigroup epilogue (shared by the single-problem and the
// batched kernels): group increments from the partials, residual sums, flux
// update, next increment's source.
template <typename T>
__device__ __forceinline__ void mgi_cell(const IterArgs & A, size_t c, T * q, double * dscratch,
                                         double & diff, double & tot)
{
  const size_t N = A.N;
  const int G = A.G;
  const int per_group = 8 * A.ngroups;
  const double V = A.vol[c];
  for (int g = 0; g < G; ++g) {
    double d = 0.0;
    if (A.exact) {
      // every ordinate in DOMA's single-thread order (octant, then ordinate)
      const double * w = A.wpsi + ((size_t)g * N + c) * (size_t)A.D;
      for (int k = 0; k < A.D; ++k) d = dA(d, w[k]);
    } else {
      PartialSum ps;
      for (int o = 0; o < 8; ++o)
        if (A.oct_mask & (1 << o))
          for (int og = 0; og < A.ngroups; ++og)
            ps.add(A.octphi[((size_t)g * per_group + (size_t)o * A.ngroups + og) * N + c]);
      d = ps.value();
    }
    double * ph = A.phi + (size_t)g * N + c;
    const double t = dA(*ph, d);
    if (A.corr) d = dA(d, -(double)A.corr[(size_t)g * N + c]);
    diff = dA(diff, dM(dM(d, d), V));
    tot = dA(tot, dM(dM(t, t), V));
    *ph = t;
    dscratch[(size_t)g * N + c] = d;
  }
  const unsigned m = A.mat[c];
  const bool fis = A.fis && A.fis[m];
  for (int h = 0; h < G; ++h) {
    double acc = 0.0;
    const double * Sh = A.scatter + ((size_t)m * G + h) * G;
    const double chi = fis ? A.chi[(size_t)m * G + h] : 0.0;
    for (int g = 0; g < G; ++g) {
      double k = Sh[g];
      if (fis) k = dA(k, dM(chi, A.nsf[(size_t)m * G + g]));
      acc = dA(acc, dM(k, dscratch[(size_t)g * N + c]));
    }
    q[(size_t)h * N + c] = (T)dD(dM(A.src_scale, acc), kPi);
  }
}

template <typename T>
__global__ void __launch_bounds__(kBlock) mgi_epilogue_kernel(const IterArgs A, T * q,
                                                             double * dscratch, double * norms,
                                                             const LoopParams L)
{
  double diff = 0.0, tot = 0.0;
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < A.N;
       c += (size_t)gridDim.x * blockDim.x)
    mgi_cell(A, c, q, dscratch, diff, tot);
  if (finish_norms(diff, tot, A.partials, A.ticket, norms) && L.graph) {
    si_loop_control(L, norms);
  }
}

// ---- batched multigroup solve ---------------------------------------------

// Epilogue of every active problem of a batch: block b works on problem
// block_prob[b] (its blocks are contiguous), writes its partial norms to that
// problem's partials; batch_finalize_kernel reduces them.
template <typename T>
__global__ void __launch_bounds__(kBlock) batch_epilogue_kernel(const BatchSlot * slots,
                                                               const int * block_prob,
                                                               const BatchLoop * loops)
{
  const int p = block_prob[blockIdx.x];
  if (!loops[p].active) return;
  const BatchSlot & S = slots[p];
  const int lb = blockIdx.x - S.block0;
  double diff = 0.0, tot = 0.0;
  for (size_t c = (size_t)lb * blockDim.x + threadIdx.x; c < S.it.N;
       c += (size_t)S.blocks * blockDim.x)
    mgi_cell(S.it, c, static_cast<T *>(S.q), S.dscratch, diff, tot);
  block_sum2(diff, tot);
  if (threadIdx.x == 0) {
    S.it.partials[2 * lb] = diff;
    S.it.partials[2 * lb + 1] = tot;
  }
}

// One block per problem: sum the problem's block partials in block order,
// then DOMA-style loop test on its relative increment norm.
__global__ void __launch_bounds__(kBlock) batch_finalize_kernel(const BatchSlot * slots,
                                                               BatchLoop * loops, double tol,
                                                               unsigned max_it,
                                                               unsigned * still_active)
{
  const int p = blockIdx.x;
  if (!loops[p].active) return;
  const BatchSlot & S = slots[p];
  double a = 0.0, b = 0.0;
  for (int k = threadIdx.x; k < S.blocks; k += blockDim.x) {
    a += S.it.partials[2 * k];
    b += S.it.partials[2 * k + 1];
  }
  block_sum2(a, b);
  if (threadIdx.x == 0) {
    BatchLoop & L = loops[p];
    const double res = norm_ratio(a, b);
    L.it += 1;
    L.res = res;
    const bool ok = finite2(a, b);
    const bool more = ok && L.it < max_it && tol < res;
    if (!more) {
      L.active = 0u;
      L.status = !ok ? DOMA_NUMERIC_ERROR : (L.it < max_it ? DOMA_OK : DOMA_NOT_CONVERGED);
    } else {
      atomicAdd(still_active, 1u);
    }
  }
}

// End of one batched iteration: count it, clear the active counter for the
// next one and decide whether the graph's loop goes on.  One thread.
__global__ void batch_continue_kernel(unsigned * still_active, const int * error, unsigned * iters,
                                      unsigned max_iters, unsigned long long handle)
{
  const unsigned n = *still_active;
  *still_active = 0u;
  const unsigned it = ++*iters;
  const bool more = n > 0u && *error == 0 && it <= max_iters;
  cudaGraphSetConditional(handle, more ? 1u : 0u);
}

}  // namespace

doma_status launch_batch_continue(unsigned * still_active, const int * error, unsigned * iters,
                                  unsigned max_iters, unsigned long long handle, cudaStream_t st)
{
  batch_continue_kernel<<<1, 1, 0, st>>>(still_active, error, iters, max_iters, handle);
  DOMA_CUDA_TRY(cudaGetLastError());
  return DOMA_OK;
}

doma_status launch_batch_epilogue(const BatchSlot * slots, const int * block_prob, int blocks,
                                  const BatchLoop * loops, int precision, cudaStream_t st)
{
  if (precision == DOMA_PREC_FP64)
    batch_epilogue_kernel<double><<<blocks, kBlock, 0, st>>>(slots, block_prob, loops);
  else
    batch_epilogue_kernel<float><<<blocks, kBlock, 0, st>>>(slots, block_prob, loops);
  DOMA_CUDA_TRY(cudaGetLastError());
  return DOMA_OK;
}

doma_status launch_batch_finalize(const BatchSlot * slots, BatchLoop * loops, int count,
                                  double tol, unsigned max_it, unsigned * still_active,
                                  cudaStream_t st)
{
  batch_finalize_kernel<<<count, kBlock, 0, st>>>(slots, loops, tol, max_it, still_active);
  DOMA_CUDA_TRY(cudaGetLastError());
  return DOMA_OK;
}

doma_status launch_mgi_init(const IterArgs & a, int precision, void * q, void * sigt,
                            cudaStream_t st)
{
  if (precision == DOMA_PREC_FP64)
    mgi_init_kernel<double><<<a.grid, kBlock, 0, st>>>(a, (double *)q, (double *)sigt);
  else
    mgi_init_kernel<float><<<a.grid, kBlock, 0, st>>>(a, (float *)q, (float *)sigt);
  DOMA_CUDA_TRY(cudaGetLastError());
  return DOMA_OK;
}

doma_status launch_mgi_epilogue(const IterArgs & a, int precision, void * q, double * dscratch,
                                double * norms, const LoopParams & L, cudaStream_t st)
{
  if (precision == DOMA_PREC_FP64)
    mgi_epilogue_kernel<double><<<a.grid, kBlock, 0, st>>>(a, (double *)q, dscratch, norms, L);
  else
    mgi_epilogue_kernel<float><<<a.grid, kBlock, 0, st>>>(a, (float *)q, dscratch, norms, L);
  DOMA_CUDA_TRY(cudaGetLastError());
  return DOMA_OK;
}

doma_status launch_mg_source(const IterArgs & a, int g, int precision, void * q, void * sigt,
                             const LoopParams & L, cudaStream_t st)
{
  if (precision == DOMA_PREC_FP64)
    mg_source_kernel<double><<<a.grid, kBlock, 0, st>>>(a, g, (double *)q, (double *)sigt, L);
  else
    mg_source_kernel<float><<<a.grid, kBlock, 0, st>>>(a, g, (float *)q, (float *)sigt, L);
  DOMA_CUDA_TRY(cudaGetLastError());
  return DOMA_OK;
}

doma_status launch_mg_source_eigen(const IterArgs & a, int g, int precision, double k,
                                   const double * k_dev, void * q, void * sigt,
                                   const LoopParams & L, cudaStream_t st)
{
  if (precision == DOMA_PREC_FP64)
    mg_source_eigen_kernel<double><<<a.grid, kBlock, 0, st>>>(a, g, k, k_dev, (double *)q,
                                                             (double *)sigt, L);
  else
    mg_source_eigen_kernel<float><<<a.grid, kBlock, 0, st>>>(a, g, k, k_dev, (float *)q,
                                                            (float *)sigt, L);
  DOMA_CUDA_TRY(cudaGetLastError());
  return DOMA_OK;
}

doma_status launch_eigen_init(const IterArgs & a, cudaStream_t st)
{
  eigen_init_kernel<<<a.grid, kBlock, 0, st>>>(a);
  DOMA_CUDA_TRY(cudaGetLastError());
  return DOMA_OK;
}

doma_status launch_mg_source_transient(const IterArgs & a, const TransientArgs & x, int g,
                                       int precision, void * q, void * sigt,
                                       const LoopParams & L, cudaStream_t st)
{
  if (precision == DOMA_PREC_FP64)
    mg_source_transient_kernel<double><<<a.grid, kBlock, 0, st>>>(a, x, g, (double *)q,
                                                                  (double *)sigt, L);
  else
    mg_source_transient_kernel<float><<<a.grid, kBlock, 0, st>>>(a, x, g, (float *)q,
                                                                 (float *)sigt, L);
  DOMA_CUDA_TRY(cudaGetLastError());
  return DOMA_OK;
}

doma_status launch_step_dnps(const IterArgs & a, const TransientArgs & x, cudaStream_t st)
{
  step_dnps_kernel<<<a.grid, kBlock, 0, st>>>(a, x);
  DOMA_CUDA_TRY(cudaGetLastError());
  return DOMA_OK;
}

doma_status launch_step_rollover(const IterArgs & a, const TransientArgs & x, cudaStream_t st)
{
  step_rollover_kernel<<<a.grid, kBlock, 0, st>>>(a, x);
  DOMA_CUDA_TRY(cudaGetLastError());
  return DOMA_OK;
}

doma_status launch_si_epilogue(const IterArgs & a, int g, int precision, void * q,
                               double * norms, const LoopParams & L, cudaStream_t st)
{
  if (precision == DOMA_PREC_FP64)
    si_epilogue_kernel<double, true><<<a.grid, kBlock, 0, st>>>(a, g, (double *)q, norms, L);
  else
    si_epilogue_kernel<float, false><<<a.epi_grid, kBlock, 0, st>>>(a, g, (float *)q, norms, L);
  DOMA_CUDA_TRY(cudaGetLastError());
  return DOMA_OK;
}

doma_status launch_mg_residual(const IterArgs & a, double * norms, const LoopParams & L,
                               cudaStream_t st)
{
  mg_residual_kernel<<<a.grid, kBlock, 0, st>>>(a, norms, L);
  DOMA_CUDA_TRY(cudaGetLastError());
  return DOMA_OK;
}

int iteration_block() { return kBlock; }

}  // namespace doma
