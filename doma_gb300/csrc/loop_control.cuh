// loop_control.cuh -- the source-iteration loop test on the device, shared by
// the stand-alone epilogue kernel (iteration.cu) and the sweep kernel's fused
// epilogue (sweep.cu).
#pragma once

#include "iteration.cuh"

namespace doma {

// DOMA's relative norm (src/TransportSolver3D.cpp:562): sqrt(diff)/sqrt(total),
// or 0 when total <= 1e-8.  IEEE sqrt and division, the same bits as the host.
__device__ __forceinline__ double norm_ratio(double diff, double tot)
{
  return tot > 1e-8 ? __ddiv_rn(__dsqrt_rn(diff), __dsqrt_rn(tot)) : 0.0;
}

__device__ __forceinline__ bool finite2(double a, double b)
{
  return isfinite(a) && isfinite(b);
}

// sourceIteration's loop test (src/TransportSolver3D.cpp:481) after one
// source iteration whose norms are in norms[0..1]: counts the iteration,
// records the residual and, when the loop ends, the pair's count and the
// reason it stopped; sets the SI WHILE node's condition.  One thread, once per
// source iteration, in a graph-driven solve (L.graph != 0).
__device__ __forceinline__ void si_loop_control(const LoopParams & L, const double * norms)
{
  LoopCtl * C = L.ctl;
  const double res = norm_ratio(norms[0], norms[1]);
  const unsigned it = ++C->si_it;
  ++C->sweeps;
  if (L.si_hist && C->hist_len < L.hist_cap) L.si_hist[C->hist_len] = res;
  ++C->hist_len;
  C->si_res = res;
  const bool ok = finite2(norms[0], norms[1]) && C->error == 0;
  const bool more = ok && it < L.fs_max_it && L.fs_tol < res;
  if (!more) {
    if (C->pairs < L.pair_cap) {
      L.pair_counts[C->pairs] = it;
      L.pair_res[C->pairs] = res;
    }
    ++C->pairs;
    if (C->error != 0) C->failed = DOMA_DEVICE_WAIT_TIMEOUT;
    else if (!ok) C->failed = DOMA_NUMERIC_ERROR;
    else if (!(it < L.fs_max_it)) C->failed = DOMA_NOT_CONVERGED;
  }
  cudaGraphSetConditional(L.si_handle, more ? 1u : 0u);
}

}  // namespace doma
