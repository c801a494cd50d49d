// accel.cuh -- per-cell kernels of the learned accelerator's correction step
// and of the reference-error stopping test (accel.cu).
//
// Multigroup source iteration with increment delta (phi_k = phi_{k-1} +
// delta) has the error e_k = ((I - K)^-1 - I) delta, K = L^-1 S.  With
// downscatter only, y = (I - K)^-1 delta = e + delta solves group by group:
//   y_g = A_g r_g,  r_g = delta_g + K_{g,g-1} y_{g-1},  A_g = (I - K_gg)^-1.
// The network stands in for (A_g - I): z_g = rms(r_g) * net(r_g / rms(r_g),
// ln sigma_t, ln(1 - c)), and K_{g,g-1} is taken locally as
// kappa_g = S[g][g-1] / sigma_t,g.  Then the correction is
//   Delta_g = z_g + kappa_g y_{g-1},   y_g = Delta_g + delta_g = z_g + r_g.
#pragma once

#include <cuda_bf16.h>

#include "iteration.cuh"

namespace doma {

// Feature scaling shared with the training data (doma_gb300/learned/data.py):
//   f_sigma = ln(sigma_t) / kFeatSigma
//   f_abs   = (ln(max(1 - c, kFeatAbsFloor)) - kFeatAbsShift) / kFeatAbsScale
constexpr float kFeatSigma = 0.8f;
constexpr float kFeatAbsFloor = 1e-6f;
constexpr float kFeatAbsShift = -4.6f;
constexpr float kFeatAbsScale = 1.5f;

// Per (group, cell): f_sigma, f_abs and kappa ([G][N] each).
doma_status accel_features(const IterArgs & a, float * fsig, float * fabs_, float * kappa,
                           cudaStream_t st);
// r = delta_g + kappa_g * y_prev (y_prev null for g = 0); *rms_out (device)
// gets sqrt(mean r^2) once the kernel finishes; partials: [grid][1] doubles.
doma_status accel_residual(const IterArgs & a, int g, const double * delta, const float * kappa,
                           const float * y_prev, float * r, double * partials, unsigned * ticket,
                           double * rms_out, cudaStream_t st);
// in[c] = (r / rms, f_sigma, f_abs, 0 ...) as bf16, 16 channels.
doma_status accel_input(size_t N, int g, const float * r, const double * rms, const float * fsig,
                        const float * fabs_, __nv_bfloat16 * in, cudaStream_t st);
// corr_g = rms * out + kappa_g * y_prev;  y_out = rms * out + r.
doma_status accel_correct(size_t N, int g, const float * out, const double * rms, const float * r,
                          const float * kappa, const float * y_prev, float * corr, float * y_out,
                          cudaStream_t st);
// q_h = src_scale / pi * sum_g (S[h][g] + chi_h nu_sigma_f_g) (delta_g + corr_g)
// (corr may be null).
doma_status accel_source(const IterArgs & a, int precision, const double * delta,
                         const float * corr, void * q, cudaStream_t st);
// sum over groups and cells of (phi - ref)^2 into *out (device) once done.
doma_status ref_error(const IterArgs & a, const double * ref, double * partials, unsigned * ticket,
                      double * out, cudaStream_t st);

}  // namespace doma
