// accel.cu -- per-cell kernels of the learned accelerator's correction step
// and of the reference-error test (see accel.cuh for the algebra).
// Reductions are deterministic: block partials in a fixed block order.
#include "accel.cuh"

#include <algorithm>
#include <cmath>

namespace doma {

namespace {

constexpr int kB = 256;

__device__ double block_sum(double v)
{
  __shared__ double sh[kB / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += sh[k];
  __syncthreads();
  return t;  // thread 0
}

// Block partial, then the last block to finish adds the partials in block
// order: *out = sum (or sqrt(sum / count) when rms), and resets the ticket.
__device__ void finish(double v, double * partials, unsigned * ticket, double * out, bool rms,
                       double count)
{
  __shared__ bool last;
  const double b = block_sum(v);
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = b;
    __threadfence();
    last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (last && threadIdx.x == 0) {
    __threadfence();
    double t = 0.0;
    for (unsigned k = 0; k < gridDim.x; ++k) t += ((volatile double *)partials)[k];
    *out = rms ? sqrt(t / count) : t;
    *ticket = 0u;
  }
}

__global__ void __launch_bounds__(kB) features_kernel(const IterArgs A, float * fsig, float * fabs_,
                                                      float * kappa)
{
  const size_t N = A.N;
  const int G = A.G;
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < N;
       c += (size_t)gridDim.x * blockDim.x) {
    const unsigned m = A.mat[c];
    for (int g = 0; g < G; ++g) {
      const double st = A.total[(size_t)m * G + g];
      const double * Sg = A.scatter + ((size_t)m * G + g) * G;
      const double cc = Sg[g] / st;
      fsig[(size_t)g * N + c] = (float)(log(st) / (double)kFeatSigma);
      const double a = fmax(1.0 - cc, (double)kFeatAbsFloor);
      fabs_[(size_t)g * N + c] = (float)((log(a) - (double)kFeatAbsShift) / (double)kFeatAbsScale);
      kappa[(size_t)g * N + c] = g > 0 ? (float)(Sg[g - 1] / st) : 0.0f;
    }
  }
}

__global__ void __launch_bounds__(kB) residual_kernel(const size_t N, const int g,
                                                      const double * delta, const float * kappa,
                                                      const float * y_prev, float * r,
                                                      double * partials, unsigned * ticket,
                                                      double * rms_out)
{
  double s = 0.0;
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < N;
       c += (size_t)gridDim.x * blockDim.x) {
    float v = (float)delta[(size_t)g * N + c];
    if (y_prev) v += kappa[(size_t)g * N + c] * y_prev[c];
    r[c] = v;
    s += (double)v * v;
  }
  finish(s, partials, ticket, rms_out, true, (double)N);
}

__global__ void __launch_bounds__(kB) input_kernel(const size_t N, const int g, const float * r,
                                                   const double * rms, const float * fsig,
                                                   const float * fabs_, __nv_bfloat16 * in)
{
  const double s = *rms;
  const float inv = s > 0.0 ? (float)(1.0 / s) : 0.0f;
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < N;
       c += (size_t)gridDim.x * blockDim.x) {
    uint4 lo = make_uint4(0u, 0u, 0u, 0u), hi = make_uint4(0u, 0u, 0u, 0u);
    __nv_bfloat162 * h = reinterpret_cast<__nv_bfloat162 *>(&lo);
    h[0] = __floats2bfloat162_rn(r[c] * inv, fsig[(size_t)g * N + c]);
    h[1] = __floats2bfloat162_rn(fabs_[(size_t)g * N + c], 0.0f);
    uint4 * dst = reinterpret_cast<uint4 *>(in + c * 16);
    dst[0] = lo;
    dst[1] = hi;
  }
}

__global__ void __launch_bounds__(kB) correct_kernel(const size_t N, const int g, const float * out,
                                                     const double * rms, const float * r,
                                                     const float * kappa, const float * y_prev,
                                                     float * corr, float * y_out)
{
  const float s = (float)*rms;
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < N;
       c += (size_t)gridDim.x * blockDim.x) {
    const float z = s * out[c];
    const float kp = y_prev ? kappa[(size_t)g * N + c] * y_prev[c] : 0.0f;
    corr[(size_t)g * N + c] = z + kp;
    y_out[c] = z + r[c];
  }
}

template <typename T>
__global__ void __launch_bounds__(kB) source_kernel(const IterArgs A, const double * delta,
                                                    const float * corr, T * q)
{
  const size_t N = A.N;
  const int G = A.G;
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < N;
       c += (size_t)gridDim.x * blockDim.x) {
    const unsigned m = A.mat[c];
    const bool fis = A.fis && A.fis[m];
    for (int h = 0; h < G; ++h) {
      const double * Sh = A.scatter + ((size_t)m * G + h) * G;
      const double chi = fis ? A.chi[(size_t)m * G + h] : 0.0;
      double acc = 0.0;
      for (int g = 0; g < G; ++g) {
        double k = Sh[g];
        if (fis) k += chi * A.nsf[(size_t)m * G + g];
        double d = delta[(size_t)g * N + c];
        if (corr) d += (double)corr[(size_t)g * N + c];
        acc += k * d;
      }
      q[(size_t)h * N + c] = (T)((A.src_scale * acc) / kPi);
    }
  }
}

__global__ void __launch_bounds__(kB) ref_error_kernel(const IterArgs A, const double * ref,
                                                       double * partials, unsigned * ticket,
                                                       double * out)
{
  const size_t NG = A.N * (size_t)A.G;
  double s = 0.0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < NG;
       i += (size_t)gridDim.x * blockDim.x) {
    const double d = A.phi[i] - ref[i];
    s += d * d;
  }
  finish(s, partials, ticket, out, false, 1.0);
}

}  // namespace

doma_status accel_features(const IterArgs & a, float * fsig, float * fabs_, float * kappa,
                           cudaStream_t st)
{
  features_kernel<<<a.grid, kB, 0, st>>>(a, fsig, fabs_, kappa);
  DOMA_CUDA_TRY(cudaGetLastError());
  return DOMA_OK;
}

doma_status accel_residual(const IterArgs & a, int g, const double * delta, const float * kappa,
                           const float * y_prev, float * r, double * partials, unsigned * ticket,
                           double * rms_out, cudaStream_t st)
{
  residual_kernel<<<a.grid, kB, 0, st>>>(a.N, g, delta, kappa, y_prev, r, partials, ticket,
                                         rms_out);
  DOMA_CUDA_TRY(cudaGetLastError());
  return DOMA_OK;
}

doma_status accel_input(size_t N, int g, const float * r, const double * rms, const float * fsig,
                        const float * fabs_, __nv_bfloat16 * in, cudaStream_t st)
{
  const int grid = (int)std::min<size_t>((N + kB - 1) / kB, 152 * 8);
  input_kernel<<<grid, kB, 0, st>>>(N, g, r, rms, fsig, fabs_, in);
  DOMA_CUDA_TRY(cudaGetLastError());
  return DOMA_OK;
}

doma_status accel_correct(size_t N, int g, const float * out, const double * rms, const float * r,
                          const float * kappa, const float * y_prev, float * corr, float * y_out,
                          cudaStream_t st)
{
  const int grid = (int)std::min<size_t>((N + kB - 1) / kB, 152 * 8);
  correct_kernel<<<grid, kB, 0, st>>>(N, g, out, rms, r, kappa, y_prev, corr, y_out);
  DOMA_CUDA_TRY(cudaGetLastError());
  return DOMA_OK;
}

doma_status accel_source(const IterArgs & a, int precision, const double * delta,
                         const float * corr, void * q, cudaStream_t st)
{
  if (precision == DOMA_PREC_FP64)
    source_kernel<double><<<a.grid, kB, 0, st>>>(a, delta, corr, static_cast<double *>(q));
  else
    source_kernel<float><<<a.grid, kB, 0, st>>>(a, delta, corr, static_cast<float *>(q));
  DOMA_CUDA_TRY(cudaGetLastError());
  return DOMA_OK;
}

doma_status ref_error(const IterArgs & a, const double * ref, double * partials, unsigned * ticket,
                      double * out, cudaStream_t st)
{
  ref_error_kernel<<<a.grid, kB, 0, st>>>(a, ref, partials, ticket, out);
  DOMA_CUDA_TRY(cudaGetLastError());
  return DOMA_OK;
}

}  // namespace doma
