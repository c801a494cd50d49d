// conv.cuh -- BF16 3D convolution kernels of the learned source-iteration
// accelerator (conv.cu): 3x3x3, stride 1, zero padding 1, channels-last
// tensors [batch][z][y][x][channel], FP32 accumulation.
//
// Weights are stored per tap, output-channel major: w[tap][cout][cin], tap =
// (dz+1)*9 + (dy+1)*3 + (dx+1).  The data gradient of a convolution is the
// same convolution run with the taps mirrored and the channel roles swapped
// (wt[tap][cin][cout] = w[26 - tap][cout][cin]).
#pragma once

#include <cuda_bf16.h>

#include "common.cuh"

namespace doma {

struct ConvShape {
  int batch = 0, nz = 0, ny = 0, nx = 0;
  size_t voxels() const { return (size_t)batch * nz * ny * nx; }
};

// Device scratch (FP32) that lets the tensor-memory convolution split its
// reduction on shapes with few voxels; without it the reduction is not split.
struct ConvScratch {
  float * p = nullptr;
  size_t floats = 0;
};

// y = act(conv(x, w) + bias); bias may be null; relu selects the activation.
// cout in {32, 64, 128, 256}; cin in {16, 32, 64, 128, 256}.
doma_status conv3_forward(const ConvShape & s, const __nv_bfloat16 * x, int cin,
                          const __nv_bfloat16 * w, const float * bias, int cout, bool relu,
                          __nv_bfloat16 * y, cudaStream_t st, ConvScratch scratch = {});

// The tensor-memory (tcgen05 + TMA) variant of conv3_forward (conv_tc.cu),
// for shapes whose 128-voxel boxes tile the volume exactly; conv3_forward
// uses it for those unless DOMA_CONV_PATH=mma.  conv3_tc_error reads the
// flag its bounded waits set when one gave up; conv3_tc_error_reset clears it
// on a stream (each U-Net forward pass and each C-ABI convolution starts with
// a clear flag, so the flag describes the latest pass).
// conv3_tc_split_scratch is the scratch (floats) with which the shape's
// reduction is split as far as the kernel would split it.
bool conv3_tc_supported(const ConvShape & s, int cin, int cout);
size_t conv3_tc_split_scratch(const ConvShape & s, int cin, int cout);
doma_status conv3_forward_tc(const ConvShape & s, const __nv_bfloat16 * x, int cin,
                             const __nv_bfloat16 * w, const float * bias, int cout, bool relu,
                             __nv_bfloat16 * y, cudaStream_t st, ConvScratch scratch = {});
doma_status conv3_forward_mma(const ConvShape & s, const __nv_bfloat16 * x, int cin,
                              const __nv_bfloat16 * w, const float * bias, int cout, bool relu,
                              __nv_bfloat16 * y, cudaStream_t st);
doma_status conv3_tc_error(int * flag);
// Weight-gradient partials on the tensor cores (conv_tc.cu): for shapes the
// tensor-memory forward supports and cin in {16, 32, 64, 128, 256}, writes
// FP32 partials [splits][27][cout][cin] (at most max_splits) and *splits_out.
bool conv3_wgrad_tc_supported(const ConvShape & s, int cin, int cout);
int conv3_wgrad_tc_splits(const ConvShape & s, int cin, int cout);  // 0 if unsupported
doma_status conv3_wgrad_tc(const ConvShape & s, const __nv_bfloat16 * x, int cin,
                           const __nv_bfloat16 * dz, int cout, float * partial, int max_splits,
                           int * splits_out, cudaStream_t st);
doma_status conv3_tc_error_reset(cudaStream_t st);

// Weight gradient: dw[tap][cout][cin] = sum over voxels m of
// dz[m][cout] * x[m + offset(tap)][cin], reduced over voxel splits in a fixed
// order (deterministic).  partial: scratch of conv3_wgrad_scratch() floats.
// path: DOMA_CONV_AUTO (tensor cores where supported), DOMA_CONV_MMA or
// DOMA_CONV_TENSOR_MEMORY; DOMA_CONV_PATH=mma in the environment forces MMA.
size_t conv3_wgrad_scratch(const ConvShape & s, int cin, int cout);
doma_status conv3_wgrad(const ConvShape & s, const __nv_bfloat16 * x, int cin,
                        const __nv_bfloat16 * dz, int cout, float * partial, float * dw,
                        cudaStream_t st, int path = DOMA_CONV_AUTO);

// Elementwise and resampling pieces of the U-Net (all channels-last, bf16).
// pool: 2x2x2 average; up: nearest-neighbour 2x; sumpool: adjoint of up.
doma_status avgpool2(const ConvShape & fine, int c, const __nv_bfloat16 * x, __nv_bfloat16 * y,
                     cudaStream_t st);
// u = relu(up(coarse) + skip)
doma_status up_add_relu(const ConvShape & fine, int c, const __nv_bfloat16 * coarse,
                        const __nv_bfloat16 * skip, __nv_bfloat16 * u, cudaStream_t st);
// g *= (y > 0)
doma_status relu_mask(size_t count, __nv_bfloat16 * g, const __nv_bfloat16 * y, cudaStream_t st);
// out = (up(g_pool) / 8 + g_skip) * (y > 0)   (fine resolution)
doma_status pool_back_add_mask(const ConvShape & fine, int c, const __nv_bfloat16 * g_pool,
                               const __nv_bfloat16 * g_skip, const __nv_bfloat16 * y,
                               __nv_bfloat16 * out, cudaStream_t st);
// coarse = sum of the 8 children of fine
doma_status sumpool2(const ConvShape & fine, int c, const __nv_bfloat16 * x, __nv_bfloat16 * y,
                     cudaStream_t st);
// Bias gradient db[c] = sum over voxels of g[m][c] (fixed-order reduction);
// partial: scratch of bias_grad_scratch(c) floats.
size_t bias_grad_scratch(int c);
doma_status bias_grad(size_t voxels, int c, const __nv_bfloat16 * g, float * partial, float * db,
                      cudaStream_t st);
// Output head: out[m] = b + sum_c w[c] x[m][c]  (FP32 result)
doma_status head_forward(size_t voxels, int c, const __nv_bfloat16 * x, const float * w,
                         const float * b, float * out, cudaStream_t st);
// Mean-square loss and the head's backward pass:
//   r = out - target; loss = sum r^2 / voxels (double, in *loss)
//   dx[m][c] = (2 r[m] / voxels) w[c] * (x[m][c] > 0)   (x is the head input, a relu output)
//   dw[c] = sum_m (2 r / voxels) x[m][c], db = sum_m 2 r / voxels
// partial: scratch of head_backward_scratch(c) doubles.  With sample_weight
// (device, one per sample of per_sample voxels) every voxel's r is weighted by
// its sample's weight: loss = sum w r^2 / voxels and the gradients follow.
size_t head_backward_scratch(int c);
doma_status head_backward(size_t voxels, int c, const __nv_bfloat16 * x, const float * w,
                          const float * out, const float * target, __nv_bfloat16 * dx, float * dw,
                          float * db, double * partial, double * loss, cudaStream_t st,
                          const float * sample_weight = nullptr, size_t per_sample = 1);
// FP32 master weights -> bf16 forward (w) and mirrored/transposed (wt) copies.
doma_status publish_weights(const float * w32, int cin, int cout, __nv_bfloat16 * w,
                            __nv_bfloat16 * wt, cudaStream_t st);
// Adam on a flat parameter array (bias-corrected; step is 1-based).
doma_status adam_update(size_t count, float * p, const float * g, float * m, float * v, float lr,
                        float beta1, float beta2, float eps, int step, cudaStream_t st);

}  // namespace doma
