// unet.cuh -- the learned accelerator's network: a 3D convolutional U-Net
// (4 levels, 32/64/128/256 channels) in BF16 with FP32 accumulation, run and
// trained entirely by this library's kernels (conv.cu).
//
//   level 0: e0a = relu(conv(x)),  e0 = relu(conv(e0a))            32 ch
//   level l: p_l = avgpool(e_{l-1}), e_la = relu(conv(p_l)),
//            e_l = relu(conv(e_la))                               32 * 2^l ch
//   up:      c_l = conv(d_{l+1} or e3), u_l = relu(up(c_l) + e_l),
//            d_l = relu(conv(u_l))                                 (l = 2, 1, 0)
//   head:    out = w . d0 + b                                      FP32, 1 ch
//
// Input: [batch][z][y][x][16] bf16 (the accelerator uses 3 channels; the rest
// are zero).  Extents must be multiples of 8.
#pragma once

#include "conv.cuh"

namespace doma {

constexpr int kUnetIn = 16;
constexpr int kUnetBase = 32;
constexpr int kUnetConvs = 14;

struct UnetLayer {
  int cin, cout;
  bool relu;
  size_t w_off, b_off;        // offsets into the flat parameter array
  __nv_bfloat16 * w = nullptr;   // [27][cout][cin]
  __nv_bfloat16 * wt = nullptr;  // [27][cin][cout], taps mirrored
};

struct UnetWork {
  ConvShape s[4];
  size_t voxels[4] = {0, 0, 0, 0};
  // activations
  __nv_bfloat16 *e0a = nullptr, *e0 = nullptr, *u0 = nullptr, *d0 = nullptr;
  __nv_bfloat16 *p[4] = {}, *ea[4] = {}, *e[4] = {}, *c[4] = {}, *u[4] = {}, *d[4] = {};
  // gradients
  __nv_bfloat16 *gA[4] = {}, *gB[4] = {}, *gs[4] = {};
  float * out = nullptr;
  float * wpartial = nullptr;
  ConvScratch fsplit;  // split reductions of the coarse levels' convolutions
  float * bpartial = nullptr;
  double * hpartial = nullptr;
  std::vector<void *> allocs;
};

}  // namespace doma

struct doma_unet {
  doma::UnetLayer layers[doma::kUnetConvs];
  size_t head_w_off = 0, head_b_off = 0, num_params = 0;
  float * params = nullptr;  // FP32 masters (flat)
  float * grads = nullptr;
  float * adam_m = nullptr;
  float * adam_v = nullptr;
  double * d_loss = nullptr;
  int adam_step = 0;
  int batch = 0, nz = 0, ny = 0, nx = 0;
  unsigned long long work_gen = 0;   // bumped whenever the workspace is reallocated
  doma::UnetWork work;
  cudaStream_t stream = nullptr;
};

namespace doma {

// Forward pass on stream st into out ([batch][z][y][x] floats, device).
doma_status unet_forward(doma_unet * n, const __nv_bfloat16 * x, float * out, int batch, int nz,
                         int ny, int nx, cudaStream_t st);

}  // namespace doma
