// unet.cu -- the learned accelerator's U-Net: parameters, workspace, forward,
// backward (every gradient by this library's kernels) and Adam, behind the
// doma_unet_* C ABI.
#include "unet.cuh"

#include <algorithm>
#include <cmath>
#include <utility>
#include <cstring>
#include <new>

namespace doma {

namespace {

using bf16 = __nv_bfloat16;

constexpr int kWidth[4] = {32, 64, 128, 256};

// Layer table: encoder (0..7), then per level up-conv and decoder conv.
void describe_layers(doma_unet * n)
{
  const int spec[kUnetConvs][3] = {
      {kUnetIn, 32, 1}, {32, 32, 1},     // level 0
      {32, 64, 1},      {64, 64, 1},     // level 1
      {64, 128, 1},     {128, 128, 1},   // level 2
      {128, 256, 1},    {256, 256, 1},   // level 3
      {256, 128, 0},    {128, 128, 1},   // up to level 2, decoder 2
      {128, 64, 0},     {64, 64, 1},     // up to level 1, decoder 1
      {64, 32, 0},      {32, 32, 1},     // up to level 0, decoder 0
  };
  size_t off = 0;
  for (int l = 0; l < kUnetConvs; ++l) {
    UnetLayer & L = n->layers[l];
    L.cin = spec[l][0];
    L.cout = spec[l][1];
    L.relu = spec[l][2] != 0;
    L.w_off = off;
    off += (size_t)27 * L.cin * L.cout;
    L.b_off = off;
    off += (size_t)L.cout;
  }
  n->head_w_off = off;
  off += kUnetBase;
  n->head_b_off = off;
  off += 1;
  n->num_params = off;
}

template <typename T>
doma_status walloc(UnetWork & w, T ** p, size_t count)
{
  void * v = nullptr;
  DOMA_CUDA_TRY(cudaMalloc(&v, std::max<size_t>(1, count) * sizeof(T)));
  w.allocs.push_back(v);
  *p = static_cast<T *>(v);
  return DOMA_OK;
}

void free_work(UnetWork & w)
{
  for (void * p : w.allocs) cudaFree(p);
  w = UnetWork{};
}

doma_status ensure_work(doma_unet * n, int batch, int nz, int ny, int nx)
{
  if (n->batch == batch && n->nz == nz && n->ny == ny && n->nx == nx) return DOMA_OK;
  free_work(n->work);
  ++n->work_gen;   // graphs captured over the old workspace are stale
  n->batch = n->nz = n->ny = n->nx = 0;
  UnetWork & w = n->work;
  for (int l = 0; l < 4; ++l) {
    w.s[l] = ConvShape{batch, nz >> l, ny >> l, nx >> l};
    w.voxels[l] = w.s[l].voxels();
  }
  const size_t V0 = w.voxels[0];
  DOMA_TRY(walloc(w, &w.e0a, V0 * 32));
  DOMA_TRY(walloc(w, &w.e0, V0 * 32));
  DOMA_TRY(walloc(w, &w.u0, V0 * 32));
  DOMA_TRY(walloc(w, &w.d0, V0 * 32));
  for (int l = 1; l < 4; ++l) {
    const size_t V = w.voxels[l];
    DOMA_TRY(walloc(w, &w.p[l], V * kWidth[l - 1]));
    DOMA_TRY(walloc(w, &w.ea[l], V * kWidth[l]));
    DOMA_TRY(walloc(w, &w.e[l], V * kWidth[l]));
    // c[l] is the up-conv output at level l, feeding level l-1 (width of l-1)
    DOMA_TRY(walloc(w, &w.c[l], V * kWidth[l - 1]));
    if (l < 3) {
      DOMA_TRY(walloc(w, &w.u[l], V * kWidth[l]));
      DOMA_TRY(walloc(w, &w.d[l], V * kWidth[l]));
    }
  }
  for (int l = 0; l < 4; ++l) {
    const size_t V = w.voxels[l];
    DOMA_TRY(walloc(w, &w.gA[l], V * kWidth[l]));
    DOMA_TRY(walloc(w, &w.gB[l], V * kWidth[l]));
    if (l < 3) DOMA_TRY(walloc(w, &w.gs[l], V * kWidth[l]));
  }
  DOMA_TRY(walloc(w, &w.out, V0));
  size_t ws = 0, fs = 0;
  for (int l = 0; l < kUnetConvs; ++l) {
    const UnetLayer & L = n->layers[l];
    const int lvl = l < 8 ? l / 2 : (l == 8 ? 3 : l == 9 ? 2 : l == 10 ? 2 : l == 11 ? 1 : l == 12 ? 1 : 0);
    ws = std::max(ws, conv3_wgrad_scratch(w.s[lvl], L.cin, L.cout));
    fs = std::max(fs, conv3_tc_split_scratch(w.s[lvl], L.cin, L.cout));
    fs = std::max(fs, conv3_tc_split_scratch(w.s[lvl], L.cout, L.cin));
  }
  DOMA_TRY(walloc(w, &w.wpartial, ws));
  if (fs > 0) {
    DOMA_TRY(walloc(w, &w.fsplit.p, fs));
    w.fsplit.floats = fs;
  }
  DOMA_TRY(walloc(w, &w.bpartial, bias_grad_scratch(256)));
  DOMA_TRY(walloc(w, &w.hpartial, head_backward_scratch(kUnetBase)));
  n->batch = batch;
  n->nz = nz;
  n->ny = ny;
  n->nx = nx;
  return DOMA_OK;
}

doma_status publish_all(doma_unet * n, cudaStream_t st)
{
  for (auto & L : n->layers) DOMA_TRY(publish_weights(n->params + L.w_off, L.cin, L.cout, L.w, L.wt, st));
  return DOMA_OK;
}

doma_status check_shape(int batch, int nz, int ny, int nx)
{
  if (batch <= 0 || nz <= 0 || ny <= 0 || nx <= 0 || nz % 8 || ny % 8 || nx % 8) {
    set_error("the U-Net needs a positive batch and extents that are multiples of 8");
    return DOMA_BAD_INPUT;
  }
  return DOMA_OK;
}

doma_status conv(doma_unet * n, int l, const ConvShape & s, const bf16 * x, bf16 * y,
                 cudaStream_t st)
{
  const UnetLayer & L = n->layers[l];
  return conv3_forward(s, x, L.cin, L.w, n->params + L.b_off, L.cout, L.relu, y, st,
                       n->work.fsplit);
}

// dgrad of layer l: gx = conv(gz, mirrored transposed weights), no bias
doma_status dgrad(doma_unet * n, int l, const ConvShape & s, const bf16 * gz, bf16 * gx,
                  cudaStream_t st)
{
  const UnetLayer & L = n->layers[l];
  return conv3_forward(s, gz, L.cout, L.wt, nullptr, L.cin, false, gx, st, n->work.fsplit);
}

doma_status wgrad(doma_unet * n, int l, const ConvShape & s, const bf16 * x, const bf16 * gz,
                  cudaStream_t st)
{
  const UnetLayer & L = n->layers[l];
  DOMA_TRY(conv3_wgrad(s, x, L.cin, gz, L.cout, n->work.wpartial, n->grads + L.w_off, st));
  return bias_grad(s.voxels(), L.cout, gz, n->work.bpartial, n->grads + L.b_off, st);
}

doma_status forward_impl(doma_unet * n, const bf16 * x, cudaStream_t st)
{
  UnetWork & w = n->work;
  DOMA_TRY(conv3_tc_error_reset(st));
  DOMA_TRY(conv(n, 0, w.s[0], x, w.e0a, st));
  DOMA_TRY(conv(n, 1, w.s[0], w.e0a, w.e0, st));
  const bf16 * prev = w.e0;
  for (int l = 1; l < 4; ++l) {
    DOMA_TRY(avgpool2(w.s[l - 1], kWidth[l - 1], prev, w.p[l], st));
    DOMA_TRY(conv(n, 2 * l, w.s[l], w.p[l], w.ea[l], st));
    DOMA_TRY(conv(n, 2 * l + 1, w.s[l], w.ea[l], w.e[l], st));
    prev = w.e[l];
  }
  // decoder: level 2, 1, 0
  const bf16 * deep = w.e[3];
  for (int l = 2; l >= 0; --l) {
    const int up = 8 + 2 * (2 - l), dec = up + 1;
    DOMA_TRY(conv(n, up, w.s[l + 1], deep, w.c[l + 1], st));
    bf16 * skip = l == 0 ? w.e0 : w.e[l];
    bf16 * u = l == 0 ? w.u0 : w.u[l];
    bf16 * d = l == 0 ? w.d0 : w.d[l];
    DOMA_TRY(up_add_relu(w.s[l], kWidth[l], w.c[l + 1], skip, u, st));
    DOMA_TRY(conv(n, dec, w.s[l], u, d, st));
    deep = d;
  }
  return head_forward(w.voxels[0], kUnetBase, w.d0, n->params + n->head_w_off,
                      n->params + n->head_b_off, w.out, st);
}

doma_status backward_impl(doma_unet * n, const bf16 * x, const float * target, cudaStream_t st,
                          const float * sample_weight = nullptr)
{
  UnetWork & w = n->work;
  DOMA_TRY(head_backward(w.voxels[0], kUnetBase, w.d0, n->params + n->head_w_off, w.out, target,
                         w.gA[0], n->grads + n->head_w_off, n->grads + n->head_b_off, w.hpartial,
                         n->d_loss, st, sample_weight, w.voxels[0] / (size_t)std::max(n->batch, 1)));
  // decoder levels 0, 1, 2: gA[l] holds the gradient of d_l's pre-activation
  for (int l = 0; l <= 2; ++l) {
    const int up = 8 + 2 * (2 - l), dec = up + 1;
    bf16 * u = l == 0 ? w.u0 : w.u[l];
    bf16 * g_dec = l == 0 ? w.gA[0] : w.gB[l];
    DOMA_TRY(wgrad(n, dec, w.s[l], u, g_dec, st));
    DOMA_TRY(dgrad(n, dec, w.s[l], g_dec, w.gs[l], st));
    DOMA_TRY(relu_mask(w.voxels[l] * kWidth[l], w.gs[l], u, st));
    // gradient of c_{l+1} (up-conv output, no activation)
    DOMA_TRY(sumpool2(w.s[l], kWidth[l], w.gs[l], w.gA[l + 1], st));
    const bf16 * deep_in = l == 2 ? w.e[3] : w.d[l + 1];
    DOMA_TRY(wgrad(n, up, w.s[l + 1], deep_in, w.gA[l + 1], st));
    DOMA_TRY(dgrad(n, up, w.s[l + 1], w.gA[l + 1], w.gB[l + 1], st));
    DOMA_TRY(relu_mask(w.voxels[l + 1] * kWidth[l + 1], w.gB[l + 1], deep_in, st));
  }
  // bottom: gB[3] = gradient of e3's pre-activation
  DOMA_TRY(wgrad(n, 7, w.s[3], w.ea[3], w.gB[3], st));
  DOMA_TRY(dgrad(n, 7, w.s[3], w.gB[3], w.gA[3], st));
  DOMA_TRY(relu_mask(w.voxels[3] * 256, w.gA[3], w.ea[3], st));
  DOMA_TRY(wgrad(n, 6, w.s[3], w.p[3], w.gA[3], st));
  DOMA_TRY(dgrad(n, 6, w.s[3], w.gA[3], w.gB[3], st));  // gradient of p3 (128 ch)
  // encoder levels 2, 1, 0: gB[l+1] holds the gradient of p_{l+1}
  for (int l = 2; l >= 0; --l) {
    bf16 * e = l == 0 ? w.e0 : w.e[l];
    bf16 * ea = l == 0 ? w.e0a : w.ea[l];
    const bf16 * in = l == 0 ? x : w.p[l];
    DOMA_TRY(pool_back_add_mask(w.s[l], kWidth[l], w.gB[l + 1], w.gs[l], e, w.gA[l], st));
    DOMA_TRY(wgrad(n, 2 * l + 1, w.s[l], ea, w.gA[l], st));
    DOMA_TRY(dgrad(n, 2 * l + 1, w.s[l], w.gA[l], w.gB[l], st));
    DOMA_TRY(relu_mask(w.voxels[l] * kWidth[l], w.gB[l], ea, st));
    DOMA_TRY(wgrad(n, 2 * l, w.s[l], in, w.gB[l], st));
    if (l > 0) DOMA_TRY(dgrad(n, 2 * l, w.s[l], w.gB[l], w.gA[l], st));  // gradient of p_l
    if (l > 0) std::swap(w.gA[l], w.gB[l]);  // keep "gB[l] = gradient of p_l" for the next level
  }
  return DOMA_OK;
}

// Portable host initialisation: SplitMix64 uniforms, Irwin-Hall normals.
uint64_t mix64(uint64_t z)
{
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

}  // namespace

doma_status unet_forward(doma_unet * n, const bf16 * x, float * out, int batch, int nz, int ny,
                         int nx, cudaStream_t st)
{
  DOMA_TRY(check_shape(batch, nz, ny, nx));
  DOMA_TRY(ensure_work(n, batch, nz, ny, nx));
  DOMA_TRY(forward_impl(n, x, st));
  if (out != n->work.out)
    DOMA_CUDA_TRY(cudaMemcpyAsync(out, n->work.out, n->work.voxels[0] * sizeof(float),
                                  cudaMemcpyDeviceToDevice, st));
  return DOMA_OK;
}

}  // namespace doma

using namespace doma;

namespace {

doma_status bad_net(const char * msg)
{
  set_error(msg);
  return DOMA_BAD_INPUT;
}

void release_net(doma_unet * n)
{
  if (!n) return;
  free_work(n->work);
  for (auto & L : n->layers) {
    cudaFree(L.w);
    cudaFree(L.wt);
  }
  cudaFree(n->params);
  cudaFree(n->grads);
  cudaFree(n->adam_m);
  cudaFree(n->adam_v);
  cudaFree(n->d_loss);
  delete n;
}

}  // namespace

extern "C" {

doma_status doma_unet_create(uint64_t seed, doma_unet ** out)
{
  if (!out) return bad_net("null output handle");
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    set_error("no CUDA device is visible");
    return DOMA_NO_DEVICE;
  }
  doma_unet * n = new (std::nothrow) doma_unet();
  if (!n) return bad_net("out of host memory");
  describe_layers(n);
  auto fail = [&](doma_status st) {
    release_net(n);
    return st;
  };
  const size_t P = n->num_params;
  if (cudaMalloc(&n->params, P * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&n->grads, P * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&n->adam_m, P * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&n->adam_v, P * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&n->d_loss, sizeof(double)) != cudaSuccess) {
    set_error("out of device memory for the U-Net parameters");
    return fail(DOMA_CUDA_ERROR);
  }
  for (auto & L : n->layers) {
    const size_t c = (size_t)27 * L.cin * L.cout;
    if (cudaMalloc(&L.w, c * sizeof(bf16)) != cudaSuccess ||
        cudaMalloc(&L.wt, c * sizeof(bf16)) != cudaSuccess) {
      set_error("out of device memory for the U-Net weights");
      return fail(DOMA_CUDA_ERROR);
    }
  }
  // He-normal weights (std sqrt(2 / fan_in); sqrt(1 / fan_in) before a
  // linear up-conv), zero biases, a small head.
  std::vector<float> h(P, 0.0f);
  uint64_t ctr = mix64(seed ^ 0x756E6574ull);
  auto normal = [&]() {
    double s = 0.0;
    for (int k = 0; k < 12; ++k) s += (double)(mix64(ctr++) >> 11) * (1.0 / 9007199254740992.0);
    return s - 6.0;
  };
  for (const auto & L : n->layers) {
    const int fan = 27 * (L.cin == kUnetIn ? 3 : L.cin);
    const double sd = std::sqrt((L.relu ? 2.0 : 1.0) / fan);
    for (size_t i = 0; i < (size_t)27 * L.cin * L.cout; ++i) {
      const int ci = (int)(i % L.cin);
      h[L.w_off + i] = (L.cin == kUnetIn && ci >= 3) ? 0.0f : (float)(sd * normal());
    }
  }
  for (int k = 0; k < kUnetBase; ++k) h[n->head_w_off + k] = (float)(0.1 * normal() / std::sqrt(32.0));
  if (cudaMemcpy(n->params, h.data(), P * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemset(n->grads, 0, P * sizeof(float)) != cudaSuccess ||
      cudaMemset(n->adam_m, 0, P * sizeof(float)) != cudaSuccess ||
      cudaMemset(n->adam_v, 0, P * sizeof(float)) != cudaSuccess ||
      cudaMemset(n->d_loss, 0, sizeof(double)) != cudaSuccess)
    return fail(DOMA_CUDA_ERROR);
  doma_status st = publish_all(n, nullptr);
  if (st == DOMA_OK && cudaDeviceSynchronize() != cudaSuccess) st = DOMA_CUDA_ERROR;
  if (st != DOMA_OK) return fail(st);
  *out = n;
  return DOMA_OK;
}

void doma_unet_destroy(doma_unet * n) { release_net(n); }

doma_status doma_unet_set_stream(doma_unet * n, void * stream)
{
  if (!n) return bad_net("null network");
  n->stream = static_cast<cudaStream_t>(stream);
  return DOMA_OK;
}

size_t doma_unet_num_params(const doma_unet * n) { return n ? n->num_params : 0; }

doma_status doma_unet_get_params(doma_unet * n, float * out, size_t count)
{
  if (!n || !out || count != n->num_params) return bad_net("parameter buffer size mismatch");
  DOMA_CUDA_TRY(cudaStreamSynchronize(n->stream));
  DOMA_CUDA_TRY(cudaMemcpy(out, n->params, count * sizeof(float), cudaMemcpyDeviceToHost));
  return DOMA_OK;
}

doma_status doma_unet_set_params(doma_unet * n, const float * in, size_t count)
{
  if (!n || !in || count != n->num_params) return bad_net("parameter buffer size mismatch");
  DOMA_CUDA_TRY(cudaStreamSynchronize(n->stream));
  DOMA_CUDA_TRY(cudaMemcpy(n->params, in, count * sizeof(float), cudaMemcpyHostToDevice));
  DOMA_TRY(publish_all(n, n->stream));
  DOMA_CUDA_TRY(cudaStreamSynchronize(n->stream));
  return DOMA_OK;
}

doma_status doma_unet_get_grads(doma_unet * n, float * out, size_t count)
{
  if (!n || !out || count != n->num_params) return bad_net("gradient buffer size mismatch");
  DOMA_CUDA_TRY(cudaStreamSynchronize(n->stream));
  DOMA_CUDA_TRY(cudaMemcpy(out, n->grads, count * sizeof(float), cudaMemcpyDeviceToHost));
  return DOMA_OK;
}

doma_status doma_unet_forward(doma_unet * n, const void * input, float * output, uint32_t batch,
                              uint32_t nz, uint32_t ny, uint32_t nx)
{
  if (!n || !input || !output) return bad_net("null network or buffer");
  return unet_forward(n, static_cast<const bf16 *>(input), output, (int)batch, (int)nz, (int)ny,
                      (int)nx, n->stream);
}

doma_status doma_unet_backward(doma_unet * n, const void * input, const float * target,
                               uint32_t batch, uint32_t nz, uint32_t ny, uint32_t nx)
{
  if (!n || !input || !target) return bad_net("null network or buffer");
  DOMA_TRY(check_shape((int)batch, (int)nz, (int)ny, (int)nx));
  DOMA_TRY(ensure_work(n, (int)batch, (int)nz, (int)ny, (int)nx));
  const bf16 * x = static_cast<const bf16 *>(input);
  DOMA_TRY(forward_impl(n, x, n->stream));
  return backward_impl(n, x, target, n->stream);
}

doma_status doma_unet_backward_weighted(doma_unet * n, const void * input, const float * target,
                                        const float * sample_weight, uint32_t batch, uint32_t nz,
                                        uint32_t ny, uint32_t nx)
{
  if (!n || !input || !target || !sample_weight) return bad_net("null network or buffer");
  DOMA_TRY(check_shape((int)batch, (int)nz, (int)ny, (int)nx));
  DOMA_TRY(ensure_work(n, (int)batch, (int)nz, (int)ny, (int)nx));
  const bf16 * x = static_cast<const bf16 *>(input);
  DOMA_TRY(forward_impl(n, x, n->stream));
  return backward_impl(n, x, target, n->stream, sample_weight);
}

doma_status doma_unet_last_loss(doma_unet * n, double * loss)
{
  if (!n || !loss) return bad_net("null network or buffer");
  DOMA_CUDA_TRY(cudaStreamSynchronize(n->stream));
  DOMA_CUDA_TRY(cudaMemcpy(loss, n->d_loss, sizeof(double), cudaMemcpyDeviceToHost));
  return DOMA_OK;
}

doma_status doma_conv3_forward(const void * x, uint32_t batch, uint32_t nz, uint32_t ny,
                               uint32_t nx, uint32_t cin, const void * w, const float * bias,
                               uint32_t cout, uint32_t relu, void * y, uint32_t path, void * stream)
{
  if (!x || !w || !y) return bad_net("null tensor");
  const ConvShape s{(int)batch, (int)nz, (int)ny, (int)nx};
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const bf16 * xb = static_cast<const bf16 *>(x);
  const bf16 * wb = static_cast<const bf16 *>(w);
  bf16 * yb = static_cast<bf16 *>(y);
  if (path == DOMA_CONV_MMA)
    return conv3_forward_mma(s, xb, (int)cin, wb, bias, (int)cout, relu != 0, yb, st);
  DOMA_TRY(conv3_tc_error_reset(st));
  // the split-reduction scratch the U-Net keeps in its workspace, stream-ordered here
  ConvScratch sc;
  sc.floats = conv3_tc_split_scratch(s, (int)cin, (int)cout);
  if (sc.floats > 0) {
    void * p = nullptr;
    DOMA_CUDA_TRY(cudaMallocAsync(&p, sc.floats * sizeof(float), st));
    sc.p = static_cast<float *>(p);
  }
  const doma_status r =
      path == DOMA_CONV_TENSOR_MEMORY
          ? conv3_forward_tc(s, xb, (int)cin, wb, bias, (int)cout, relu != 0, yb, st, sc)
          : conv3_forward(s, xb, (int)cin, wb, bias, (int)cout, relu != 0, yb, st, sc);
  if (sc.p) {
    const cudaError_t e = cudaFreeAsync(sc.p, st);
    if (r == DOMA_OK && e != cudaSuccess) {
      set_error(std::string("cudaFreeAsync: ") + cudaGetErrorString(e));
      return DOMA_CUDA_ERROR;
    }
  }
  return r;
}

doma_status doma_conv3_wgrad(const void * x, uint32_t batch, uint32_t nz, uint32_t ny, uint32_t nx,
                             uint32_t cin, const void * dz, uint32_t cout, float * dw,
                             uint32_t path, void * stream)
{
  if (!x || !dz || !dw) return bad_net("null tensor");
  const ConvShape s{(int)batch, (int)nz, (int)ny, (int)nx};
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (path == DOMA_CONV_TENSOR_MEMORY || path == DOMA_CONV_AUTO) DOMA_TRY(conv3_tc_error_reset(st));
  // the split partials, stream-ordered here (the U-Net keeps them in its workspace)
  void * p = nullptr;
  const size_t floats = conv3_wgrad_scratch(s, (int)cin, (int)cout);
  DOMA_CUDA_TRY(cudaMallocAsync(&p, std::max<size_t>(floats, 1) * sizeof(float), st));
  const doma_status r = conv3_wgrad(s, static_cast<const bf16 *>(x), (int)cin,
                                    static_cast<const bf16 *>(dz), (int)cout,
                                    static_cast<float *>(p), dw, st, (int)path);
  const cudaError_t e = cudaFreeAsync(p, st);
  if (r == DOMA_OK && e != cudaSuccess) {
    set_error(std::string("cudaFreeAsync: ") + cudaGetErrorString(e));
    return DOMA_CUDA_ERROR;
  }
  return r;
}

doma_status doma_conv_wait_error(int * flag)
{
  if (!flag) return bad_net("null flag");
  return conv3_tc_error(flag);
}

doma_status doma_unet_adam(doma_unet * n, float lr, float beta1, float beta2, float eps)
{
  if (!n) return bad_net("null network");
  ++n->adam_step;
  DOMA_TRY(adam_update(n->num_params, n->params, n->grads, n->adam_m, n->adam_v, lr, beta1, beta2,
                       eps, n->adam_step, n->stream));
  return publish_all(n, n->stream);
}

}  // extern "C"
