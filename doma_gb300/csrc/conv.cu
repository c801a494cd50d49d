// conv.cu -- BF16 3D convolution and U-Net pieces on the CUDA cores' warp-
// level tensor instructions (mma.sync m16n8k16, FP32 accumulation).
//
// conv3_forward is an implicit GEMM: rows are voxels (128 per CTA), columns
// are output channels, the reduction runs over 27 taps x input channels.  The
// A tile of one (tap, channel chunk) step is gathered straight from the
// channels-last input with 16-byte cp.async copies (zero-filled outside the
// volume, which is the convolution's zero padding); B is the tap's weight
// slab.  Tiles live in XOR-swizzled shared memory (ldmatrix reads 8 rows at
// one 16-byte column without bank conflicts), three stages deep.
//
// conv3_wgrad reduces over voxels instead: per (tap, cout tile, cin tile) and
// voxel split it multiplies dz^T by the shifted input, both staged as
// [voxel][channel] tiles and read transposed by ldmatrix.trans.  Splits write
// partial sums that one kernel adds in split order, so the result does not
// depend on scheduling.
#include "conv.cuh"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <string>

namespace doma {

namespace {

using bf16 = __nv_bfloat16;

constexpr int kStages = 3;
constexpr int kReduceBlocks = 256;  // fixed block count of the fixed-order reductions

__device__ __forceinline__ unsigned smem_u32(const void * p)
{
  return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void cp_async16(unsigned dst, const void * src, bool valid)
{
  const int n = valid ? 16 : 0;
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src), "r"(n));
}

__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::); }

template <int N>
__device__ __forceinline__ void cp_wait()
{
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N));
}

__device__ __forceinline__ void ldsm_x4(unsigned addr, unsigned & r0, unsigned & r1, unsigned & r2,
                                        unsigned & r3)
{
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(addr));
}

__device__ __forceinline__ void ldsm_x4_t(unsigned addr, unsigned & r0, unsigned & r1,
                                          unsigned & r2, unsigned & r3)
{
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(addr));
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], const unsigned (&a)[4], unsigned b0,
                                         unsigned b1)
{
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Byte offset of 16-byte chunk `chunk` of row `row` in a tile whose rows are
// CH chunks long: the chunk index is XORed with the row's position among the
// rows that share a 128-byte line group, so 8 consecutive rows read at one
// logical chunk hit 8 different bank groups.
template <int CH>
__device__ __forceinline__ int swz(int row, int chunk)
{
  return (row * CH + (chunk ^ ((row / (8 / CH)) & (CH - 1)))) * 16;
}

__device__ __forceinline__ void tap_offsets(int tap, int & dz, int & dy, int & dx)
{
  dz = tap / 9 - 1;
  dy = (tap / 3) % 3 - 1;
  dx = tap % 3 - 1;
}

struct ConvArgs {
  const bf16 * x;
  const bf16 * w;
  const float * bias;
  bf16 * y;
  int nz, ny, nx;
  long long M;
  int cin, cout;
};

template <int BN, int KC, bool RELU>
__global__ void __launch_bounds__(256) conv3_fwd_kernel(const ConvArgs a)
{
  constexpr int BM = 128, THREADS = 256;
  constexpr int CH = KC / 8;
  constexpr int WARPS_N = BN >= 128 ? 4 : 2;
  constexpr int WARPS_M = 8 / WARPS_N;
  constexpr int WTM = BM / WARPS_M, WTN = BN / WARPS_N;
  constexpr int MT = WTM / 16, NT = WTN / 8;
  constexpr int A_BYTES = BM * KC * 2, B_BYTES = BN * KC * 2, STAGE = A_BYTES + B_BYTES;
  constexpr int A_ITERS = BM * CH / THREADS;
  static_assert(A_ITERS >= 1 && NT % 2 == 0, "tile shape");
  extern __shared__ __align__(128) unsigned char smem[];

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = warp / WARPS_N, wn = warp % WARPS_N;
  const long long m0 = (long long)blockIdx.x * BM;
  const int n0 = blockIdx.y * BN;

  int rz[A_ITERS], ry[A_ITERS], rx[A_ITERS];
  long long rm[A_ITERS];
  bool rv[A_ITERS];
#pragma unroll
  for (int j = 0; j < A_ITERS; ++j) {
    const int row = (tid + j * THREADS) / CH;
    const long long m = m0 + row;
    rv[j] = m < a.M;
    const long long mm = rv[j] ? m : 0;
    rm[j] = mm;
    rx[j] = (int)(mm % a.nx);
    const long long t = mm / a.nx;
    ry[j] = (int)(t % a.ny);
    rz[j] = (int)((t / a.ny) % a.nz);
  }

  const int steps_per_tap = a.cin / KC;
  const int k_steps = 27 * steps_per_tap;

  auto load = [&](int stage, int ks) {
    const int tap = ks / steps_per_tap, c0 = (ks % steps_per_tap) * KC;
    int dz, dy, dx;
    tap_offsets(tap, dz, dy, dx);
    unsigned char * As = smem + stage * STAGE;
    unsigned char * Bs = As + A_BYTES;
    const long long shift = ((long long)dz * a.ny + dy) * a.nx + dx;
#pragma unroll
    for (int j = 0; j < A_ITERS; ++j) {
      const int i = tid + j * THREADS, row = i / CH, ch = i % CH;
      const bool valid = rv[j] && (unsigned)(rz[j] + dz) < (unsigned)a.nz &&
                         (unsigned)(ry[j] + dy) < (unsigned)a.ny &&
                         (unsigned)(rx[j] + dx) < (unsigned)a.nx;
      const bf16 * src = valid ? a.x + (rm[j] + shift) * a.cin + c0 + ch * 8 : a.x;
      cp_async16(smem_u32(As + swz<CH>(row, ch)), src, valid);
    }
    for (int i = tid; i < BN * CH; i += THREADS) {
      const int row = i / CH, ch = i % CH;
      const bf16 * src = a.w + ((size_t)tap * a.cout + n0 + row) * a.cin + c0 + ch * 8;
      cp_async16(smem_u32(Bs + swz<CH>(row, ch)), src, true);
    }
  };

  float acc[MT][NT][4];
#pragma unroll
  for (int i = 0; i < MT; ++i)
#pragma unroll
    for (int j = 0; j < NT; ++j)
#pragma unroll
      for (int k = 0; k < 4; ++k) acc[i][j][k] = 0.0f;

#pragma unroll
  for (int s = 0; s < kStages - 1; ++s) {
    if (s < k_steps) load(s, s);
    cp_commit();
  }
  for (int ks = 0; ks < k_steps; ++ks) {
    cp_wait<kStages - 2>();
    __syncthreads();
    const int nk = ks + kStages - 1;
    if (nk < k_steps) load(nk % kStages, nk);
    cp_commit();
    const unsigned char * As = smem + (ks % kStages) * STAGE;
    const unsigned char * Bs = As + A_BYTES;
#pragma unroll
    for (int kk = 0; kk < KC / 16; ++kk) {
      unsigned af[MT][4];
#pragma unroll
      for (int mt = 0; mt < MT; ++mt) {
        const int row = wm * WTM + mt * 16 + (lane & 15);
        const int chunk = kk * 2 + (lane >> 4);
        ldsm_x4(smem_u32(As + swz<CH>(row, chunk)), af[mt][0], af[mt][1], af[mt][2], af[mt][3]);
      }
      unsigned bfr[NT][2];
#pragma unroll
      for (int np = 0; np < NT / 2; ++np) {
        const int row = wn * WTN + np * 16 + (lane & 7) + ((lane >> 4) << 3);
        const int chunk = kk * 2 + ((lane >> 3) & 1);
        ldsm_x4(smem_u32(Bs + swz<CH>(row, chunk)), bfr[2 * np][0], bfr[2 * np][1],
                bfr[2 * np + 1][0], bfr[2 * np + 1][1]);
      }
#pragma unroll
      for (int mt = 0; mt < MT; ++mt)
#pragma unroll
        for (int nt = 0; nt < NT; ++nt) mma_bf16(acc[mt][nt], af[mt], bfr[nt][0], bfr[nt][1]);
    }
  }
  cp_wait<0>();

  const int g = lane >> 2, t4 = lane & 3;
#pragma unroll
  for (int nt = 0; nt < NT; ++nt) {
    const int col = n0 + wn * WTN + nt * 8 + 2 * t4;
    const float b0 = a.bias ? a.bias[col] : 0.0f;
    const float b1 = a.bias ? a.bias[col + 1] : 0.0f;
#pragma unroll
    for (int mt = 0; mt < MT; ++mt)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const long long row = m0 + wm * WTM + mt * 16 + g + 8 * h;
        if (row < a.M) {
          float v0 = acc[mt][nt][2 * h] + b0, v1 = acc[mt][nt][2 * h + 1] + b1;
          if (RELU) {
            v0 = fmaxf(v0, 0.0f);
            v1 = fmaxf(v1, 0.0f);
          }
          *reinterpret_cast<__nv_bfloat162 *>(a.y + row * a.cout + col) =
              __floats2bfloat162_rn(v0, v1);
        }
      }
  }
}

struct WgradArgs {
  const bf16 * x;
  const bf16 * dz;
  float * partial;
  int nz, ny, nx;
  long long M;
  int cin, cout;
  long long chunks_per_split;
  int ci_tiles;
};

template <int BMO, int BNI>
__global__ void __launch_bounds__(32 * (BMO / 16) * (BNI / 16)) conv3_wgrad_kernel(const WgradArgs a)
{
  constexpr int WN = BNI / 16, THREADS = 32 * (BMO / 16) * WN;
  constexpr int KV = 32;  // voxels per stage
  constexpr int CHO = BMO / 8, CHI = BNI / 8;
  constexpr int D_BYTES = KV * BMO * 2, X_BYTES = KV * BNI * 2, STAGE = D_BYTES + X_BYTES;
  extern __shared__ __align__(128) unsigned char smem[];

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = warp / WN, wn = warp % WN;
  int bid = blockIdx.x;
  const int tap = bid % 27;
  bid /= 27;
  const int ci0 = (bid % a.ci_tiles) * BNI, co0 = (bid / a.ci_tiles) * BMO;
  const int split = blockIdx.y;
  int ddz, ddy, ddx;
  tap_offsets(tap, ddz, ddy, ddx);
  const long long shift = ((long long)ddz * a.ny + ddy) * a.nx + ddx;
  const long long total = (a.M + KV - 1) / KV;
  const long long c_begin = (long long)split * a.chunks_per_split;
  const long long c_end = c_begin + a.chunks_per_split < total ? c_begin + a.chunks_per_split : total;
  const int nsteps = c_end > c_begin ? (int)(c_end - c_begin) : 0;

  auto load = [&](int stage, long long chunk) {
    const long long mbase = chunk * KV;
    unsigned char * Ds = smem + stage * STAGE;
    unsigned char * Xs = Ds + D_BYTES;
    for (int i = tid; i < KV * CHO; i += THREADS) {
      const int row = i / CHO, ch = i % CHO;
      const long long m = mbase + row;
      const bool valid = m < a.M;
      const bf16 * src = valid ? a.dz + m * a.cout + co0 + ch * 8 : a.dz;
      cp_async16(smem_u32(Ds + swz<CHO>(row, ch)), src, valid);
    }
    for (int i = tid; i < KV * CHI; i += THREADS) {
      const int row = i / CHI, ch = i % CHI;
      const long long m = mbase + row;
      bool valid = m < a.M;
      if (valid) {
        const int x = (int)(m % a.nx);
        const long long t = m / a.nx;
        const int y = (int)(t % a.ny), z = (int)((t / a.ny) % a.nz);
        valid = (unsigned)(z + ddz) < (unsigned)a.nz && (unsigned)(y + ddy) < (unsigned)a.ny &&
                (unsigned)(x + ddx) < (unsigned)a.nx;
      }
      const bf16 * src = valid ? a.x + (m + shift) * a.cin + ci0 + ch * 8 : a.x;
      cp_async16(smem_u32(Xs + swz<CHI>(row, ch)), src, valid);
    }
  };

  float acc[2][4];
#pragma unroll
  for (int j = 0; j < 2; ++j)
#pragma unroll
    for (int k = 0; k < 4; ++k) acc[j][k] = 0.0f;

#pragma unroll
  for (int s = 0; s < kStages - 1; ++s) {
    if (s < nsteps) load(s, c_begin + s);
    cp_commit();
  }
  for (int ks = 0; ks < nsteps; ++ks) {
    cp_wait<kStages - 2>();
    __syncthreads();
    const int nk = ks + kStages - 1;
    if (nk < nsteps) load(nk % kStages, c_begin + nk);
    cp_commit();
    const unsigned char * Ds = smem + (ks % kStages) * STAGE;
    const unsigned char * Xs = Ds + D_BYTES;
    const int j = lane >> 3;
#pragma unroll
    for (int kk = 0; kk < KV / 16; ++kk) {
      unsigned af[4];
      {
        const int row = kk * 16 + (j >> 1) * 8 + (lane & 7);
        const int chunk = wm * 2 + (j & 1);
        ldsm_x4_t(smem_u32(Ds + swz<CHO>(row, chunk)), af[0], af[1], af[2], af[3]);
      }
      unsigned b00, b01, b10, b11;
      {
        const int row = kk * 16 + (j & 1) * 8 + (lane & 7);
        const int chunk = wn * 2 + (j >> 1);
        ldsm_x4_t(smem_u32(Xs + swz<CHI>(row, chunk)), b00, b01, b10, b11);
      }
      mma_bf16(acc[0], af, b00, b01);
      mma_bf16(acc[1], af, b10, b11);
    }
  }
  cp_wait<0>();

  const int g = lane >> 2, t4 = lane & 3;
  float * out = a.partial + ((size_t)split * 27 + tap) * a.cout * a.cin;
#pragma unroll
  for (int nt = 0; nt < 2; ++nt) {
    const int ci = ci0 + wn * 16 + nt * 8 + 2 * t4;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int co = co0 + wm * 16 + g + 8 * h;
      *reinterpret_cast<float2 *>(out + (size_t)co * a.cin + ci) =
          make_float2(acc[nt][2 * h], acc[nt][2 * h + 1]);
    }
  }
}

__global__ void reduce_splits_kernel(const float * partial, int splits, size_t count, float * out)
{
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < count;
       i += (size_t)gridDim.x * blockDim.x) {
    float s = 0.0f;
    for (int k = 0; k < splits; ++k) s += partial[(size_t)k * count + i];
    out[i] = s;
  }
}

// ---- elementwise / resampling (8 channels = one 16-byte vector per thread) ----

struct Vec8 {
  float v[8];
};

__device__ __forceinline__ Vec8 load8(const bf16 * p)
{
  const uint4 u = *reinterpret_cast<const uint4 *>(p);
  const __nv_bfloat162 * h = reinterpret_cast<const __nv_bfloat162 *>(&u);
  Vec8 r;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const float2 f = __bfloat1622float2(h[k]);
    r.v[2 * k] = f.x;
    r.v[2 * k + 1] = f.y;
  }
  return r;
}

__device__ __forceinline__ void store8(bf16 * p, const Vec8 & r)
{
  uint4 u;
  __nv_bfloat162 * h = reinterpret_cast<__nv_bfloat162 *>(&u);
#pragma unroll
  for (int k = 0; k < 4; ++k) h[k] = __floats2bfloat162_rn(r.v[2 * k], r.v[2 * k + 1]);
  *reinterpret_cast<uint4 *>(p) = u;
}

struct Grid5 {
  int nz, ny, nx;  // fine extents
};

// fine voxel index of child (i, j, k) of coarse voxel (b, Z, Y, X)
__device__ __forceinline__ long long child(const Grid5 f, long long coarse, int i, int j, int k)
{
  const int cx = f.nx / 2, cy = f.ny / 2, cz = f.nz / 2;
  const int X = (int)(coarse % cx);
  long long t = coarse / cx;
  const int Y = (int)(t % cy);
  t /= cy;
  const int Z = (int)(t % cz);
  const long long b = t / cz;
  return ((b * f.nz + 2 * Z + i) * f.ny + 2 * Y + j) * f.nx + 2 * X + k;
}

__device__ __forceinline__ long long parent(const Grid5 f, long long fine)
{
  const int x = (int)(fine % f.nx);
  long long t = fine / f.nx;
  const int y = (int)(t % f.ny);
  t /= f.ny;
  const int z = (int)(t % f.nz);
  const long long b = t / f.nz;
  return ((b * (f.nz / 2) + z / 2) * (f.ny / 2) + y / 2) * (f.nx / 2) + x / 2;
}

__global__ void avgpool2_kernel(Grid5 f, long long coarse_voxels, int c, const bf16 * x, bf16 * y)
{
  const int cv = c / 8;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < coarse_voxels * cv;
       i += (long long)gridDim.x * blockDim.x) {
    const long long v = i / cv;
    const int k8 = (int)(i % cv) * 8;
    Vec8 s{};
    for (int a = 0; a < 2; ++a)
      for (int b = 0; b < 2; ++b)
        for (int d = 0; d < 2; ++d) {
          const Vec8 r = load8(x + child(f, v, a, b, d) * c + k8);
#pragma unroll
          for (int q = 0; q < 8; ++q) s.v[q] += r.v[q];
        }
#pragma unroll
    for (int q = 0; q < 8; ++q) s.v[q] *= 0.125f;
    store8(y + v * c + k8, s);
  }
}

__global__ void sumpool2_kernel(Grid5 f, long long coarse_voxels, int c, const bf16 * x, bf16 * y)
{
  const int cv = c / 8;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < coarse_voxels * cv;
       i += (long long)gridDim.x * blockDim.x) {
    const long long v = i / cv;
    const int k8 = (int)(i % cv) * 8;
    Vec8 s{};
    for (int a = 0; a < 2; ++a)
      for (int b = 0; b < 2; ++b)
        for (int d = 0; d < 2; ++d) {
          const Vec8 r = load8(x + child(f, v, a, b, d) * c + k8);
#pragma unroll
          for (int q = 0; q < 8; ++q) s.v[q] += r.v[q];
        }
    store8(y + v * c + k8, s);
  }
}

__global__ void up_add_relu_kernel(Grid5 f, long long fine_voxels, int c, const bf16 * coarse,
                                   const bf16 * skip, bf16 * u)
{
  const int cv = c / 8;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < fine_voxels * cv;
       i += (long long)gridDim.x * blockDim.x) {
    const long long v = i / cv;
    const int k8 = (int)(i % cv) * 8;
    const Vec8 a = load8(coarse + parent(f, v) * c + k8);
    const Vec8 b = load8(skip + v * c + k8);
    Vec8 r;
#pragma unroll
    for (int q = 0; q < 8; ++q) r.v[q] = fmaxf(a.v[q] + b.v[q], 0.0f);
    store8(u + v * c + k8, r);
  }
}

__global__ void pool_back_add_mask_kernel(Grid5 f, long long fine_voxels, int c,
                                          const bf16 * g_pool, const bf16 * g_skip,
                                          const bf16 * y, bf16 * out)
{
  const int cv = c / 8;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < fine_voxels * cv;
       i += (long long)gridDim.x * blockDim.x) {
    const long long v = i / cv;
    const int k8 = (int)(i % cv) * 8;
    const Vec8 a = load8(g_pool + parent(f, v) * c + k8);
    const Vec8 b = load8(g_skip + v * c + k8);
    const Vec8 m = load8(y + v * c + k8);
    Vec8 r;
#pragma unroll
    for (int q = 0; q < 8; ++q) r.v[q] = m.v[q] > 0.0f ? a.v[q] * 0.125f + b.v[q] : 0.0f;
    store8(out + v * c + k8, r);
  }
}

__global__ void relu_mask_kernel(size_t vecs, bf16 * g, const bf16 * y)
{
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < vecs;
       i += (size_t)gridDim.x * blockDim.x) {
    Vec8 a = load8(g + i * 8);
    const Vec8 m = load8(y + i * 8);
#pragma unroll
    for (int q = 0; q < 8; ++q) a.v[q] = m.v[q] > 0.0f ? a.v[q] : 0.0f;
    store8(g + i * 8, a);
  }
}

// Bias gradient: block b sums voxels b, b + B, ... of each channel; the
// block partials are then added in block order.
// Per-block partial column sums of g [voxels][c] (bf16): each thread owns one
// 8-channel group of a fixed set of voxels and reads it as one 16-byte vector;
// the block then adds its voxel lanes per channel in lane order (fixed, so
// deterministic).
__global__ void bias_grad_kernel(long long voxels, int c, const bf16 * g, float * partial)
{
  extern __shared__ float sh[];  // [lanes][c]
  const int groups = c / 8;
  const int lanes = blockDim.x / groups;   // blockDim is a multiple of c / 8
  const int cg = threadIdx.x % groups, lane = threadIdx.x / groups;
  float acc[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  if (lane < lanes) {
#pragma unroll 4
    for (long long m = (long long)blockIdx.x * lanes + lane; m < voxels;
         m += (long long)gridDim.x * lanes) {
      const Vec8 v = load8(g + m * c + cg * 8);
#pragma unroll
      for (int q = 0; q < 8; ++q) acc[q] += v.v[q];
    }
#pragma unroll
    for (int q = 0; q < 8; ++q) sh[lane * c + cg * 8 + q] = acc[q];
  }
  __syncthreads();
  for (int ch = threadIdx.x; ch < c; ch += blockDim.x) {
    float t = 0.0f;
    for (int l = 0; l < lanes; ++l) t += sh[l * c + ch];
    partial[(size_t)blockIdx.x * c + ch] = t;
  }
}

// out[ch] = sum over blocks of partial[b][ch]: one warp per channel, each lane
// adding every 32nd block in order, then a fixed shuffle tree (deterministic).
__global__ void sum_blocks_kernel(const float * partial, int blocks, int c, float * out)
{
  const int ch = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (ch >= c) return;
  float t = 0.0f;
  for (int b = lane; b < blocks; b += 32) t += partial[(size_t)b * c + ch];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  if (lane == 0) out[ch] = t;
}

__global__ void head_forward_kernel(long long voxels, int c, const bf16 * x, const float * w,
                                    const float * b, float * out)
{
  for (long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x; m < voxels;
       m += (long long)gridDim.x * blockDim.x) {
    float s = b[0];
    for (int k = 0; k < c; k += 8) {
      const Vec8 r = load8(x + m * c + k);
#pragma unroll
      for (int q = 0; q < 8; ++q) s = fmaf(w[k + q], r.v[q], s);
    }
    out[m] = s;
  }
}

// Head backward and loss: per block, double partials [c dw, db, loss].
// With sample weights, voxel m belongs to sample m / per_sample and its term
// of the loss (and of every gradient) is scaled by that sample's weight.
__global__ void head_backward_kernel(long long voxels, int c, const bf16 * x, const float * w,
                                     const float * out, const float * target, bf16 * dx,
                                     double * partial, const float * sample_weight,
                                     long long per_sample)
{
  extern __shared__ double dsh[];  // [blockDim][c + 2]
  const int W = c + 2;
  double acc[34];
  for (int k = 0; k < W; ++k) acc[k] = 0.0;
  const double inv = 1.0 / (double)voxels;
  for (long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x; m < voxels;
       m += (long long)gridDim.x * blockDim.x) {
    const double r = (double)out[m] - (double)target[m];
    const double sw = sample_weight ? (double)sample_weight[m / per_sample] : 1.0;
    const float gs = (float)(2.0 * sw * r * inv);
    for (int k = 0; k < c; k += 8) {
      const Vec8 xv = load8(x + m * c + k);
      Vec8 d;
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        d.v[q] = xv.v[q] > 0.0f ? gs * w[k + q] : 0.0f;
        acc[k + q] += (double)gs * xv.v[q];
      }
      store8(dx + m * c + k, d);
    }
    acc[c] += gs;
    acc[c + 1] += sw * r * r;
  }
  for (int k = 0; k < W; ++k) dsh[threadIdx.x * W + k] = acc[k];
  __syncthreads();
  for (int k = threadIdx.x; k < W; k += blockDim.x) {
    double t = 0.0;
    for (int l = 0; l < (int)blockDim.x; ++l) t += dsh[l * W + k];
    partial[(size_t)blockIdx.x * W + k] = t;
  }
}

__global__ void head_finish_kernel(const double * partial, int blocks, int c, long long voxels,
                                   float * dw, float * db, double * loss)
{
  const int W = c + 2;
  for (int k = threadIdx.x; k < W; k += blockDim.x) {
    double t = 0.0;
    for (int b = 0; b < blocks; ++b) t += partial[(size_t)b * W + k];
    if (k < c) dw[k] = (float)t;
    else if (k == c) db[0] = (float)t;
    else loss[0] = t / (double)voxels;
  }
}

__global__ void publish_kernel(const float * w32, int cin, int cout, bf16 * w, bf16 * wt)
{
  const size_t n = (size_t)27 * cin * cout;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const int ci = (int)(i % cin);
    const size_t r = i / cin;
    const int co = (int)(r % cout);
    const int tap = (int)(r / cout);
    const bf16 v = __float2bfloat16_rn(w32[i]);
    w[i] = v;
    wt[((size_t)(26 - tap) * cin + ci) * cout + co] = v;
  }
}

__global__ void adam_kernel(size_t n, float * p, const float * g, float * m, float * v, float lr,
                            float b1, float b2, float eps, float bc1, float bc2)
{
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
  }
}

int blocks_for(long long work, int threads = 256)
{
  const long long b = (work + threads - 1) / threads;
  return (int)std::max<long long>(1, std::min<long long>(b, 152LL * 16));
}

template <typename K>
void allow_smem(K kernel, int bytes)
{
  if (bytes > 48 * 1024) cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

template <int BN, int KC, bool RELU>
doma_status launch_fwd(const ConvArgs & a, cudaStream_t st)
{
  constexpr int smem = kStages * (128 * KC * 2 + BN * KC * 2);
  allow_smem(conv3_fwd_kernel<BN, KC, RELU>, smem);
  const dim3 grid((unsigned)((a.M + 127) / 128), (unsigned)(a.cout / BN));
  conv3_fwd_kernel<BN, KC, RELU><<<grid, 256, smem, st>>>(a);
  DOMA_CUDA_TRY(cudaGetLastError());
  return DOMA_OK;
}

template <int BN, int KC>
doma_status launch_fwd_act(const ConvArgs & a, bool relu, cudaStream_t st)
{
  return relu ? launch_fwd<BN, KC, true>(a, st) : launch_fwd<BN, KC, false>(a, st);
}

bool valid_channels(int c, bool allow16)
{
  return (allow16 && c == 16) || c == 32 || c == 64 || c == 128 || c == 256;
}

// Voxel splits of a weight-gradient launch (a function of the shape only).
void wgrad_plan(const ConvShape & s, int cin, int cout, int & bmo, int & bni, int & tiles,
                int & splits, long long & per_split)
{
  bmo = std::min(cout, 64);
  bni = std::min(cin, 64);
  tiles = 27 * (cout / bmo) * (cin / bni);
  const long long chunks = ((long long)s.voxels() + 31) / 32;
  long long want = (4LL * 152 + tiles - 1) / tiles;
  want = std::min<long long>(want, std::max<long long>(1, chunks / 8));
  want = std::max<long long>(1, std::min<long long>(want, 64));
  per_split = (chunks + want - 1) / want;
  splits = (int)((chunks + per_split - 1) / per_split);
}

template <int BMO, int BNI>
doma_status launch_wgrad(const WgradArgs & a, int tiles, int splits, cudaStream_t st)
{
  constexpr int threads = 32 * (BMO / 16) * (BNI / 16);
  constexpr int smem = kStages * 32 * (BMO + BNI) * 2;
  allow_smem(conv3_wgrad_kernel<BMO, BNI>, smem);
  conv3_wgrad_kernel<BMO, BNI><<<dim3((unsigned)tiles, (unsigned)splits), threads, smem, st>>>(a);
  DOMA_CUDA_TRY(cudaGetLastError());
  return DOMA_OK;
}

}  // namespace

doma_status conv3_forward(const ConvShape & s, const bf16 * x, int cin, const bf16 * w,
                          const float * bias, int cout, bool relu, bf16 * y, cudaStream_t st,
                          ConvScratch scratch)
{
  static const bool mma_only = [] {
    const char * e = std::getenv("DOMA_CONV_PATH");
    return e && std::string(e) == "mma";
  }();
  if (!mma_only && conv3_tc_supported(s, cin, cout))
    return conv3_forward_tc(s, x, cin, w, bias, cout, relu, y, st, scratch);
  return conv3_forward_mma(s, x, cin, w, bias, cout, relu, y, st);
}

doma_status conv3_forward_mma(const ConvShape & s, const bf16 * x, int cin, const bf16 * w,
                              const float * bias, int cout, bool relu, bf16 * y, cudaStream_t st)
{
  if (!valid_channels(cin, true) || !valid_channels(cout, false)) {
    set_error("conv3_forward: unsupported channel counts");
    return DOMA_BAD_INPUT;
  }
  ConvArgs a{x, w, bias, y, s.nz, s.ny, s.nx, (long long)s.voxels(), cin, cout};
  if (a.M == 0) return DOMA_OK;
  const int bn = std::min(cout, 128);
  if (cin == 16) {
    if (bn == 32) return launch_fwd_act<32, 16>(a, relu, st);
    if (bn == 64) return launch_fwd_act<64, 16>(a, relu, st);
    return launch_fwd_act<128, 16>(a, relu, st);
  }
  if (bn == 32) return launch_fwd_act<32, 32>(a, relu, st);
  if (bn == 64) return launch_fwd_act<64, 32>(a, relu, st);
  return launch_fwd_act<128, 32>(a, relu, st);
}

size_t conv3_wgrad_scratch(const ConvShape & s, int cin, int cout)
{
  int bmo, bni, tiles, splits;
  long long per;
  wgrad_plan(s, cin, cout, bmo, bni, tiles, splits, per);
  splits = std::max(splits, conv3_wgrad_tc_splits(s, cin, cout));
  return (size_t)splits * 27 * cin * cout;
}

doma_status conv3_wgrad(const ConvShape & s, const bf16 * x, int cin, const bf16 * dz, int cout,
                        float * partial, float * dw, cudaStream_t st, int path)
{
  if (!valid_channels(cin, true) || !valid_channels(cout, false)) {
    set_error("conv3_wgrad: unsupported channel counts");
    return DOMA_BAD_INPUT;
  }
  int bmo, bni, tiles, splits;
  long long per;
  wgrad_plan(s, cin, cout, bmo, bni, tiles, splits, per);
  static const bool mma_only = [] {
    const char * e = std::getenv("DOMA_CONV_PATH");
    return e && std::string(e) == "mma";
  }();
  const bool tc_ok = conv3_wgrad_tc_supported(s, cin, cout);
  if (path == DOMA_CONV_TENSOR_MEMORY && !tc_ok) {
    set_error("conv3_wgrad: shape not supported by the tensor-memory kernel");
    return DOMA_BAD_INPUT;
  }
  if (tc_ok && (path == DOMA_CONV_TENSOR_MEMORY || (path == DOMA_CONV_AUTO && !mma_only))) {
    // tensor cores: partials within the same scratch (at most the MMA plan's splits)
    int tc_splits = 0;
    const int room = std::max(splits, conv3_wgrad_tc_splits(s, cin, cout));  // conv3_wgrad_scratch
    DOMA_TRY(conv3_wgrad_tc(s, x, cin, dz, cout, partial, room, &tc_splits, st));
    const size_t count = (size_t)27 * cin * cout;
    reduce_splits_kernel<<<blocks_for((long long)count), 256, 0, st>>>(partial, tc_splits, count, dw);
    DOMA_CUDA_TRY(cudaGetLastError());
    return DOMA_OK;
  }
  WgradArgs a{x, dz, partial, s.nz, s.ny, s.nx, (long long)s.voxels(), cin, cout, per, cin / bni};
  doma_status r;
  if (bmo == 32) {
    if (bni == 16) r = launch_wgrad<32, 16>(a, tiles, splits, st);
    else if (bni == 32) r = launch_wgrad<32, 32>(a, tiles, splits, st);
    else r = launch_wgrad<32, 64>(a, tiles, splits, st);
  } else {
    if (bni == 16) r = launch_wgrad<64, 16>(a, tiles, splits, st);
    else if (bni == 32) r = launch_wgrad<64, 32>(a, tiles, splits, st);
    else r = launch_wgrad<64, 64>(a, tiles, splits, st);
  }
  if (r != DOMA_OK) return r;
  const size_t count = (size_t)27 * cin * cout;
  reduce_splits_kernel<<<blocks_for((long long)count), 256, 0, st>>>(partial, splits, count, dw);
  DOMA_CUDA_TRY(cudaGetLastError());
  return DOMA_OK;
}

doma_status avgpool2(const ConvShape & f, int c, const bf16 * x, bf16 * y, cudaStream_t st)
{
  const long long cv = (long long)f.voxels() / 8;
  avgpool2_kernel<<<blocks_for(cv * c / 8), 256, 0, st>>>(Grid5{f.nz, f.ny, f.nx}, cv, c, x, y);
  DOMA_CUDA_TRY(cudaGetLastError());
  return DOMA_OK;
}

doma_status sumpool2(const ConvShape & f, int c, const bf16 * x, bf16 * y, cudaStream_t st)
{
  const long long cv = (long long)f.voxels() / 8;
  sumpool2_kernel<<<blocks_for(cv * c / 8), 256, 0, st>>>(Grid5{f.nz, f.ny, f.nx}, cv, c, x, y);
  DOMA_CUDA_TRY(cudaGetLastError());
  return DOMA_OK;
}

doma_status up_add_relu(const ConvShape & f, int c, const bf16 * coarse, const bf16 * skip,
                        bf16 * u, cudaStream_t st)
{
  const long long v = (long long)f.voxels();
  up_add_relu_kernel<<<blocks_for(v * c / 8), 256, 0, st>>>(Grid5{f.nz, f.ny, f.nx}, v, c, coarse,
                                                            skip, u);
  DOMA_CUDA_TRY(cudaGetLastError());
  return DOMA_OK;
}

doma_status pool_back_add_mask(const ConvShape & f, int c, const bf16 * g_pool,
                               const bf16 * g_skip, const bf16 * y, bf16 * out, cudaStream_t st)
{
  const long long v = (long long)f.voxels();
  pool_back_add_mask_kernel<<<blocks_for(v * c / 8), 256, 0, st>>>(Grid5{f.nz, f.ny, f.nx}, v, c,
                                                                   g_pool, g_skip, y, out);
  DOMA_CUDA_TRY(cudaGetLastError());
  return DOMA_OK;
}

doma_status relu_mask(size_t count, bf16 * g, const bf16 * y, cudaStream_t st)
{
  relu_mask_kernel<<<blocks_for((long long)(count / 8)), 256, 0, st>>>(count / 8, g, y);
  DOMA_CUDA_TRY(cudaGetLastError());
  return DOMA_OK;
}

size_t bias_grad_scratch(int c) { return (size_t)kReduceBlocks * c; }

doma_status bias_grad(size_t voxels, int c, const bf16 * g, float * partial, float * db,
                      cudaStream_t st)
{
  const int threads = 256;  // a multiple of every channel count <= 256
  if (c % 8 || threads % (c / 8)) {
    set_error("bias_grad: the channel count must be a multiple of 8 with c / 8 dividing 256");
    return DOMA_BAD_INPUT;
  }
  // shared memory: [threads / (c / 8) voxel lanes][c] floats = threads * 8 floats
  bias_grad_kernel<<<kReduceBlocks, threads, threads * 8 * sizeof(float), st>>>((long long)voxels, c, g,
                                                                           partial);
  DOMA_CUDA_TRY(cudaGetLastError());
  sum_blocks_kernel<<<(c + 7) / 8, 256, 0, st>>>(partial, kReduceBlocks, c, db);
  DOMA_CUDA_TRY(cudaGetLastError());
  return DOMA_OK;
}

doma_status head_forward(size_t voxels, int c, const bf16 * x, const float * w, const float * b,
                         float * out, cudaStream_t st)
{
  head_forward_kernel<<<blocks_for((long long)voxels), 256, 0, st>>>((long long)voxels, c, x, w, b,
                                                                     out);
  DOMA_CUDA_TRY(cudaGetLastError());
  return DOMA_OK;
}

size_t head_backward_scratch(int c) { return (size_t)kReduceBlocks * (c + 2); }

doma_status head_backward(size_t voxels, int c, const bf16 * x, const float * w, const float * out,
                          const float * target, bf16 * dx, float * dw, float * db,
                          double * partial, double * loss, cudaStream_t st,
                          const float * sample_weight, size_t per_sample)
{
  if (c > 32 || c % 8) {
    set_error("head_backward: the head takes at most 32 channels");
    return DOMA_BAD_INPUT;
  }
  const int threads = 128;
  head_backward_kernel<<<kReduceBlocks, threads, threads * (c + 2) * sizeof(double), st>>>(
      (long long)voxels, c, x, w, out, target, dx, partial, sample_weight,
      (long long)std::max<size_t>(per_sample, 1));
  DOMA_CUDA_TRY(cudaGetLastError());
  head_finish_kernel<<<1, 64, 0, st>>>(partial, kReduceBlocks, c, (long long)voxels, dw, db, loss);
  DOMA_CUDA_TRY(cudaGetLastError());
  return DOMA_OK;
}

doma_status publish_weights(const float * w32, int cin, int cout, bf16 * w, bf16 * wt,
                            cudaStream_t st)
{
  publish_kernel<<<blocks_for(27LL * cin * cout), 256, 0, st>>>(w32, cin, cout, w, wt);
  DOMA_CUDA_TRY(cudaGetLastError());
  return DOMA_OK;
}

doma_status adam_update(size_t count, float * p, const float * g, float * m, float * v, float lr,
                        float beta1, float beta2, float eps, int step, cudaStream_t st)
{
  const float bc1 = 1.0f - std::pow(beta1, (float)step);
  const float bc2 = 1.0f - std::pow(beta2, (float)step);
  adam_kernel<<<blocks_for((long long)count), 256, 0, st>>>(count, p, g, m, v, lr, beta1, beta2,
                                                            eps, bc1, bc2);
  DOMA_CUDA_TRY(cudaGetLastError());
  return DOMA_OK;
}

}  // namespace doma
