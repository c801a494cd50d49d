// conv_tc.cu -- the 3x3x3 BF16 convolution on the 5th-generation tensor
// cores: tcgen05.mma with the FP32 accumulator in tensor memory, operands
// staged by TMA.
//
// One CTA computes a 128-voxel x cout tile (M = 128, N = cout <= 256) of
// y = act(conv(x, w) + b).  The reduction runs over 27 taps x input-channel
// chunks of KC (64, 32 or 16 channels = one 128/64/32-byte swizzle row):
//   * A, the shifted input tile of one (tap, chunk) step, is one TMA load of
//     a 5D box {KC channels, bx, by, bz, bb} of the channels-last tensor at
//     the tile origin plus the tap's offset.  Boxes that reach outside the
//     volume are zero-filled by TMA -- that is the convolution's padding.
//     The box lands as 128 rows (voxels, x fastest) of KC channels in the
//     swizzled K-major layout the MMA reads.
//   * B, the tap's weight slab w[tap][n0 .. n0+N][chunk], is a 2D TMA load.
//   * KC / 16 tcgen05.mma (kind::f16, M=128, N, K=16) per step accumulate
//     into N TMEM columns; each step's commit releases its smem stage.
// Warp roles: warp 0 issues TMA, warp 1 owns TMEM and issues the MMAs, warps
// 2-5 (one per TMEM lane quarter) drain the accumulator: tcgen05.ld, bias,
// ReLU, bf16 pack, store.  Every mbarrier wait is bounded; a wait that gives
// up sets an error flag (read by conv3_tc_error) and the CTA still releases
// its tensor memory before it exits.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstdlib>
#include <string>
#include <mutex>

#include "conv.cuh"

namespace doma {

namespace {

using bf16 = __nv_bfloat16;

__device__ int g_tc_error = 0;

constexpr int kThreads = 192;
// Pipeline stages per CTA fill about 48 KB: four or five CTAs per SM for the
// 32- and 64-channel slices, whose prologue, pipeline fill and epilogue then
// overlap other CTAs' main loops (100 KB, two per SM, was 6 % slower at batch
// 1 and 19 % at batch 8 on the U-Net at 64^3); at least two stages always.
constexpr int kSmemBudget = 48 * 1024;

__device__ __forceinline__ uint32_t saddr(const void * p)
{
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t * bar, uint32_t count)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(saddr(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t * bar, uint32_t bytes)
{
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(saddr(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t * bar, uint32_t parity)
{
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(saddr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait for the completion of phase `parity`; false after about a
// second of polling (then the error flag is set).
__device__ bool mbar_wait(uint64_t * bar, uint32_t parity)
{
  for (uint32_t i = 0; i < (1u << 24); ++i) {
    if (mbar_try_wait(bar, parity)) return true;
    if (i >= 64) __nanosleep(64);
  }
  atomicExch(&g_tc_error, 1);
  return false;
}

__device__ __forceinline__ void tma_load_5d(void * dst, const CUtensorMap * map, uint64_t * bar,
                                            int c0, int c1, int c2, int c3, int c4)
{
  asm volatile(
      "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes "
      "[%0], [%1, {%3, %4, %5, %6, %7}], [%2];" ::"r"(saddr(dst)),
      "l"(map), "r"(saddr(bar)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4)
      : "memory");
}

__device__ __forceinline__ void tma_load_2d(void * dst, const CUtensorMap * map, uint64_t * bar,
                                            int c0, int c1)
{
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes "
      "[%0], [%1, {%3, %4}], [%2];" ::"r"(saddr(dst)),
      "l"(map), "r"(saddr(bar)), "r"(c0), "r"(c1)
      : "memory");
}

// Shared-memory matrix descriptor of a K-major swizzled tile: start address,
// leading byte offset 16 (unused by swizzled K-major layouts), stride byte
// offset between 8-row groups, descriptor version 1, swizzle mode.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t sbo, uint32_t mode)
{
  uint64_t d = (uint64_t)((addr & 0x3FFFFu) >> 4);
  d |= (uint64_t)1u << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1u << 46;
  d |= (uint64_t)mode << 61;
  return d;
}

// Instruction descriptor, kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, N >> 3 at bit 17, M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N)
{
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc,
                                          uint32_t accumulate)
{
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void umma_commit(uint64_t * bar)
{
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          saddr(bar))
      : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32])
{
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
        "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
        "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

struct TcArgs {
  const float * bias;
  bf16 * y;
  float * partial;            // split reduction: FP32 partials [splits][voxels][cout], else null
  long long voxels;           // batch * nz * ny * nx
  int nz, ny, nx;             // volume extents
  int bx, by, bz, bb;         // voxel box of one tile (bx*by*bz*bb = 128)
  int tx, ty, tz;             // tiles per axis
  int cin, cout;
  int splits;                 // the (tap, chunk) steps are cut into this many contiguous ranges
};

template <int N, int KC, bool RELU>
__global__ void __launch_bounds__(kThreads, 1)
    conv3_tc_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                    const TcArgs a)
{
  constexpr int BM = 128;
  constexpr int A_BYTES = BM * KC * 2, B_BYTES = N * KC * 2, STAGE = A_BYTES + B_BYTES;
  constexpr int STAGES = std::max(2, std::min(8, kSmemBudget / STAGE));
  constexpr uint32_t SW = KC * 2;                       // swizzle span in bytes
  constexpr uint32_t MODE = KC == 64 ? 2u : (KC == 32 ? 4u : 6u);  // 128B / 64B / 32B
  constexpr uint32_t SBO = 8 * SW;
  constexpr uint32_t TMEM_COLS = N;
  constexpr uint32_t IDESC = idesc_bf16(BM, N);
  static_assert(N >= 32 && N <= 256 && (N & (N - 1)) == 0, "N");
  static_assert(A_BYTES % 1024 == 0 && B_BYTES % 1024 == 0, "tile alignment");

  extern __shared__ uint8_t smem_raw[];
  uint8_t * smem = smem_raw + ((1024u - (saddr(smem_raw) & 1023u)) & 1023u);
  uint64_t * full = reinterpret_cast<uint64_t *>(smem + STAGES * STAGE);
  uint64_t * empty = full + STAGES;
  uint64_t * tmem_full = empty + STAGES;
  uint32_t * tmem_slot = reinterpret_cast<uint32_t *>(tmem_full + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (warp == 0 && lane == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(full + s, 1);
      mbar_init(empty + s, 1);
    }
    mbar_init(tmem_full, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __shared__ int s_issued, s_consumed;
  if (threadIdx.x == 0) s_issued = s_consumed = 0;
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     saddr(tmem_slot)),
                 "r"(TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  // tile origin
  int t = blockIdx.x;
  const int x0 = (t % a.tx) * a.bx;
  t /= a.tx;
  const int y0 = (t % a.ty) * a.by;
  t /= a.ty;
  const int z0 = (t % a.tz) * a.bz;
  const int b0 = (t / a.tz) * a.bb;
  const int steps_per_tap = a.cin / KC;
  const int k_steps = 27 * steps_per_tap;
  // this CTA's range of (tap, chunk) steps: all of them unless the reduction is split
  const int split = (int)blockIdx.z;
  const int kb = (int)((long long)split * k_steps / a.splits);
  const int kn = (int)((long long)(split + 1) * k_steps / a.splits) - kb;

  if (warp == 0) {
    if (lane == 0) {
      asm volatile("prefetch.tensormap [%0];" ::"l"(&tmA) : "memory");
      asm volatile("prefetch.tensormap [%0];" ::"l"(&tmB) : "memory");
      int j = 0;
      for (; j < kn; ++j) {
        const int s = j % STAGES;
        const uint32_t use = (uint32_t)(j / STAGES);
        if (j >= STAGES && !mbar_wait(empty + s, (use & 1u) ^ 1u)) break;
        const int ks = kb + j;
        const int tap = ks / steps_per_tap, c0 = (ks % steps_per_tap) * KC;
        const int dz = tap / 9 - 1, dy = (tap / 3) % 3 - 1, dx = tap % 3 - 1;
        uint8_t * As = smem + s * STAGE;
        mbar_expect_tx(full + s, (uint32_t)STAGE);
        tma_load_5d(As, &tmA, full + s, c0, x0 + dx, y0 + dy, z0 + dz, b0);
        tma_load_2d(As + A_BYTES, &tmB, full + s, c0, tap * a.cout + (int)blockIdx.y * N);
      }
      s_issued = j;
    }
  } else if (warp == 1) {
    if (lane == 0) {
      int j = 0;
      for (; j < kn; ++j) {
        const int s = j % STAGES;
        const uint32_t use = (uint32_t)(j / STAGES);
        if (!mbar_wait(full + s, use & 1u)) break;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t a_addr = saddr(smem + s * STAGE);
        const uint32_t b_addr = a_addr + A_BYTES;
#pragma unroll
        for (int k = 0; k < KC / 16; ++k) {
          const uint64_t ad = smem_desc(a_addr + k * 32, SBO, MODE);
          const uint64_t bd = smem_desc(b_addr + k * 32, SBO, MODE);
          umma_bf16(tmem, ad, bd, IDESC, (j | k) != 0 ? 1u : 0u);
        }
        umma_commit(empty + s);
      }
      s_consumed = j;
      umma_commit(tmem_full);  // also after a failed wait, so the epilogue is released
    }
  } else {
    // epilogue: warps 2..5 cover TMEM lane quarters 2, 3, 0, 1
    const int q = warp & 3;
    int ok = 0;
    if (lane == 0) ok = mbar_wait(tmem_full, 0) ? 1 : 0;
    ok = __shfl_sync(0xffffffffu, ok, 0);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const int row = q * 32 + lane;
    int r = row;
    const int x = r % a.bx;
    r /= a.bx;
    const int yy = r % a.by;
    r /= a.by;
    const int zz = r % a.bz;
    const int bb = r / a.bz;
    const long long vox =
        (((long long)(b0 + bb) * a.nz + (z0 + zz)) * a.ny + (y0 + yy)) * a.nx + (x0 + x);
    if (a.partial) {
      // split reduction: this range's FP32 sums, summed in split order by conv_split_reduce
      float * outp = a.partial + ((long long)split * a.voxels + vox) * a.cout + (int)blockIdx.y * N;
#pragma unroll 1
      for (int c0 = 0; ok && c0 < N; c0 += 32) {
        uint32_t v[32];
        tmem_ld32(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)c0, v);
        uint4 * dst = reinterpret_cast<uint4 *>(outp + c0);
#pragma unroll
        for (int j = 0; j < 8; ++j) dst[j] = make_uint4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
      }
      ok = 0;
    }
    bf16 * out = a.y + vox * a.cout + (int)blockIdx.y * N;
    const float * bias = a.bias ? a.bias + (int)blockIdx.y * N : nullptr;
#pragma unroll 1
    for (int c0 = 0; ok && c0 < N; c0 += 32) {
      uint32_t v[32];
      tmem_ld32(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)c0, v);
      uint4 pk[4];
      uint32_t * pw = reinterpret_cast<uint32_t *>(pk);
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        float f0 = __uint_as_float(v[2 * j]), f1 = __uint_as_float(v[2 * j + 1]);
        if (bias) {
          f0 += __ldg(bias + c0 + 2 * j);
          f1 += __ldg(bias + c0 + 2 * j + 1);
        }
        if (RELU) {
          f0 = fmaxf(f0, 0.0f);
          f1 = fmaxf(f1, 0.0f);
        }
        const __nv_bfloat162 h = __floats2bfloat162_rn(f0, f1);
        pw[j] = *reinterpret_cast<const uint32_t *>(&h);
      }
      uint4 * dst = reinterpret_cast<uint4 *>(out + c0);
#pragma unroll
      for (int j = 0; j < 4; ++j) dst[j] = pk[j];
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  // Teardown after a failed wait: let this CTA's own copies and MMAs in
  // flight land (bounded) before its shared and tensor memory go away.
  if (threadIdx.x == 0)
    for (int i = s_consumed; i < s_issued; ++i)
      mbar_wait(full + i % STAGES, (uint32_t)(i / STAGES) & 1u);
  if (threadIdx.x == 32) mbar_wait(tmem_full, 0);
  __syncthreads();
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(TMEM_COLS));
  }
}

PFN_cuTensorMapEncodeTiled_v12000 encoder()
{
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void * p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

CUtensorMapSwizzle swizzle_for(int kc)
{
  return kc == 64 ? CU_TENSOR_MAP_SWIZZLE_128B
                  : (kc == 32 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_32B);
}

template <int N, int KC, bool RELU>
doma_status launch_tc(const CUtensorMap & ma, const CUtensorMap & mb, const TcArgs & a, int tiles,
                      cudaStream_t st)
{
  constexpr int STAGE = 128 * KC * 2 + N * KC * 2;
  constexpr int STAGES = std::max(2, std::min(8, kSmemBudget / STAGE));
  constexpr int smem = STAGES * STAGE + 1024 + (2 * STAGES + 2) * 8;
  static bool configured = false;
  if (!configured) {
    DOMA_CUDA_TRY(cudaFuncSetAttribute(conv3_tc_kernel<N, KC, RELU>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    configured = true;
  }
  conv3_tc_kernel<N, KC, RELU>
      <<<dim3((unsigned)tiles, (unsigned)(a.cout / N), (unsigned)a.splits), kThreads, smem, st>>>(ma, mb,
                                                                                                 a);
  DOMA_CUDA_TRY(cudaGetLastError());
  return DOMA_OK;
}

template <int N, int KC>
doma_status launch_tc_act(const CUtensorMap & ma, const CUtensorMap & mb, const TcArgs & a,
                          int tiles, bool relu, cudaStream_t st)
{
  return relu ? launch_tc<N, KC, true>(ma, mb, a, tiles, st)
              : launch_tc<N, KC, false>(ma, mb, a, tiles, st);
}

template <int KC>
doma_status dispatch_n(const CUtensorMap & ma, const CUtensorMap & mb, const TcArgs & a, int n,
                       int tiles, bool relu, cudaStream_t st)
{
  switch (n) {
    case 32: return launch_tc_act<32, KC>(ma, mb, a, tiles, relu, st);
    case 64: return launch_tc_act<64, KC>(ma, mb, a, tiles, relu, st);
    case 128: return launch_tc_act<128, KC>(ma, mb, a, tiles, relu, st);
    default: return launch_tc_act<256, KC>(ma, mb, a, tiles, relu, st);
  }
}

// y = act(sum over splits of the FP32 partials + bias), the splits added in
// order; four channels per thread.
__global__ void conv_split_reduce_kernel(const float4 * __restrict__ p, int splits, size_t count4,
                                         int cout, const float * __restrict__ bias, int relu,
                                         uint2 * __restrict__ y)
{
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < count4;
       i += (size_t)gridDim.x * blockDim.x) {
    float4 acc = p[i];
    for (int sp = 1; sp < splits; ++sp) {
      const float4 v = p[(size_t)sp * count4 + i];
      acc.x += v.x;
      acc.y += v.y;
      acc.z += v.z;
      acc.w += v.w;
    }
    if (bias) {
      const int c = (int)((i * 4) % (size_t)cout);
      acc.x += bias[c];
      acc.y += bias[c + 1];
      acc.z += bias[c + 2];
      acc.w += bias[c + 3];
    }
    if (relu) {
      acc.x = fmaxf(acc.x, 0.0f);
      acc.y = fmaxf(acc.y, 0.0f);
      acc.z = fmaxf(acc.z, 0.0f);
      acc.w = fmaxf(acc.w, 0.0f);
    }
    const __nv_bfloat162 lo = __floats2bfloat162_rn(acc.x, acc.y);
    const __nv_bfloat162 hi = __floats2bfloat162_rn(acc.z, acc.w);
    y[i] = make_uint2(*reinterpret_cast<const uint32_t *>(&lo), *reinterpret_cast<const uint32_t *>(&hi));
  }
}

// ---- weight gradient on the tensor cores ------------------------------------------
//
// dw[tap][co][ci] = sum over voxels m of x[m + offset(tap)][ci] * dz[m][co].
// One GEMM per tap with K = voxels.  The rows (M = 128) stack several taps of
// one input-channel block: 128 / ci_blk taps of ci_blk channels (8 taps of 16
// channels, 4 of 32, 2 of 64, or one of 128), so that even the 16- and
// 32-channel layers fill a 128-row MMA.  N = cout.  Both operands come from
// TMA boxes of the channels-last activations -- a box of SPAN channels over a
// 128-voxel brick, the tap's shift applied to the brick's (x, y, z)
// coordinates as in the forward kernel (zero fill outside the volume) -- so
// the channels are the contiguous (MN) dimension and the voxels the K rows:
// MN-major operands (instruction-descriptor bits 15 and 16).  In the
// canonical MN-major swizzled layout an atom is 8 K rows of SPAN channels;
// SBO steps 8 rows, LBO steps from one SPAN-channel block (one box) to the
// next along M or N.  Each CTA covers one (tap group, channel block) over a
// contiguous range of voxel bricks and writes its FP32 sums as partials
// [split][tap][co][ci], which are added in split order afterwards
// (deterministic).

// Shared-memory descriptor of an MN-major swizzled tile.
__device__ __forceinline__ uint64_t smem_desc_mn(uint32_t addr, uint32_t lbo, uint32_t sbo,
                                                 uint32_t mode)
{
  uint64_t d = (uint64_t)((addr & 0x3FFFFu) >> 4);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1u << 46;
  d |= (uint64_t)mode << 61;
  return d;
}

struct WgArgs {
  float * partial;            // [splits][27][cout][cin]
  long long bricks;           // 128-voxel bricks in the volume
  int bx, by, bz, bb;         // voxel brick (bx*by*bz*bb = 128)
  int tx, ty, tz;             // bricks per axis
  int cin, cout;
  int ci_blk;                 // input channels of one block (16, 32, 64 or 128)
  int tpg;                    // taps per group: 128 / ci_blk
  int groups;                 // tap groups: ceil(27 / tpg)
  int splits;
};

constexpr uint32_t swizzle_mode(int span_bytes)
{
  return span_bytes == 128 ? 2u : (span_bytes == 64 ? 4u : 6u);
}

// Two pipeline stages per CTA; with N <= 64 two CTAs share an SM (their
// prologues and epilogues overlap each other's main loops), wider N take one.
constexpr int kWgStages = 2;
constexpr int wg_stage_bytes(int n) { return 128 * 128 * 2 + 128 * n * 2; }
constexpr int wg_smem_bytes(int n) { return kWgStages * wg_stage_bytes(n) + 1024 + (2 * kWgStages + 2) * 8; }
constexpr int wg_ctas_per_sm(int n) { return n <= 64 ? 2 : 1; }

template <int SPAN_A, int N>
__global__ void __launch_bounds__(kThreads, wg_ctas_per_sm(N))
    conv3_wgrad_tc_kernel(const __grid_constant__ CUtensorMap tmX,
                          const __grid_constant__ CUtensorMap tmD, const WgArgs a)
{
  constexpr int SPAN_B = N < 64 ? N : 64;            // dz channels per box
  constexpr int NBA = 128 / SPAN_A, NBB = N / SPAN_B;
  constexpr int A_BOX = 128 * SPAN_A * 2, B_BOX = 128 * SPAN_B * 2;
  constexpr int A_BYTES = NBA * A_BOX, B_BYTES = NBB * B_BOX, STAGE = A_BYTES + B_BYTES;
  constexpr int STAGES = kWgStages;
  constexpr uint32_t SBO_A = 8 * SPAN_A * 2, SBO_B = 8 * SPAN_B * 2;
  constexpr uint32_t MODE_A = swizzle_mode(SPAN_A * 2), MODE_B = swizzle_mode(SPAN_B * 2);
  constexpr uint32_t IDESC = idesc_bf16(128, N) | (1u << 15) | (1u << 16);
  static_assert(A_BYTES == 128 * 128 * 2, "A stage: 128 rows x 128 voxels");
  static_assert(STAGE == wg_stage_bytes(N), "stage layout");

  extern __shared__ uint8_t smem_raw[];
  uint8_t * smem = smem_raw + ((1024u - (saddr(smem_raw) & 1023u)) & 1023u);
  uint64_t * full = reinterpret_cast<uint64_t *>(smem + STAGES * STAGE);
  uint64_t * empty = full + STAGES;
  uint64_t * tmem_full = empty + STAGES;
  uint32_t * tmem_slot = reinterpret_cast<uint32_t *>(tmem_full + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (warp == 0 && lane == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(full + s, 1);
      mbar_init(empty + s, 1);
    }
    mbar_init(tmem_full, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __shared__ int s_issued, s_consumed;
  if (threadIdx.x == 0) s_issued = s_consumed = 0;
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     saddr(tmem_slot)),
                 "r"((uint32_t)N));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  const int g = (int)blockIdx.x % a.groups;          // tap group
  const int cb = (int)blockIdx.x / a.groups;         // input-channel block
  const int split = (int)blockIdx.y;
  const long long k0 = (long long)split * a.bricks / a.splits;
  const int kn = (int)((long long)(split + 1) * a.bricks / a.splits - k0);
  const int bpt = a.ci_blk / SPAN_A;                 // A boxes per tap
  // A boxes that carry a tap (the last group may have fewer than tpg taps)
  const int taps_here = min(a.tpg, 27 - g * a.tpg);
  const int boxes_a = taps_here * bpt;

  if (warp == 0) {
    if (lane == 0) {
      asm volatile("prefetch.tensormap [%0];" ::"l"(&tmX) : "memory");
      asm volatile("prefetch.tensormap [%0];" ::"l"(&tmD) : "memory");
      int j = 0;
      for (; j < kn; ++j) {
        const int s = j % STAGES;
        const uint32_t use = (uint32_t)(j / STAGES);
        if (j >= STAGES && !mbar_wait(empty + s, (use & 1u) ^ 1u)) break;
        long long t = k0 + j;
        const int x0 = (int)(t % a.tx) * a.bx;
        t /= a.tx;
        const int y0 = (int)(t % a.ty) * a.by;
        t /= a.ty;
        const int z0 = (int)(t % a.tz) * a.bz;
        const int b0 = (int)(t / a.tz) * a.bb;
        uint8_t * As = smem + s * STAGE;
        uint8_t * Bs = As + A_BYTES;
        mbar_expect_tx(full + s, (uint32_t)(boxes_a * A_BOX + B_BYTES));
        for (int b = 0; b < boxes_a; ++b) {
          const int tap = g * a.tpg + b / bpt;
          const int c0 = cb * a.ci_blk + (b % bpt) * SPAN_A;
          const int dz = tap / 9 - 1, dy = (tap / 3) % 3 - 1, dx = tap % 3 - 1;
          tma_load_5d(As + b * A_BOX, &tmX, full + s, c0, x0 + dx, y0 + dy, z0 + dz, b0);
        }
        for (int b = 0; b < NBB; ++b)
          tma_load_5d(Bs + b * B_BOX, &tmD, full + s, b * SPAN_B, x0, y0, z0, b0);
      }
      s_issued = j;
    }
  } else if (warp == 1) {
    if (lane == 0) {
      int j = 0;
      for (; j < kn; ++j) {
        const int s = j % STAGES;
        const uint32_t use = (uint32_t)(j / STAGES);
        if (!mbar_wait(full + s, use & 1u)) break;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t a_addr = saddr(smem + s * STAGE);
        const uint32_t b_addr = a_addr + A_BYTES;
#pragma unroll
        for (int k = 0; k < 8; ++k) {   // 16 voxels (two 8-row atoms) per MMA
          const uint64_t ad = smem_desc_mn(a_addr + k * 2 * SBO_A, A_BOX, SBO_A, MODE_A);
          const uint64_t bd = smem_desc_mn(b_addr + k * 2 * SBO_B, B_BOX, SBO_B, MODE_B);
          umma_bf16(tmem, ad, bd, IDESC, (j | k) != 0 ? 1u : 0u);
        }
        umma_commit(empty + s);
      }
      s_consumed = j;
      umma_commit(tmem_full);  // also after a failed wait, so the epilogue is released
    }
  } else {
    // epilogue: warps 2..5 cover TMEM lane quarters 2, 3, 0, 1; row = (tap slot, channel)
    const int q = warp & 3;
    int ok = 0;
    if (lane == 0) ok = mbar_wait(tmem_full, 0) ? 1 : 0;
    ok = __shfl_sync(0xffffffffu, ok, 0) && kn > 0;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const int row = q * 32 + lane;
    const int tap = g * a.tpg + row / a.ci_blk;
    const int ci = cb * a.ci_blk + row % a.ci_blk;
    float * out = a.partial + ((long long)split * 27 + tap) * a.cout * (long long)a.cin + ci;
#pragma unroll 1
    for (int c0 = 0; ok && c0 < N; c0 += 32) {
      uint32_t v[32];
      tmem_ld32(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)c0, v);
      if (tap < 27) {
#pragma unroll
        for (int j = 0; j < 32; ++j) out[(long long)(c0 + j) * a.cin] = __uint_as_float(v[j]);
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  // Teardown after a failed wait: let this CTA's own copies and MMAs in
  // flight land (bounded) before its shared and tensor memory go away.
  if (threadIdx.x == 0)
    for (int i = s_consumed; i < s_issued; ++i)
      mbar_wait(full + i % STAGES, (uint32_t)(i / STAGES) & 1u);
  if (threadIdx.x == 32) mbar_wait(tmem_full, 0);
  __syncthreads();
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"((uint32_t)N));
  }
}

template <int SPAN_A, int N>
doma_status launch_wgrad_tc(const CUtensorMap & mx, const CUtensorMap & md, const WgArgs & a,
                            cudaStream_t st)
{
  constexpr int smem = wg_smem_bytes(N);
  static bool configured = false;
  if (!configured) {
    DOMA_CUDA_TRY(cudaFuncSetAttribute(conv3_wgrad_tc_kernel<SPAN_A, N>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    configured = true;
  }
  conv3_wgrad_tc_kernel<SPAN_A, N><<<dim3((unsigned)(a.groups * (a.cin / a.ci_blk)),
                                          (unsigned)a.splits), kThreads, smem, st>>>(mx, md, a);
  DOMA_CUDA_TRY(cudaGetLastError());
  return DOMA_OK;
}

template <int SPAN_A>
doma_status dispatch_wgrad_n(const CUtensorMap & mx, const CUtensorMap & md, const WgArgs & a,
                             cudaStream_t st)
{
  switch (a.cout) {
    case 32: return launch_wgrad_tc<SPAN_A, 32>(mx, md, a, st);
    case 64: return launch_wgrad_tc<SPAN_A, 64>(mx, md, a, st);
    case 128: return launch_wgrad_tc<SPAN_A, 128>(mx, md, a, st);
    default: return launch_wgrad_tc<SPAN_A, 256>(mx, md, a, st);
  }
}

// ---- halo-tile forward convolution (16- and 32-channel inputs) ------------------
//
// For inputs of at most 32 channels the tile's A operand is staged once per
// tile instead of once per tap: the CTA loads the output brick's halo --
// (8 + 2) x (16 + 2) x 3 voxels around an 8 x 16 x 1 brick -- as one TMA box
// per 8-channel group, unswizzled, so each plane is [z][y][x] x 16 bytes.  In
// the canonical K-major layout without swizzle a core matrix is 8 rows x 16
// bytes: here 8 consecutive x of one y row.  The 128 rows of the brick are 16
// such core matrices one halo row (10 voxels, 160 B = SBO) apart, the K
// dimension steps from one 8-channel plane to the next (LBO = plane stride),
// and tap (dz, dy, dx) starts ((dz+1) 180 + (dy+1) 10 + (dx+1)) x 16 bytes into
// the halo.  So 27 taps read 540 staged rows per 8 channels, against
// 27 x 128 = 3,456 for one shifted box per tap.  The weights of all 27 taps
// (27 x cout x cin, at most 108 KB) stay resident: the CTA is persistent over
// output bricks, the halo stages are triple-buffered, and the accumulator is
// double-buffered in tensor memory so a brick's epilogue overlaps the next
// brick's MMAs.  Each brick accumulates tap by tap in the same order as
// conv3_tc_kernel (one channel chunk), so the sums are the same.

constexpr int kHaloPlane = 8704;    // 10 x 18 x 3 x 16 B = 8640, padded to 128 B
constexpr int kHaloStages = 3;

__device__ __forceinline__ void tma_load_3d(void * dst, const CUtensorMap * map, uint64_t * bar,
                                            int c0, int c1, int c2)
{
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes "
      "[%0], [%1, {%3, %4, %5}], [%2];" ::"r"(saddr(dst)),
      "l"(map), "r"(saddr(bar)), "r"(c0), "r"(c1), "r"(c2)
      : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t * bar)
{
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(saddr(bar)) : "memory");
}

struct HaloArgs {
  const float * bias;
  bf16 * y;
  int nz, ny, nx;
  int tiles_x, tiles_y;       // nx / 8, ny / 16
  long long tiles;            // batch * nz * tiles_y * tiles_x
};

template <int KC, int N>
constexpr int halo_smem_bytes()
{
  return 27 * N * KC * 2 + kHaloStages * (KC / 8) * kHaloPlane + 1024 + 16 * 8;
}

template <int KC, int N, bool RELU>
__global__ void __launch_bounds__(kThreads, 1)
    conv3_halo_kernel(const __grid_constant__ CUtensorMap tmX, const __grid_constant__ CUtensorMap tmW,
                      const HaloArgs a)
{
  constexpr int PLANES = KC / 8;
  constexpr int A_STAGE = PLANES * kHaloPlane;
  constexpr int B_TAP = N * KC * 2;
  constexpr int B_BYTES = 27 * B_TAP;
  constexpr uint32_t MODE_B = KC == 32 ? 4u : 6u;      // 64- or 32-byte swizzle rows
  constexpr uint32_t SBO_B = 8 * KC * 2;
  constexpr uint32_t IDESC = idesc_bf16(128, N);
  constexpr uint32_t TMEM_COLS = 2 * N;
  static_assert(B_BYTES % 1024 == 0, "the halo stages start 1024-byte aligned");

  extern __shared__ uint8_t smem_raw[];
  uint8_t * smem = smem_raw + ((1024u - (saddr(smem_raw) & 1023u)) & 1023u);
  uint8_t * Bsm = smem;
  uint8_t * Asm = smem + B_BYTES;
  uint64_t * bars = reinterpret_cast<uint64_t *>(Asm + kHaloStages * A_STAGE);
  uint64_t * b_full = bars;
  uint64_t * full = bars + 1;
  uint64_t * empty = full + kHaloStages;
  uint64_t * tfull = empty + kHaloStages;             // [2]
  uint64_t * tempty = tfull + 2;                      // [2]
  uint32_t * tmem_slot = reinterpret_cast<uint32_t *>(tempty + 2);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (warp == 0 && lane == 0) {
    mbar_init(b_full, 1);
    for (int s = 0; s < kHaloStages; ++s) {
      mbar_init(full + s, 1);
      mbar_init(empty + s, 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(tfull + b, 1);
      mbar_init(tempty + b, 128);   // every epilogue thread arrives
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __shared__ int s_issued, s_consumed, s_committed;
  if (threadIdx.x == 0) s_issued = s_consumed = s_committed = 0;
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     saddr(tmem_slot)),
                 "r"(TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;
  // this CTA's bricks: blockIdx.x, blockIdx.x + gridDim.x, ...
  const int my = (int)((a.tiles - blockIdx.x + gridDim.x - 1) / gridDim.x);

  if (warp == 0) {
    if (lane == 0) {
      asm volatile("prefetch.tensormap [%0];" ::"l"(&tmX) : "memory");
      asm volatile("prefetch.tensormap [%0];" ::"l"(&tmW) : "memory");
      mbar_expect_tx(b_full, (uint32_t)B_BYTES);
      tma_load_3d(Bsm, &tmW, b_full, 0, 0, 0);
      int i = 0;
      for (; i < my; ++i) {
        const int s = i % kHaloStages;
        const uint32_t use = (uint32_t)(i / kHaloStages);
        if (i >= kHaloStages && !mbar_wait(empty + s, (use & 1u) ^ 1u)) break;
        long long t = blockIdx.x + (long long)i * gridDim.x;
        const int x0 = (int)(t % a.tiles_x) * 8;
        t /= a.tiles_x;
        const int y0 = (int)(t % a.tiles_y) * 16;
        t /= a.tiles_y;
        const int z0 = (int)(t % a.nz);
        const int b0 = (int)(t / a.nz);
        uint8_t * As = Asm + s * A_STAGE;
        mbar_expect_tx(full + s, (uint32_t)(PLANES * 8640));
        for (int p = 0; p < PLANES; ++p)
          tma_load_5d(As + p * kHaloPlane, &tmX, full + s, p * 8, x0 - 1, y0 - 1, z0 - 1, b0);
      }
      s_issued = i;
    }
  } else if (warp == 1) {
    if (lane == 0) {
      int i = 0;
      bool ok = mbar_wait(b_full, 0);
      for (; ok && i < my; ++i) {
        const int s = i % kHaloStages, buf = i & 1;
        const uint32_t use = (uint32_t)(i / kHaloStages);
        if (!mbar_wait(full + s, use & 1u)) break;
        if (i >= 2 && !mbar_wait(tempty + buf, (uint32_t)((i >> 1) - 1) & 1u)) {
          s_consumed = i;   // stage s landed but is not used
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t a_addr = saddr(Asm + s * A_STAGE);
        const uint32_t b_addr = saddr(Bsm);
        const uint32_t d = tmem + (uint32_t)(buf * N);
        for (int tap = 0; tap < 27; ++tap) {
          const uint32_t off = (uint32_t)(((tap / 9) * 180 + ((tap / 3) % 3) * 10 + tap % 3) * 16);
#pragma unroll
          for (int k = 0; k < KC / 16; ++k) {
            const uint64_t ad = smem_desc_mn(a_addr + off + k * 2 * kHaloPlane, kHaloPlane, 160, 0u);
            const uint64_t bd = smem_desc(b_addr + tap * B_TAP + k * 32, SBO_B, MODE_B);
            umma_bf16(d, ad, bd, IDESC, (tap | k) != 0 ? 1u : 0u);
          }
        }
        umma_commit(empty + s);
        umma_commit(tfull + buf);
        s_committed = i + 1;
      }
      if (ok) s_consumed = i;
    }
  } else {
    // epilogue: warps 2..5 cover TMEM lane quarters 2, 3, 0, 1
    const int q = warp & 3;
    const int row = q * 32 + lane;
    for (int i = 0; i < my; ++i) {
      const int buf = i & 1;
      int ok = 0;
      if (lane == 0) ok = mbar_wait(tfull + buf, (uint32_t)(i >> 1) & 1u) ? 1 : 0;
      ok = __shfl_sync(0xffffffffu, ok, 0);
      if (!ok) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      long long t = blockIdx.x + (long long)i * gridDim.x;
      const int x0 = (int)(t % a.tiles_x) * 8;
      t /= a.tiles_x;
      const int y0 = (int)(t % a.tiles_y) * 16;
      t /= a.tiles_y;
      const int z0 = (int)(t % a.nz);
      const long long b0 = t / a.nz;
      const long long vox = ((b0 * a.nz + z0) * a.ny + (y0 + row / 8)) * a.nx + (x0 + row % 8);
      bf16 * out = a.y + vox * N;
#pragma unroll 1
      for (int c0 = 0; c0 < N; c0 += 32) {
        uint32_t v[32];
        tmem_ld32(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(buf * N + c0), v);
        uint4 pk[4];
        uint32_t * pw = reinterpret_cast<uint32_t *>(pk);
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          float f0 = __uint_as_float(v[2 * j]), f1 = __uint_as_float(v[2 * j + 1]);
          if (a.bias) {
            f0 += __ldg(a.bias + c0 + 2 * j);
            f1 += __ldg(a.bias + c0 + 2 * j + 1);
          }
          if (RELU) {
            f0 = fmaxf(f0, 0.0f);
            f1 = fmaxf(f1, 0.0f);
          }
          const __nv_bfloat162 h = __floats2bfloat162_rn(f0, f1);
          pw[j] = *reinterpret_cast<const uint32_t *>(&h);
        }
        uint4 * dst = reinterpret_cast<uint4 *>(out + c0);
#pragma unroll
        for (int j = 0; j < 4; ++j) dst[j] = pk[j];
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      mbar_arrive(tempty + buf);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  // Teardown after a failed wait: let this CTA's own copies and MMAs in
  // flight land (bounded) before its shared and tensor memory go away.
  if (threadIdx.x == 0) {
    mbar_wait(b_full, 0);
    for (int i = s_consumed; i < s_issued; ++i)
      mbar_wait(full + i % kHaloStages, (uint32_t)(i / kHaloStages) & 1u);
  }
  if (threadIdx.x == 32 && s_committed > 0) {
    const int last = s_committed - 1;
    mbar_wait(tfull + (last & 1), (uint32_t)(last >> 1) & 1u);
  }
  __syncthreads();
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(TMEM_COLS));
  }
}

int sm_count();

template <int KC, int N, bool RELU>
doma_status launch_halo(const CUtensorMap & mx, const CUtensorMap & mw, const HaloArgs & a,
                        cudaStream_t st)
{
  constexpr int smem = halo_smem_bytes<KC, N>();
  static bool configured = false;
  if (!configured) {
    DOMA_CUDA_TRY(cudaFuncSetAttribute(conv3_halo_kernel<KC, N, RELU>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    configured = true;
  }
  const unsigned grid = (unsigned)std::min<long long>(a.tiles, (long long)sm_count());
  conv3_halo_kernel<KC, N, RELU><<<grid, kThreads, smem, st>>>(mx, mw, a);
  DOMA_CUDA_TRY(cudaGetLastError());
  return DOMA_OK;
}

template <int KC, int N>
doma_status launch_halo_act(const CUtensorMap & mx, const CUtensorMap & mw, const HaloArgs & a,
                            bool relu, cudaStream_t st)
{
  return relu ? launch_halo<KC, N, true>(mx, mw, a, st) : launch_halo<KC, N, false>(mx, mw, a, st);
}

int sm_count()
{
  static int n = 0;
  static std::once_flag once;
  std::call_once(once, [] {
    int dev = 0, v = 0;
    if (cudaGetDevice(&dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && v > 0)
      n = v;
    else
      n = 148;
  });
  return n;
}

// How one convolution is cut into CTAs.  Shapes with few 128-voxel tiles (the
// coarse U-Net levels) would leave most SMs idle: the output channels are cut
// into N-wide slices first (down to 64; the same sums, the same bits); if that
// still leaves SMs idle, the (tap, chunk) steps are cut into `splits` ranges
// whose FP32 partials a second kernel adds in order.  A range keeps at least
// four steps.
struct TcPlan {
  int n = 0, splits = 1;
};

TcPlan tc_plan(const ConvShape & s, int cin, int cout, size_t scratch_floats)
{
  const long long tiles = (long long)(s.voxels() / 128);
  const long long target = 2LL * sm_count();
  TcPlan p;
  p.n = cout;
  while (p.n > 64 && tiles * (cout / p.n) < target) p.n >>= 1;
  const long long ctas = tiles * (cout / p.n);
  const int kc = cin >= 64 ? 64 : cin;
  const int k_steps = 27 * (cin / kc);
  if (ctas < sm_count()) {
    p.splits = (int)std::min<long long>((target + ctas - 1) / ctas, std::max(1, k_steps / 4));
    while (p.splits > 1 && (size_t)p.splits * s.voxels() * (size_t)cout > scratch_floats) --p.splits;
  }
  return p;
}

}  // namespace

size_t conv3_tc_split_scratch(const ConvShape & s, int cin, int cout)
{
  if (!conv3_tc_supported(s, cin, cout)) return 0;
  const TcPlan p = tc_plan(s, cin, cout, SIZE_MAX);
  return p.splits > 1 ? (size_t)p.splits * s.voxels() * (size_t)cout : 0;
}

bool conv3_tc_supported(const ConvShape & s, int cin, int cout)
{
  if (!(cin == 16 || cin == 32 || cin % 64 == 0) || cin > 256) return false;
  if (!(cout == 32 || cout == 64 || cout == 128 || cout == 256)) return false;
  if (s.voxels() % 128 != 0) return false;
  // the 128-voxel box must tile the volume exactly
  const int bx = std::min(s.nx, 128);
  if (s.nx % bx) return false;
  const int by = std::min(s.ny, 128 / bx);
  if (s.ny % by || (128 / bx) % by) return false;
  const int bz = std::min(s.nz, 128 / (bx * by));
  if (s.nz % bz || (128 / (bx * by)) % bz) return false;
  const int bb = 128 / (bx * by * bz);
  if (bx * by * bz * bb != 128 || s.batch % bb) return false;
  return encoder() != nullptr;
}

bool conv3_halo_supported(const ConvShape & s, int cin, int cout)
{
  return (cin == 16 || cin == 32) && (cout == 32 || cout == 64) && s.nx % 8 == 0 &&
         s.ny % 16 == 0 && s.nz >= 1 && s.batch >= 1 && encoder() != nullptr;
}

// Where the halo kernel is the faster one.  Its planes are 16-byte rows (8
// channels of a voxel), which TMA moves row by row with 32-byte sectors: for
// 16-channel inputs that still beats 27 shifted boxes (24 vs 52 us for the
// 64^3 input layer on GB300), for 32-channel inputs it does not (58 vs 53 us),
// so those keep the per-tap kernel.  DOMA_CONV_HALO=1 forces it wherever it
// applies (tests), 0 turns it off.
bool conv3_halo_preferred(const ConvShape & s, int cin, int cout)
{
  static const int mode = [] {
    const char * e = std::getenv("DOMA_CONV_HALO");
    return e ? std::atoi(e) : -1;
  }();
  if (mode == 0 || !conv3_halo_supported(s, cin, cout)) return false;
  return mode == 1 || cin == 16;
}

// The halo-tile kernel for one convolution (conv3_halo_supported shapes).
doma_status conv3_forward_halo(const ConvShape & s, const bf16 * x, int cin, const bf16 * w,
                               const float * bias, int cout, bool relu, bf16 * y, cudaStream_t st)
{
  HaloArgs a{};
  a.bias = bias;
  a.y = y;
  a.nz = s.nz;
  a.ny = s.ny;
  a.nx = s.nx;
  a.tiles_x = s.nx / 8;
  a.tiles_y = s.ny / 16;
  a.tiles = (long long)s.batch * s.nz * a.tiles_y * a.tiles_x;
  const cuuint32_t estr[5] = {1, 1, 1, 1, 1};
  CUtensorMap mx, mw;
  {
    const cuuint64_t gdim[5] = {(cuuint64_t)cin, (cuuint64_t)s.nx, (cuuint64_t)s.ny,
                                (cuuint64_t)s.nz, (cuuint64_t)s.batch};
    const cuuint64_t row = (cuuint64_t)cin * 2;
    const cuuint64_t gstr[4] = {row, row * s.nx, row * s.nx * s.ny, row * s.nx * s.ny * s.nz};
    const cuuint32_t box[5] = {8, 10, 18, 3, 1};   // one 8-channel plane of the brick's halo
    const CUresult r = encoder()(&mx, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<bf16 *>(x),
                                 gdim, gstr, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                 CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                                 CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
      set_error("cuTensorMapEncodeTiled (halo) failed: " + std::to_string((int)r));
      return DOMA_CUDA_ERROR;
    }
  }
  {
    const cuuint64_t gdim[3] = {(cuuint64_t)cin, (cuuint64_t)cout, 27};
    const cuuint64_t gstr[2] = {(cuuint64_t)cin * 2, (cuuint64_t)cin * cout * 2};
    const cuuint32_t box[3] = {(cuuint32_t)cin, (cuuint32_t)cout, 27};   // every tap's weights
    const CUresult r = encoder()(&mw, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<bf16 *>(w),
                                 gdim, gstr, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                 swizzle_for(cin), CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                                 CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
      set_error("cuTensorMapEncodeTiled (halo weights) failed: " + std::to_string((int)r));
      return DOMA_CUDA_ERROR;
    }
  }
  if (cin == 32) {
    if (cout == 32) return launch_halo_act<32, 32>(mx, mw, a, relu, st);
    return launch_halo_act<32, 64>(mx, mw, a, relu, st);
  }
  if (cout == 32) return launch_halo_act<16, 32>(mx, mw, a, relu, st);
  return launch_halo_act<16, 64>(mx, mw, a, relu, st);
}

doma_status conv3_forward_tc(const ConvShape & s, const bf16 * x, int cin, const bf16 * w,
                             const float * bias, int cout, bool relu, bf16 * y, cudaStream_t st,
                             ConvScratch scratch)
{
  if (!scratch.p) scratch.floats = 0;
  if (conv3_halo_preferred(s, cin, cout))
    return conv3_forward_halo(s, x, cin, w, bias, cout, relu, y, st);
  if (!conv3_tc_supported(s, cin, cout)) {
    set_error("conv3_forward_tc: shape not supported by the tensor-memory kernel");
    return DOMA_BAD_INPUT;
  }
  const int kc = cin >= 64 ? 64 : cin;
  TcArgs a{};
  a.bias = bias;
  a.y = y;
  a.nz = s.nz;
  a.ny = s.ny;
  a.nx = s.nx;
  a.bx = std::min(s.nx, 128);
  a.by = std::min(s.ny, 128 / a.bx);
  a.bz = std::min(s.nz, 128 / (a.bx * a.by));
  a.bb = 128 / (a.bx * a.by * a.bz);
  a.tx = s.nx / a.bx;
  a.ty = s.ny / a.by;
  a.tz = s.nz / a.bz;
  a.cin = cin;
  a.cout = cout;
  a.voxels = (long long)s.voxels();
  const int tiles = a.tx * a.ty * a.tz * (s.batch / a.bb);
  const TcPlan plan = tc_plan(s, cin, cout, scratch.floats);
  a.splits = plan.splits;
  a.partial = plan.splits > 1 ? scratch.p : nullptr;

  CUtensorMap ma, mb;
  const cuuint64_t gdim_a[5] = {(cuuint64_t)cin, (cuuint64_t)s.nx, (cuuint64_t)s.ny,
                                (cuuint64_t)s.nz, (cuuint64_t)s.batch};
  const cuuint64_t row = (cuuint64_t)cin * 2;
  const cuuint64_t gstr_a[4] = {row, row * s.nx, row * s.nx * s.ny, row * s.nx * s.ny * s.nz};
  const cuuint32_t box_a[5] = {(cuuint32_t)kc, (cuuint32_t)a.bx, (cuuint32_t)a.by,
                               (cuuint32_t)a.bz, (cuuint32_t)a.bb};
  const cuuint32_t estr[5] = {1, 1, 1, 1, 1};
  CUresult r = encoder()(&ma, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<bf16 *>(x), gdim_a,
                         gstr_a, box_a, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle_for(kc),
                         CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error("cuTensorMapEncodeTiled (activations) failed: " + std::to_string((int)r));
    return DOMA_CUDA_ERROR;
  }
  const cuuint64_t gdim_b[2] = {(cuuint64_t)cin, (cuuint64_t)27 * cout};
  const cuuint64_t gstr_b[1] = {row};
  // one CTA's slice: N output channels of one tap
  const cuuint32_t box_b[2] = {(cuuint32_t)kc, (cuuint32_t)plan.n};
  r = encoder()(&mb, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<bf16 *>(w), gdim_b, gstr_b,
                box_b, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle_for(kc),
                CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error("cuTensorMapEncodeTiled (weights) failed: " + std::to_string((int)r));
    return DOMA_CUDA_ERROR;
  }
  if (kc == 64) DOMA_TRY(dispatch_n<64>(ma, mb, a, plan.n, tiles, relu, st));
  else if (kc == 32) DOMA_TRY(dispatch_n<32>(ma, mb, a, plan.n, tiles, relu, st));
  else DOMA_TRY(dispatch_n<16>(ma, mb, a, plan.n, tiles, relu, st));
  if (a.partial) {
    const size_t count4 = s.voxels() * (size_t)cout / 4;
    const unsigned blocks = (unsigned)std::min<size_t>((count4 + 255) / 256, (size_t)sm_count() * 8);
    conv_split_reduce_kernel<<<blocks, 256, 0, st>>>(reinterpret_cast<const float4 *>(a.partial),
                                                     a.splits, count4, cout, bias, relu ? 1 : 0,
                                                     reinterpret_cast<uint2 *>(y));
    DOMA_CUDA_TRY(cudaGetLastError());
  }
  return DOMA_OK;
}

bool conv3_wgrad_tc_supported(const ConvShape & s, int cin, int cout)
{
  if (!(cin == 16 || cin == 32 || cin == 64 || cin == 128 || cin == 256)) return false;
  return conv3_tc_supported(s, cin, cout);
}

int conv3_wgrad_tc_splits(const ConvShape & s, int cin, int cout)
{
  if (!conv3_wgrad_tc_supported(s, cin, cout)) return 0;
  const int ci_blk = std::min(cin, 128);
  const int tpg = 128 / ci_blk;
  const int ctas = ((27 + tpg - 1) / tpg) * (cin / ci_blk);
  const long long bricks = (long long)(s.voxels() / 128);
  // whole waves: as many splits as fill the resident CTA slots once, at
  // least two bricks per split
  const long long slots = (long long)sm_count() * wg_ctas_per_sm(cout);
  long long want = std::max<long long>(1, slots / ctas);
  want = std::min<long long>(want, std::max<long long>(1, bricks / 2));
  return (int)want;
}

doma_status conv3_wgrad_tc(const ConvShape & s, const bf16 * x, int cin, const bf16 * dz, int cout,
                           float * partial, int max_splits, int * splits_out, cudaStream_t st)
{
  if (!conv3_wgrad_tc_supported(s, cin, cout)) {
    set_error("conv3_wgrad_tc: shape not supported by the tensor-memory kernel");
    return DOMA_BAD_INPUT;
  }
  WgArgs a{};
  a.partial = partial;
  a.bx = std::min(s.nx, 128);
  a.by = std::min(s.ny, 128 / a.bx);
  a.bz = std::min(s.nz, 128 / (a.bx * a.by));
  a.bb = 128 / (a.bx * a.by * a.bz);
  a.tx = s.nx / a.bx;
  a.ty = s.ny / a.by;
  a.tz = s.nz / a.bz;
  a.bricks = (long long)(s.voxels() / 128);
  a.cin = cin;
  a.cout = cout;
  a.ci_blk = std::min(cin, 128);
  a.tpg = 128 / a.ci_blk;
  a.groups = (27 + a.tpg - 1) / a.tpg;
  a.splits = std::max(1, std::min(conv3_wgrad_tc_splits(s, cin, cout), std::max(1, max_splits)));
  const int span_a = std::min(a.ci_blk, 64), span_b = std::min(cout, 64);
  CUtensorMap mx, md;
  const cuuint32_t estr[5] = {1, 1, 1, 1, 1};
  {
    const cuuint64_t gdim[5] = {(cuuint64_t)cin, (cuuint64_t)s.nx, (cuuint64_t)s.ny,
                                (cuuint64_t)s.nz, (cuuint64_t)s.batch};
    const cuuint64_t row = (cuuint64_t)cin * 2;
    const cuuint64_t gstr[4] = {row, row * s.nx, row * s.nx * s.ny, row * s.nx * s.ny * s.nz};
    const cuuint32_t box[5] = {(cuuint32_t)span_a, (cuuint32_t)a.bx, (cuuint32_t)a.by,
                               (cuuint32_t)a.bz, (cuuint32_t)a.bb};
    const CUresult r = encoder()(&mx, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<bf16 *>(x),
                                 gdim, gstr, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                 swizzle_for(span_a), CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                                 CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
      set_error("cuTensorMapEncodeTiled (wgrad activations) failed: " + std::to_string((int)r));
      return DOMA_CUDA_ERROR;
    }
  }
  {
    const cuuint64_t gdim[5] = {(cuuint64_t)cout, (cuuint64_t)s.nx, (cuuint64_t)s.ny,
                                (cuuint64_t)s.nz, (cuuint64_t)s.batch};
    const cuuint64_t row = (cuuint64_t)cout * 2;
    const cuuint64_t gstr[4] = {row, row * s.nx, row * s.nx * s.ny, row * s.nx * s.ny * s.nz};
    const cuuint32_t box[5] = {(cuuint32_t)span_b, (cuuint32_t)a.bx, (cuuint32_t)a.by,
                               (cuuint32_t)a.bz, (cuuint32_t)a.bb};
    const CUresult r = encoder()(&md, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<bf16 *>(dz),
                                 gdim, gstr, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                 swizzle_for(span_b), CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                                 CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
      set_error("cuTensorMapEncodeTiled (wgrad output gradient) failed: " + std::to_string((int)r));
      return DOMA_CUDA_ERROR;
    }
  }
  if (span_a == 64) DOMA_TRY(dispatch_wgrad_n<64>(mx, md, a, st));
  else if (span_a == 32) DOMA_TRY(dispatch_wgrad_n<32>(mx, md, a, st));
  else DOMA_TRY(dispatch_wgrad_n<16>(mx, md, a, st));
  if (splits_out) *splits_out = a.splits;
  return DOMA_OK;
}

doma_status conv3_tc_error(int * flag)
{
  DOMA_CUDA_TRY(cudaMemcpyFromSymbol(flag, g_tc_error, sizeof(int)));
  return DOMA_OK;
}

doma_status conv3_tc_error_reset(cudaStream_t st)
{
  void * p = nullptr;
  DOMA_CUDA_TRY(cudaGetSymbolAddress(&p, g_tc_error));
  DOMA_CUDA_TRY(cudaMemsetAsync(p, 0, sizeof(int), st));
  return DOMA_OK;
}

}  // namespace doma
