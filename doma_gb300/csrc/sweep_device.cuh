// sweep_device.cuh -- device helpers shared by the sweep kernels (sweep.cu,
// sweep_warp.cu): the single-precision cell solves, the done-flag and
// tagged-face-word primitives of the task hand-off.
#pragma once

#include "common.cuh"

namespace doma {
namespace sweep_dev {

// ---- single-precision cell solves ------------------------------------------
// Every operation is an explicit intrinsic (separately rounded add/mul, fused
// multiply-add where written), so the compiler has no contraction choices and
// the bits do not depend on which kernel the solve is inlined into.
//
// The cell balance is written divided by the cell volume, with the per-axis
// streaming coefficients hx = |mu|/dx, hy = |eta|/dy, hz = |xi|/dz (DD uses
// their doubles 2|mu|/dx, ...).  This is the same equation as DOMA's
// (include/DiamondDifference3D.h:28-48, include/TWDiamondDifference3D.h:32-91),
// rearranged so that the volume and face areas cancel.

__device__ __forceinline__ float fA(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fS(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fM(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fF(float a, float b, float c) { return __fmaf_rn(a, b, c); }

// One MUFU reciprocal (approximate, flush-to-zero; every argument here is a
// normal number).
__device__ __forceinline__ float rcp_approx(float a)
{
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(a));
  return r;
}

// DD: psi = (q + cx x + cy y + cz z) / (cx + cy + cz + st), cyz = cy + cz.
__device__ __forceinline__ float dd3_fast(float q, float st, float cx, float cy, float cz,
                                          float cyz, float & x, float & y, float & z)
{
  const float num = fF(cz, z, fF(cy, y, fF(cx, x, q)));
  const float c = fM(num, rcp_approx(fA(fA(cx, cyz), st)));
  x = fF(2.0f, c, -x);
  y = fF(2.0f, c, -y);
  z = fF(2.0f, c, -z);
  return c;
}

__device__ __forceinline__ float dd2_fast(float q, float st, float cx, float cy, float & x,
                                          float & y)
{
  const float c = fM(fF(cy, y, fF(cx, x, q)), rcp_approx(fA(fA(cx, cy), st)));
  x = fF(2.0f, c, -x);
  y = fF(2.0f, c, -y);
  return c;
}

// Reciprocal r = 1/a of one TW-DD axis weight.  DOMA's weight is
// a = 1 - n / (D flux) when the upwind flux exceeds 1e-8 (else 0.5), clamped
// to [0.5, 1] (include/TWDiamondDifference3D.h:43-75).  With Dx = D flux > 0,
// 1/a = Dx / (Dx - n): a >= 1 <-> r <= 1, a in [0.5, 1] <-> r in [1, 2],
// a < 0.5 (including a <= 0, Dx - n <= 0) <-> r = 2 after the clamp; the
// floor 1e-30 on Dx - n sends a <= 0 to the r = 2 side.  r is clamped to
// [1, 2] as 1 + sat(r - 1).
__device__ __forceinline__ float tw_rweight(float n, float D, float flux)
{
  const float dx = fM(D, flux);
  const float den = fmaxf(fS(dx, n), 1e-30f);
  const float r = fA(1.0f, __saturatef(fF(dx, rcp_approx(den), -1.0f)));
  return flux > 1e-8f ? r : 2.0f;
}

// TW-DD, volume-normalized.  With X = hx x, Y = hy y, Z = hz z and
// B = theta (q + X + Y + Z), the weight numerators are B + (1 - theta) X etc.
// and the denominators (st + 2 hy + 2 hz) x etc. (DOMA's, divided by V).
// psi = (q + rx X + ry Y + rz Z) / (st + hx rx + hy ry + hz rz) and the
// outgoing faces x' = (psi - (1 - a) x) / a = x + rx (psi - x).
// sz = st + 2 hz and sy = st + 2 hy, syz = st + 2 hy + 2 hz.
__device__ __forceinline__ float twdd3_fast(float q, float st, float hx, float hy, float hz,
                                            float th, float om, float & x, float & y, float & z)
{
  const float X = fM(hx, x), Y = fM(hy, y), Z = fM(hz, z);
  const float B = fF(th, fA(fA(X, Y), Z), fM(th, q));
  const float h2x = fA(hx, hx), h2y = fA(hy, hy), h2z = fA(hz, hz);
  const float ra = tw_rweight(fF(om, X, B), fA(fA(st, h2y), h2z), x);
  const float rb = tw_rweight(fF(om, Y, B), fA(fA(st, h2z), h2x), y);
  const float rc = tw_rweight(fF(om, Z, B), fA(fA(st, h2y), h2x), z);
  const float num = fF(rc, Z, fF(rb, Y, fF(ra, X, q)));
  const float den = fF(hz, rc, fF(hy, rb, fF(hx, ra, st)));
  const float c = fM(num, rcp_approx(den));
  x = fF(ra, fS(c, x), x);
  y = fF(rb, fS(c, y), y);
  z = fF(rc, fS(c, z), z);
  return c;
}

// 2D TW-DD keeps DOMA's bare |xi| term in the y weight
// (include/TWDiamondDifference2D.h:51), volume-normalized: theta |xi| / V,
// passed in as txv.
__device__ __forceinline__ float twdd2_fast(float q, float st, float hx, float hy, float txv,
                                            float th, float om, float & x, float & y)
{
  const float X = fM(hx, x), Y = fM(hy, y);
  const float B = fF(th, fA(X, Y), fM(th, q));
  const float ra = tw_rweight(fF(om, X, B), fA(st, fA(hy, hy)), x);
  const float rb = tw_rweight(fA(fF(om, Y, B), txv), fA(st, fA(hx, hx)), y);
  const float num = fF(rb, Y, fF(ra, X, q));
  const float den = fF(hy, rb, fF(hx, ra, st));
  const float c = fM(num, rcp_approx(den));
  x = fF(ra, fS(c, x), x);
  y = fF(rb, fS(c, y), y);
  return c;
}

// ---- scheduling primitives -------------------------------------------------

__device__ __forceinline__ void st_release(unsigned * p, unsigned v)
{
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ unsigned ld_acquire(const unsigned * p)
{
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ int ld_relaxed(const int * p)
{
  int v;
  asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Wait until *flag == epoch.  Bounded: the first 32 polls are back to back,
// then back-off of 32..128 ns; after `limit` polls it records
// DOMA_DEVICE_WAIT_TIMEOUT in *error and returns false.  It also gives up at
// once when another CTA has already failed.
static __device__ bool wait_for(const unsigned * flag, unsigned epoch, unsigned limit, int * error)
{
  unsigned ns = 32;
  for (unsigned it = 0; it < limit; ++it) {
    if (ld_acquire(flag) == epoch) return true;
    if (ld_relaxed(error) != 0) return false;
    if (it >= 32) {
      __nanosleep(ns);
      if (ns < 128) ns *= 2;
    }
  }
  atomicCAS(error, 0, (int)DOMA_DEVICE_WAIT_TIMEOUT);
  return false;
}

// Tagged face words (single precision).  A face travels between tasks as one
// 8-byte word: the float value in the low 32 bits and a tag in the high 32
// bits, the sweep's epoch (low 16 bits) over the index of the producing
// block along the face's axis.  Aligned 8-byte accesses are single-copy
// atomic, so a reader that sees the tag it expects also sees that producer's
// value, with no fence and no separate flag (the scheme of NCCL's
// low-latency "LL" buffers).  The producer index matters: the blocks along an
// axis write the same face slots in turn, so while block b waits for block
// b - 1 a slot can still hold the word of block b - 2 (or b - 3, ...) of the
// same sweep.  Every sweep rewrites every slot it reads, and the planes start
// zeroed with epochs from 1, so an older word never carries the tag expected.
__device__ __forceinline__ unsigned face_tag(unsigned epoch, int block)
{
  return (epoch << 16) | ((unsigned)block & 0xffffu);
}

// (a plain aligned 8-byte store: one untorn write, which the compiler schedules
// freely among the wavefront's shared-memory accesses; readers use relaxed
// loads that bypass L1)
__device__ __forceinline__ void st_tagged(unsigned long long * p, float v, unsigned tag)
{
  *p = ((unsigned long long)tag << 32) | __float_as_uint(v);
}

__device__ __forceinline__ unsigned long long ld_tagged(const unsigned long long * p)
{
  unsigned long long w;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(w) : "l"(p));
  return w;
}

__device__ __forceinline__ void ld_tagged2(const unsigned long long * p, unsigned long long & a,
                                           unsigned long long & b)
{
  asm volatile("ld.relaxed.gpu.global.v2.u64 {%0, %1}, [%2];" : "=l"(a), "=l"(b) : "l"(p));
}

__device__ __forceinline__ void st_relaxed(unsigned * p, unsigned v)
{
  asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ unsigned ld_relaxed_u32(const unsigned * p)
{
  unsigned v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// wait_for with relaxed loads (the single-precision hand-off checks its data
// words itself, so the flag needs no acquire)
static __device__ bool wait_flag_relaxed(const unsigned * flag, unsigned epoch, unsigned limit, int * error)
{
  unsigned ns = 32;
  for (unsigned it = 0; it < limit; ++it) {
    if (ld_relaxed_u32(flag) == epoch) return true;
    if ((it & 15) == 15 && ld_relaxed(error) != 0) return false;
    if (it >= 16) {
      __nanosleep(ns);
      if (ns < 128) ns *= 2;
    }
  }
  atomicCAS(error, 0, (int)DOMA_DEVICE_WAIT_TIMEOUT);
  return false;
}

__device__ __forceinline__ unsigned tag_of(unsigned long long w) { return (unsigned)(w >> 32); }
__device__ __forceinline__ float value_of(unsigned long long w) { return __uint_as_float((unsigned)w); }

}  // namespace sweep_dev
}  // namespace doma
