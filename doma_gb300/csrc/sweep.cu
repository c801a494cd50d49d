// sweep.cu -- the transport sweep: DD / TW-DD cell solves over hyperplane
// wavefronts, all ordinates of an octant in flight, all octants concurrently.
//
// Replaces TransportSolver3D::sweep / parallelSweepOctant / sweepPPP..MMM
// (src/TransportSolver3D.cpp:565-874) and the cell policies
// DiamondDifference3D / TWDiamondDifference3D (include/DiamondDifference3D.h:14-49,
// include/TWDiamondDifference3D.h:15-92), plus their 2D twins
// (src/TransportSolver2D.cpp:567-725, include/DiamondDifference2D.h:14-45,
// include/TWDiamondDifference2D.h:15-76).
//
// Decomposition.  The mesh, seen in each octant's sweep frame (every axis
// running downwind), is cut into TX x TY x TZ cell blocks.  One CTA solves one
// (octant, block) task for all ordinates of that octant: thread (n, jl, kl)
// owns ordinate n and the x-pencil (jl, kl) of the block and walks it cell by
// cell on a skewed schedule (cell il at step il + jl + kl), so every step is a
// hyperplane i+j+k = const of the block and one __syncthreads separates
// dependent hyperplanes.  The x face stays in a register; y and z faces live
// in shared memory (one slot per (kl, il) and (jl, il), written by one thread
// and read by its downwind neighbour on the next step).  Faces crossing a
// block boundary go through per-octant global face planes, one slot per face
// position, read only after the upstream block has published them.
//
// Scheduling.  A persistent grid (the CTAs that fit on the device) claims
// tasks from a ticket counter in level order (level = bi + bj + bk, all
// octants interleaved), stages the task's cell data, waits -- bounded, with
// an acquire load -- for the done flags of its upstream blocks, and publishes
// its own done flag (the sweep's epoch number) with a release store.  The
// last CTA to leave re-arms the counters, so consecutive sweeps need no
// host work.  A level-synchronous variant (one launch per level, ordering by
// kernel boundaries) runs the same task body and is kept for cross-checks.
//
// Arithmetic.
//   * double ("exact"): each cell solve evaluates DOMA's expression with
//     DOMA's association, with __dadd_rn/__dmul_rn/__ddiv_rn so nothing is
//     fused, contracted or approximated; w*psi goes to a per-(cell, ordinate)
//     buffer that a later pass sums in DOMA's single-thread order.  Given the
//     same source, the swept flux is then bit-equal to DOMA's.
//   * float: algebraically simplified solves (precomputed 2|mu|/dx
//     coefficients, one reciprocal), and a compensated (Kahan) sum of w*psi
//     over the ordinates of each cell, stored per octant in double.
#include <type_traits>

#include "common.cuh"

#ifndef DOMA_SWEEP_MIN_CTAS_DD
#define DOMA_SWEEP_MIN_CTAS_DD 8
#endif
#ifndef DOMA_SWEEP_MIN_CTAS_DD_MANY
#define DOMA_SWEEP_MIN_CTAS_DD_MANY 12
#endif
#ifndef DOMA_SWEEP_BATCH_MIN_CTAS_DD
#define DOMA_SWEEP_BATCH_MIN_CTAS_DD 8
#endif
#ifndef DOMA_SWEEP_MIN_CTAS_FP64
#define DOMA_SWEEP_MIN_CTAS_FP64 1
#endif
#ifndef DOMA_SWEEP_MIN_CTAS
#define DOMA_SWEEP_MIN_CTAS 5
#endif
#ifndef DOMA_SWEEP_MIN_CTAS_MANY
#define DOMA_SWEEP_MIN_CTAS_MANY 6
#endif

namespace doma {
namespace {

__device__ __forceinline__ double dA(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dS(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dM(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dD(double a, double b) { return __ddiv_rn(a, b); }

// ---- exact (reference-order) cell solves ----------------------------------

// DiamondDifference3D::solve (include/DiamondDifference3D.h:28-48).
// geo = (2|mu|/lx + 2|eta|/ly) + 2|xi|/lz, precomputed with the same operations.
__device__ __forceinline__ double dd3_exact(double q, double st, double amu, double aeta,
                                            double axi, double lx, double ly, double lz,
                                            double geo, double & x, double & y, double & z)
{
  double c = dA(dA(dA(q, dD(dM(dM(2.0, x), amu), lx)), dD(dM(dM(2.0, y), aeta), ly)),
                dD(dM(dM(2.0, z), axi), lz));
  c = dD(c, dA(geo, st));
  x = dS(dM(2.0, c), x);
  y = dS(dM(2.0, c), y);
  z = dS(dM(2.0, c), z);
  return c;
}

// TWDiamondDifference3D::solve (include/TWDiamondDifference3D.h:29-91), theta
// = theta_s = th.
__device__ __forceinline__ double twdd3_exact(double q, double st, double amu, double aeta,
                                              double axi, double lx, double ly, double lz,
                                              double th, double & x, double & y, double & z)
{
  const double A = dM(ly, lz), B = dM(lx, lz), C = dM(lx, ly);
  const double V = dM(dM(lx, ly), lz);
  const double xu = x, yu = y, zu = z;
  const double qV = dM(q, V), qVt = dM(qV, th), sV = dM(st, V);
  const double muA = dM(amu, A), etB = dM(aeta, B), xiC = dM(axi, C);
  double a = 0.5;
  if (xu > 1e-8) {
    a = dA(dA(qVt, dM(dA(dM(etB, yu), dM(xiC, zu)), th)), dM(muA, xu));
    a = dD(a, dM(dA(dA(sV, dM(dM(2.0, aeta), B)), dM(dM(2.0, axi), C)), xu));
    a = dM(-1.0, dS(a, 1.0));
  }
  double b = 0.5;
  if (yu > 1e-8) {
    b = dA(dA(qVt, dM(dA(dM(muA, xu), dM(xiC, zu)), th)), dM(etB, yu));
    b = dD(b, dM(dA(dA(sV, dM(dM(2.0, amu), A)), dM(dM(2.0, axi), C)), yu));
    b = dM(-1.0, dS(b, 1.0));
  }
  double cw = 0.5;
  if (zu > 1e-8) {
    cw = dA(dA(qVt, dM(dA(dM(muA, xu), dM(etB, yu)), th)), dM(xiC, zu));
    cw = dD(cw, dM(dA(dA(sV, dM(dM(2.0, amu), A)), dM(dM(2.0, aeta), B)), zu));
    cw = dM(-1.0, dS(cw, 1.0));
  }
  a = a < 0.5 ? 0.5 : a;
  a = a > 1.0 ? 1.0 : a;
  b = b < 0.5 ? 0.5 : b;
  b = b > 1.0 ? 1.0 : b;
  cw = cw < 0.5 ? 0.5 : cw;
  cw = cw > 1.0 ? 1.0 : cw;
  const double ta = dD(muA, a), tb = dD(etB, b), tc = dD(xiC, cw);
  double c = dA(dA(dA(qV, dM(ta, xu)), dM(tb, yu)), dM(tc, zu));
  c = dD(c, dA(dA(dA(sV, ta), tb), tc));
  x = dS(dD(c, a), dM(dD(dS(1.0, a), a), xu));
  y = dS(dD(c, b), dM(dD(dS(1.0, b), b), yu));
  z = dS(dD(c, cw), dM(dD(dS(1.0, cw), cw), zu));
  return c;
}

// DiamondDifference2D::solve (include/DiamondDifference2D.h:28-44).
__device__ __forceinline__ double dd2_exact(double q, double st, double amu, double aeta,
                                            double lx, double ly, double geo, double & x,
                                            double & y)
{
  double c = dA(dA(q, dD(dM(dM(2.0, x), amu), lx)), dD(dM(dM(2.0, y), aeta), ly));
  c = dD(c, dA(geo, st));
  x = dS(dM(2.0, c), x);
  y = dS(dM(2.0, c), y);
  return c;
}

// TWDiamondDifference2D::solve (include/TWDiamondDifference2D.h:32-75),
// including the bare |xi| term of the b weight (:51).
__device__ __forceinline__ double twdd2_exact(double q, double st, double amu, double aeta,
                                              double axi, double lx, double ly, double th,
                                              double & x, double & y)
{
  const double A = ly, B = lx, V = dM(lx, ly);
  const double xu = x, yu = y;
  const double qV = dM(q, V), qVt = dM(qV, th), sV = dM(st, V);
  const double muA = dM(amu, A), etB = dM(aeta, B);
  double a = 0.5;
  if (xu > 1e-8) {
    a = dA(dA(qVt, dM(dM(etB, yu), th)), dM(muA, xu));
    a = dD(a, dM(dA(sV, dM(dM(2.0, aeta), B)), xu));
    a = dM(-1.0, dS(a, 1.0));
  }
  double b = 0.5;
  if (yu > 1e-8) {
    b = dA(dA(qVt, dM(dA(dM(muA, xu), axi), th)), dM(etB, yu));
    b = dD(b, dM(dA(sV, dM(dM(2.0, amu), A)), yu));
    b = dM(-1.0, dS(b, 1.0));
  }
  a = a < 0.5 ? 0.5 : a;
  a = a > 1.0 ? 1.0 : a;
  b = b < 0.5 ? 0.5 : b;
  b = b > 1.0 ? 1.0 : b;
  const double ta = dD(muA, a), tb = dD(etB, b);
  double c = dA(dA(qV, dM(ta, xu)), dM(tb, yu));
  c = dD(c, dA(dA(sV, ta), tb));
  x = dS(dD(c, a), dM(dD(dS(1.0, a), a), xu));
  y = dS(dD(c, b), dM(dD(dS(1.0, b), b), yu));
  return c;
}

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

// Stores under a per-lane predicate, as predicated instructions: the unrolled
// wavefront has no branch (and no reconvergence point) per conditional store.
__device__ __forceinline__ void st_global_if(float * p, float v, bool c)
{
  asm volatile("{\n\t.reg .pred q;\n\tsetp.ne.u32 q, %2, 0;\n\t@q st.global.f32 [%0], %1;\n\t}"
               ::"l"(p), "f"(v), "r"((unsigned)c));
}

__device__ __forceinline__ void st_shared_if(float * p, float v, bool c)
{
  const unsigned a = (unsigned)__cvta_generic_to_shared(p);
  asm volatile("{\n\t.reg .pred q;\n\tsetp.ne.u32 q, %2, 0;\n\t@q st.shared.f32 [%0], %1;\n\t}"
               ::"r"(a), "f"(v), "r"((unsigned)c));
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
__device__ bool wait_for(const unsigned * flag, unsigned epoch, unsigned limit, int * error)
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

// ---- one task: (octant, ordinate group, block) --------------------------------
//
// Lanes are pencil-major: a warp holds two ordinates, each over a 16-pencil
// cross-section of the block (4 x 4 in (y, z) for 3D, 16 in y for 2D), and
// every thread walks its x-pencil on the skewed schedule il = s - jl - kl.
// A cell's y-upwind neighbour is then lane - 1 and its z-upwind neighbour
// lane - PY, both computed on the previous step, so faces move between
// lanes with __shfl_up_sync and the warps advance with no block barrier.
//
// Face planes (sweep frame, ordinate-group major, KG = ordinate_group(precision,
// scheme) slots per face so that one task's faces along a row are contiguous):
//   x [G*8][ngroups][nz][ny][KG], y [G*8][ngroups][nz][nx][KG],
//   z [G*8][ngroups][ny][nx][KG].

template <int DIMS> struct Pencils;
template <> struct Pencils<3> { static constexpr int PY = 4, PZ = 4; };
template <> struct Pencils<2> { static constexpr int PY = 16, PZ = 1; };

template <typename T, int KG>
struct FacePlanes {
  const SweepArgs<T> & A;
  size_t plane;  // (group in flight, octant, ordinate group)
  __device__ FacePlanes(const SweepArgs<T> & a, int of, int og) : A(a), plane((size_t)of * a.ngroups + og) {}
  __device__ size_t x(int k, int j) const { return ((plane * A.nz + k) * A.ny + j) * KG; }
  __device__ size_t y(int k, int i) const { return ((plane * A.nz + k) * A.nx + i) * KG; }
  __device__ size_t z(int j, int i) const { return ((plane * A.ny + j) * A.nx + i) * KG; }
};

// Done flag of block (bk, bj, bi) of a (group, octant, ordinate group) slot.
template <typename T>
__device__ __forceinline__ unsigned * done_flag(const SweepArgs<T> & A, size_t slot, int bk, int bj, int bi)
{
  return A.done + ((slot * A.nbz + bk) * A.nby + bj) * A.nbx + bi;
}

// Wait for the upstream blocks of a task: threads 0, 1, 2 poll the x, y and
// z neighbours' flags concurrently, then the CTA synchronises.
template <typename T, int DIMS>
__device__ __forceinline__ void wait_upstream(const SweepArgs<T> & A, const Task & task, size_t slot,
                                              unsigned epoch)
{
  const int t = threadIdx.x;
  if (t < DIMS) {
    const unsigned * f = nullptr;
    if (t == 0 && task.bi > 0) f = done_flag(A, slot, task.bk, task.bj, task.bi - 1);
    if (t == 1 && task.bj > 0) f = done_flag(A, slot, task.bk, task.bj - 1, task.bi);
    if (t == 2 && task.bk > 0) f = done_flag(A, slot, task.bk - 1, task.bj, task.bi);
    if (f) wait_for(f, epoch + A.wait_bias, A.spin_limit, A.error);
  }
  __syncthreads();
}

// ---- double precision (exact, DOMA's arithmetic) ------------------------------

template <int DIMS, int TX>
struct TaskSmemExact {
  static constexpr int PY = Pencils<DIMS>::PY, PZ = Pencils<DIMS>::PZ;
  static constexpr int CELLS = TX * PY * PZ;
  static constexpr int KG = kGroupExact;                    // ordinate_group(DOMA_PREC_FP64, *)
  static constexpr int YF = PZ * TX * KG;                  // y faces [PZ][TX][KG]
  static constexpr int ZF = DIMS == 3 ? PY * TX * KG : 0;  // z faces [PY][TX][KG]
  static constexpr int NT = 2 * YF + 2 * ZF + 2 * CELLS + TX + PY + PZ + KG * (TX + PY + PZ);
  static constexpr size_t bytes = NT * sizeof(double);
};

template <int DIMS, int SCHEME, int TX>
__device__ __forceinline__ void run_task_exact(const SweepArgs<double> & A, const Task task,
                                               unsigned char * smem_raw, bool dataflow, unsigned epoch)
{
  using T = double;
  using SM = TaskSmemExact<DIMS, TX>;
  constexpr int PY = SM::PY, PZ = SM::PZ, CELLS = SM::CELLS, KG = SM::KG;
  static_assert(KG == ordinate_group(DOMA_PREC_FP64, SCHEME), "one ordinate-group size per mode");
  constexpr unsigned FULL = 0xffffffffu;
  const int og = task.og;
  const int o = task.oct;                 // octant: sweep directions
  const int of = task.grp * 8 + o;        // (group in flight, octant) plane index
  const bool rx = (o & 4) != 0, ry = (o & 2) != 0, rz = (o & 1) != 0;
  const int nx = A.nx, ny = A.ny, nz = DIMS == 3 ? A.nz : 1;
  const size_t N = (size_t)nx * ny * nz;
  const T * gq = A.q + (size_t)task.grp * N;
  const T * gsig = A.sigt + (size_t)task.grp * N;
  const int Do = A.d_oct;
  const int n0 = og * KG;
  const int gs = min(KG, Do - n0);
  const int i0 = task.bi * TX, j0 = task.bj * PY, k0 = task.bk * PZ;
  const int vx = min(TX, nx - i0), vy = min(PY, ny - j0), vz = min(PZ, nz - k0);
  const FacePlanes<T, KG> F(A, of, og);

  const int t = threadIdx.x;
  const int lane = t & 31;
  const int p = lane & 15;
  const int nl = (t >> 5) * 2 + (lane >> 4);
  const int jl = DIMS == 3 ? (p & 3) : p;
  const int kl = DIMS == 3 ? (p >> 2) : 0;
  const bool active = nl < gs && jl < vy && kl < vz;
  const int ob = A.oct_offset[o] + n0;        // first global ordinate of the group
  const int ord = ob + min(nl, gs - 1);

  T * yin = reinterpret_cast<T *>(smem_raw);
  T * yout = yin + SM::YF;
  T * zin = yout + SM::YF;
  T * zout = zin + SM::ZF;
  T * qs = zout + SM::ZF;
  T * ss = qs + CELLS;
  T * lxs = ss + CELLS;
  T * lys = lxs + TX;
  T * lzs = lys + PY;
  T * cxs = lzs + PZ;                 // [KG][TX]
  T * cys = cxs + KG * TX;        // [KG][PY]
  T * czs = cys + KG * PY;        // [KG][PZ]

  auto phys_i = [&](int il) { return rx ? nx - 1 - (i0 + il) : i0 + il; };
  auto phys_j = [&](int jj) { return ry ? ny - 1 - (j0 + jj) : j0 + jj; };
  auto phys_k = [&](int kk) { return rz ? nz - 1 - (k0 + kk) : k0 + kk; };

  // -- stage what does not depend on upstream blocks ----------------------------
  for (int e = t; e < CELLS; e += blockDim.x) {
    const int il = e % TX, r = e / TX, jj = r % PY, kk = r / PY;
    if (il < vx && jj < vy && kk < vz) {
      const size_t c = ((size_t)phys_k(kk) * ny + phys_j(jj)) * nx + phys_i(il);
      qs[e] = gq[c];
      ss[e] = gsig[c];
    }
  }
  for (int e = t; e < TX; e += blockDim.x) lxs[e] = e < vx ? A.wx[phys_i(e)] : (T)1;
  for (int e = t; e < PY; e += blockDim.x) lys[e] = e < vy ? A.wy[phys_j(e)] : (T)1;
  if (DIMS == 3)
    for (int e = t; e < PZ; e += blockDim.x) lzs[e] = e < vz ? A.wz[phys_k(e)] : (T)1;
  for (int e = t; e < KG * TX; e += blockDim.x) {
    const int nn = e / TX, il = e % TX;
    cxs[e] = (nn < gs && il < vx) ? A.cx[(size_t)(ob + nn) * nx + phys_i(il)] : (T)0;
  }
  for (int e = t; e < KG * PY; e += blockDim.x) {
    const int nn = e / PY, jj = e % PY;
    cys[e] = (nn < gs && jj < vy) ? A.cy[(size_t)(ob + nn) * ny + phys_j(jj)] : (T)0;
  }
  if (DIMS == 3)
    for (int e = t; e < KG * PZ; e += blockDim.x) {
      const int nn = e / PZ, kk = e % PZ;
      czs[e] = (nn < gs && kk < vz) ? A.cz[(size_t)(ob + nn) * nz + phys_k(kk)] : (T)0;
    }
  const T amu = A.amu[ord], aeta = A.aeta[ord], axi = A.axi[ord];
  const double wgt = A.wgt[ord];
  const T th = A.theta;
  const size_t slot = (size_t)of * A.ngroups + og;   // (group, octant, ordinate group) slot

  if (dataflow) wait_upstream<T, DIMS>(A, task, slot, epoch);

  // -- incoming faces (written by other CTAs: read through L2) -----------------------
  for (int e = t; e < SM::YF; e += blockDim.x) {
    const int nn = e % KG, r = e / KG, il = r % TX, kk = r / TX;
    T v = (T)0;
    if (task.bj > 0 && nn < gs && il < vx && kk < vz) v = __ldcg(A.yf + F.y(k0 + kk, i0 + il) + nn);
    yin[e] = v;
  }
  if (DIMS == 3)
    for (int e = t; e < SM::ZF; e += blockDim.x) {
      const int nn = e % KG, r = e / KG, il = r % TX, jj = r / TX;
      T v = (T)0;
      if (task.bk > 0 && nn < gs && il < vx && jj < vy) v = __ldcg(A.zf + F.z(j0 + jj, i0 + il) + nn);
      zin[e] = v;
    }
  T xin = (T)0;
  const size_t xslot = F.x(k0 + kl, j0 + jl) + nl;
  if (active && task.bi > 0) xin = __ldcg(A.xf + xslot);
  __syncthreads();

  // -- wavefront: step s solves the cells with il + jl + kl == s, warp-synchronously --
  const int ebase = (kl * PY + jl) * TX;          // cell index of il = 0
  const int ybase = kl * TX * KG + nl;        // y-face slot of il = 0
  const int zbase = jl * TX * KG + nl;        // z-face slot of il = 0
  const int cxbase = nl * TX;
  const T cy_t = cys[nl * PY + jl];
  const T cz_t = DIMS == 3 ? czs[nl * PZ + kl] : (T)0;
  const T ly_t = lys[jl];
  const T lz_t = DIMS == 3 ? lzs[kl] : (T)1;
  T ysh = (T)0, zsh = (T)0;   // faces handed over by the upwind lanes
  T yo = (T)0, zo = (T)0;
  constexpr int STEPS = TX + PY + PZ - 2;
#pragma unroll 2
  for (int s = 0; s < STEPS; ++s) {
    const int il = s - jl - kl;
    const bool valid = active && (unsigned)il < (unsigned)vx;
    if (valid) {
      T y = jl == 0 ? yin[ybase + il * KG] : ysh;
      T z = (T)0;
      if (DIMS == 3) z = kl == 0 ? zin[zbase + il * KG] : zsh;
      const int e = ebase + il;
      const T q = qs[e], st = ss[e];
      T psi;
      if constexpr (DIMS == 3) {
        if constexpr (SCHEME == DOMA_SCHEME_DD) {
          const double geo = dA(dA(cxs[cxbase + il], cy_t), cz_t);
          psi = dd3_exact(q, st, amu, aeta, axi, lxs[il], ly_t, lz_t, geo, xin, y, z);
        } else {
          psi = twdd3_exact(q, st, amu, aeta, axi, lxs[il], ly_t, lz_t, th, xin, y, z);
        }
      } else {
        if constexpr (SCHEME == DOMA_SCHEME_DD) {
          const double geo = dA(cxs[cxbase + il], cy_t);
          psi = dd2_exact(q, st, amu, aeta, lxs[il], ly_t, geo, xin, y);
        } else {
          psi = twdd2_exact(q, st, amu, aeta, axi, lxs[il], ly_t, th, xin, y);
        }
      }
      const size_t cg = ((size_t)phys_k(kl) * ny + phys_j(jl)) * nx + phys_i(il);
      A.wpsi[((size_t)task.grp * N + cg) * A.d_total + ord] = dM(wgt, psi);
      yo = y;
      zo = z;
      if (jl == vy - 1) yout[ybase + il * KG] = y;
      if (DIMS == 3 && kl == vz - 1) zout[zbase + il * KG] = z;
    }
    ysh = __shfl_up_sync(FULL, yo, 1);
    if (DIMS == 3) zsh = __shfl_up_sync(FULL, zo, PY);
  }
  __syncthreads();

  // -- outgoing faces -----------------------------------------------------------------
  if (active) A.xf[xslot] = xin;
  for (int e = t; e < SM::YF; e += blockDim.x) {
    const int nn = e % KG, r = e / KG, il = r % TX, kk = r / TX;
    if (nn < gs && il < vx && kk < vz) A.yf[F.y(k0 + kk, i0 + il) + nn] = yout[e];
  }
  if (DIMS == 3)
    for (int e = t; e < SM::ZF; e += blockDim.x) {
      const int nn = e % KG, r = e / KG, il = r % TX, jj = r / TX;
      if (nn < gs && il < vx && jj < vy) A.zf[F.z(j0 + jj, i0 + il) + nn] = zout[e];
    }

  // -- publish completion (dataflow mode): the barrier orders every thread's
  // face stores before thread 0's release, and a release store is cumulative
  // (PTX memory model), so the consumer's acquire sees them ---------------------------
  if (dataflow) {
    __syncthreads();
    if (t == 0) st_release(done_flag(A, slot, task.bk, task.bj, task.bi), epoch);
  }
}

// ---- single precision -----------------------------------------------------------

template <int DIMS, int TX, int KG>
struct TaskSmemF32 {
  static constexpr int PY = Pencils<DIMS>::PY, PZ = Pencils<DIMS>::PZ;
  static constexpr int CELLS = TX * PY * PZ;
  // Lane (jl, kl) is at il = s - (jl + kl) on step s.  Every per-step array is
  // padded by the largest skew on both sides, so a lane reads at its own base
  // plus s times the stride (a constant offset in the unrolled walk) with no
  // clamp; reads outside its pencil land in finite data it discards.
  static constexpr int SKEW = PY + PZ - 2;
  static constexpr int FPAD = SKEW * KG;                   // face pad (floats), each side
  static constexpr int YF = PZ * TX * KG;                  // y faces [PZ][TX][KG]
  static constexpr int ZF = DIMS == 3 ? PY * TX * KG : 0;  // z faces [PY][TX][KG]
  static constexpr int YREG = YF + 2 * FPAD;
  static constexpr int ZREG = DIMS == 3 ? ZF + 2 * FPAD : 0;
  static constexpr int CREG = 2 * (CELLS + 2 * SKEW);          // {q, sigma_t} per cell
  static constexpr int HREG = KG * TX + 2 * SKEW;          // x coefficients [KG][TX]
  static constexpr int RREG = TX + 2 * SKEW;                   // 1/dx [TX] (2D TW-DD)
  // The walk stores psi per ordinate and cell ([KG][CELLS]; weighted and
  // summed after the walk) -- or, for long blocks whose array would cost a CTA
  // per SM, w psi summed over ordinate pairs across half-warps ([KG / 2][CELLS]).
  static constexpr bool PAIRS = CELLS >= 512;
  static constexpr int PROWS = PAIRS ? KG / 2 : KG;
  // floats: the padded regions, the ordinate weights [KG], then those sums
  static constexpr size_t floats = YREG + ZREG + CREG + HREG + RREG + KG + PROWS * CELLS;
  static constexpr size_t bytes = floats * sizeof(float);
  static_assert(FPAD % 4 == 0 && YREG % 4 == 0, "face regions stay float4-aligned");
  static_assert(CREG % 2 == 0 && (YREG + ZREG) % 2 == 0, "cell region stays float2-aligned");
};

// Coalesced, all-loads-first copy of `count` float4s: in each round every
// load of a thread is issued before its first shared-memory store, so the
// round trips overlap.  A full-size CTA (kMaxSweepThreads) needs one round.
template <int COUNT, typename L>
__device__ __forceinline__ void stage_f4(float4 * dst, L load)
{
  constexpr int IT = (COUNT + kMaxSweepThreads - 1) / kMaxSweepThreads;
  for (int base = 0; base < COUNT; base += IT * (int)blockDim.x) {
    float4 v[IT];
#pragma unroll
    for (int u = 0; u < IT; ++u) {
      const int e = base + (int)threadIdx.x + u * (int)blockDim.x;
      v[u] = e < COUNT ? load(e) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
#pragma unroll
    for (int u = 0; u < IT; ++u) {
      const int e = base + (int)threadIdx.x + u * (int)blockDim.x;
      if (e < COUNT) dst[e] = v[u];
    }
  }
}

template <int DIMS, int SCHEME, int TX, bool SKIP_IDLE = false>
__device__ __forceinline__ void run_task_f32(const SweepArgs<float> & A, const Task task,
                                             unsigned char * smem_raw, bool dataflow, unsigned epoch)
{
  constexpr int KG = ordinate_group(DOMA_PREC_FP32, SCHEME);
  using SM = TaskSmemF32<DIMS, TX, KG>;
  constexpr int PY = SM::PY, PZ = SM::PZ, CELLS = SM::CELLS;
  constexpr unsigned FULL = 0xffffffffu;
  constexpr bool TW = SCHEME == DOMA_SCHEME_TW_DD;
  // TW-DD works with |mu|/dx, DD with 2|mu|/dx (the tables hold the latter)
  constexpr float HS = TW ? 0.5f : 1.0f;
  const int og = task.og;
  const int o = task.oct;
  const int of = task.grp * 8 + o;
  const bool rx = (o & 4) != 0, ry = (o & 2) != 0, rz = (o & 1) != 0;
  const int nx = A.nx, ny = A.ny, nz = DIMS == 3 ? A.nz : 1;
  const size_t N = (size_t)nx * ny * nz;
  const float * gq = A.q + (size_t)task.grp * N;
  const float * gsig = A.sigt + (size_t)task.grp * N;
  const int n0 = og * KG;
  const int gs = min(KG, A.d_oct - n0);
  const int i0 = task.bi * TX, j0 = task.bj * PY, k0 = task.bk * PZ;
  const int vx = min(TX, nx - i0), vy = min(PY, ny - j0), vz = min(PZ, nz - k0);
  const FacePlanes<float, KG> F(A, of, og);
  const size_t slot = F.plane;

  const int t = threadIdx.x;
  const int lane = t & 31;
  const int p = lane & 15;
  const int nl = (t >> 5) * 2 + (lane >> 4);
  const int jl = DIMS == 3 ? (p & 3) : p;
  const int kl = DIMS == 3 ? (p >> 2) : 0;
  const bool active = nl < gs && jl < vy && kl < vz;
  const int ob = A.oct_offset[o] + n0;
  const int ord = ob + min(nl, gs - 1);

  constexpr int SKEW = SM::SKEW, FPAD = SM::FPAD;
  float * const sbase = reinterpret_cast<float *>(smem_raw);
  float * yin = sbase + FPAD;                                            // [PZ][TX][KG]
  float * zin = sbase + SM::YREG + (DIMS == 3 ? FPAD : 0);               // [PY][TX][KG]
  float2 * cell = reinterpret_cast<float2 *>(sbase + SM::YREG + SM::ZREG) + SKEW;  // {q, sigma_t}
  float * hxs = sbase + SM::YREG + SM::ZREG + SM::CREG + SKEW;           // [KG][TX]
  float * rlx = hxs - SKEW + SM::HREG + SKEW;                            // [TX] 1/dx
  float * wts = rlx - SKEW + SM::RREG;                                   // [KG] weights
  float * P = wts + KG;                                              // [PROWS][CELLS]
  constexpr bool PAIRS = SM::PAIRS;

  // the pads: finite values for the reads of steps outside a lane's pencil
  for (int e = t; e < FPAD; e += blockDim.x) {
    yin[e - FPAD] = 0.f;
    yin[SM::YF + e] = 0.f;
    if constexpr (DIMS == 3) {
      zin[e - FPAD] = 0.f;
      zin[SM::ZF + e] = 0.f;
    }
  }
  for (int e = t; e < SKEW; e += blockDim.x) {
    cell[e - SKEW] = make_float2(0.f, 1.f);
    cell[CELLS + e] = make_float2(0.f, 1.f);
    hxs[e - SKEW] = 0.f;
    hxs[KG * TX + e] = 0.f;
    rlx[e - SKEW] = 0.f;
    rlx[TX + e] = 0.f;
  }

  auto phys_i = [&](int il) { return rx ? nx - 1 - (i0 + il) : i0 + il; };
  auto phys_j = [&](int jj) { return ry ? ny - 1 - (j0 + jj) : j0 + jj; };
  auto phys_k = [&](int kk) { return rz ? nz - 1 - (k0 + kk) : k0 + kk; };

  // -- stage what does not depend on upstream blocks ----------------------------
  {
    constexpr int IT = (CELLS + kMaxSweepThreads - 1) / kMaxSweepThreads;
    for (int base = 0; base < CELLS; base += IT * (int)blockDim.x) {
      float2 v[IT];
#pragma unroll
      for (int u = 0; u < IT; ++u) {
        const int e = base + t + u * (int)blockDim.x;
        const int il = e % TX, r = e / TX, jj = r % PY, kk = r / PY;
        v[u] = make_float2(0.f, 1.f);
        if (e < CELLS && il < vx && jj < vy && kk < vz) {
          const size_t c = ((size_t)phys_k(kk) * ny + phys_j(jj)) * nx + phys_i(il);
          v[u] = make_float2(gq[c], gsig[c]);
        }
      }
#pragma unroll
      for (int u = 0; u < IT; ++u) {
        const int e = base + t + u * (int)blockDim.x;
        if (e < CELLS) cell[e] = v[u];
      }
    }
  }
  for (int e = t; e < KG * TX; e += blockDim.x) {
    const int nn = e / TX, il = e % TX;
    hxs[e] = (nn < gs && il < vx) ? fM(HS, A.cx[(size_t)(ob + nn) * nx + phys_i(il)]) : 0.f;
  }
  for (int e = t; e < KG; e += blockDim.x) wts[e] = e < gs ? (float)A.wgt[ob + e] : 0.f;
  if (DIMS == 2 && TW)
    for (int e = t; e < TX; e += blockDim.x) rlx[e] = e < vx ? __frcp_rn(A.wx[phys_i(e)]) : 0.f;
  // per-thread constants of the pencil (clamped indices for inactive lanes)
  const float cy_t = fM(HS, A.cy[(size_t)ord * ny + phys_j(min(jl, vy - 1))]);
  const float cz_t = DIMS == 3 ? fM(HS, A.cz[(size_t)ord * nz + phys_k(min(kl, vz - 1))]) : 0.f;
  const float cyz = fA(cy_t, cz_t);
  const float th = (float)A.theta, om = fS(1.0f, th);
  // 2D TW-DD: theta |xi| / (dx dy) = txy / dx
  const float txy = DIMS == 2 && TW ? fM(fM(th, A.axi_f[ord]), __frcp_rn(A.wy[phys_j(min(jl, vy - 1))])) : 0.f;

  if (dataflow) wait_upstream<float, DIMS>(A, task, slot, epoch);

  // -- incoming faces: every load issued before the first store ----------------------
  {
    constexpr int Y4 = SM::YF / 4, R4 = TX * KG / 4;   // float4s per block / per row
    float xin_v = 0.f;
    const size_t xslot = F.x(k0 + kl, j0 + jl) + nl;
    if (active && task.bi > 0) xin_v = __ldcg(A.xf + xslot);
    stage_f4<Y4>(reinterpret_cast<float4 *>(yin), [&](int e) {
      const int kk = e / R4, r = e % R4;
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      if (task.bj > 0 && kk < vz && r / (KG / 4) < vx)
        v = __ldcg(reinterpret_cast<const float4 *>(A.yf + F.y(k0 + kk, i0)) + r);
      return v;
    });
    if constexpr (DIMS == 3)
      stage_f4<SM::ZF / 4>(reinterpret_cast<float4 *>(zin), [&](int e) {
        const int jj = e / R4, r = e % R4;
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (task.bk > 0 && jj < vy && r / (KG / 4) < vx)
          v = __ldcg(reinterpret_cast<const float4 *>(A.zf + F.z(j0 + jj, i0)) + r);
        return v;
      });
    __syncthreads();

    // -- wavefront: step s solves the cells with il + jl + kl == s ---------------------
    // Every lane runs every step (no divergence); steps outside the lane's
    // pencil compute on clamped indices and keep nothing.  A lane's upwind
    // neighbours are invalid exactly when it is, so no lane consumes a value
    // from an invalid step.
    const int d = jl + kl;
    const int ebase = (kl * PY + jl) * TX;
    // per-lane bases shifted by -d: step s reads element s of the lane's row
    const float * yin_l = yin + (kl * TX - d) * KG + nl;
    const float * zin_l = zin + (jl * TX - d) * KG + nl;
    const float2 * cell_l = cell + (ebase - d);
    const float * hx_l = hxs + (nl * TX - d);
    const float * rlx_l = rlx - d;
    const bool ybound = active && jl == vy - 1;
    const bool zbound = DIMS == 3 && active && kl == vz - 1;
    // store bases shifted by -d as well: step s stores at a constant offset
    float * yout_l = A.yf + F.y(k0 + kl, i0) + nl - (ptrdiff_t)d * KG;
    float * zout_l = DIMS == 3 ? A.zf + F.z(j0 + jl, i0) + nl - (ptrdiff_t)d * KG : nullptr;
    float * P_l = P + (PAIRS ? nl >> 1 : nl) * CELLS + ebase - d;
    const float wgt = PAIRS ? wts[min(nl, KG - 1)] : 0.f;
    float x = xin_v, ysh = 0.f, zsh = 0.f;
    constexpr int STEPS = TX + PY + PZ - 2;
    // SKIP_IDLE (the batched kernel): a warp whose two ordinates both lie
    // past the group's last one has nothing to solve and skips the walk
    // (warp-uniform).  The batched launch sizes every CTA for a full group, so
    // a problem with 4 or 9 ordinates per octant would otherwise spend 6 or 3
    // idle warps' issue slots here.  A single problem's CTAs are sized to its
    // group, and its kernel keeps the branch-free walk.
    const bool warp_busy = !SKIP_IDLE || 2 * (t >> 5) < gs;
    // 3D: fully unrolled; 2D (long skew) partly, which keeps it out of local memory
    if (warp_busy)
#pragma unroll (DIMS == 3 ? STEPS : 4)
    for (int s = 0; s < STEPS; ++s) {
      const int il = s - d;
      const bool valid = active && (unsigned)il < (unsigned)vx;
      // unconditional loads (the padded rows are always in range), then a select
      const float yl = yin_l[s * KG];
      float y = jl == 0 ? yl : ysh;
      float z = 0.f;
      if constexpr (DIMS == 3) {
        const float zl = zin_l[s * KG];
        z = kl == 0 ? zl : zsh;
      }
      const float2 qc = cell_l[s];
      const float hx = hx_l[s];
      float xo = x, psi;
      if constexpr (DIMS == 3) {
        if constexpr (TW) psi = twdd3_fast(qc.x, qc.y, hx, cy_t, cz_t, th, om, xo, y, z);
        else psi = dd3_fast(qc.x, qc.y, hx, cy_t, cz_t, cyz, xo, y, z);
      } else {
        if constexpr (TW) psi = twdd2_fast(qc.x, qc.y, hx, cy_t, fM(txy, rlx_l[s]), th, om, xo, y);
        else psi = dd2_fast(qc.x, qc.y, hx, cy_t, xo, y);
      }
      x = valid ? xo : x;
      st_global_if(yout_l + s * KG, y, valid && ybound);
      if constexpr (DIMS == 3) st_global_if(zout_l + s * KG, z, valid && zbound);
      if constexpr (PAIRS) {
        // lanes l and l + 16 hold the same cell for ordinates nl and nl + 1
        const float wp = valid ? fM(wgt, psi) : 0.f;
        const float pair = fA(wp, __shfl_xor_sync(FULL, wp, 16));
        st_shared_if(P_l + s, pair, valid && lane < 16);
      } else {
        st_shared_if(P_l + s, psi, valid);
      }
      ysh = __shfl_up_sync(FULL, y, 1);
      if (DIMS == 3) zsh = __shfl_up_sync(FULL, z, PY);
    }
    if (active) A.xf[xslot] = x;
  }
  __syncthreads();

  // -- publish completion first: nothing downstream reads the scalar flux.  The
  // barrier above orders every thread's face stores before thread 0's release,
  // and a release store is cumulative (PTX memory model) ------------------------------
  if (dataflow && t == 0) st_release(done_flag(A, slot, task.bk, task.bj, task.bi), epoch);

  // -- the slot's scalar-flux partial: Kahan over the ordinates' w psi, fixed order -----
  for (int e = t; e < CELLS; e += blockDim.x) {
    const int il = e % TX, r = e / TX, jj = r % PY, kk = r / PY;
    if (il < vx && jj < vy && kk < vz) {
      // Kahan over ordinate pairs: the stored pair sums, or the same pair sums
      // formed here from per-ordinate psi (so every block length gives the same bits)
      float sum = 0.0f, comp = 0.0f;
      const int npairs = (gs + 1) >> 1;
      for (int nn = 0; nn < npairs; ++nn) {
        float v;
        if constexpr (PAIRS) {
          v = P[nn * CELLS + e];
        } else {
          const int n0 = 2 * nn, n1 = n0 + 1;
          const float a = fM(wts[n0], P[n0 * CELLS + e]);
          const float b = n1 < gs ? fM(wts[n1], P[n1 * CELLS + e]) : 0.f;
          v = fA(a, b);
        }
        const float yv = fS(v, comp);
        const float tv = fA(sum, yv);
        comp = fS(fS(tv, sum), yv);
        sum = tv;
      }
      const size_t cg = ((size_t)phys_k(kk) * ny + phys_j(jj)) * nx + phys_i(il);
      A.octphi[slot * N + cg] = make_float2(sum, -comp);   // sum - comp, unevaluated
    }
  }
}

template <typename T, int DIMS, int SCHEME, int TX, bool SKIP_IDLE = false>
__device__ __forceinline__ void run_task(const SweepArgs<T> & A, const Task task,
                                         unsigned char * smem_raw, bool dataflow, unsigned epoch)
{
  if constexpr (std::is_same<T, double>::value)
    run_task_exact<DIMS, SCHEME, TX>(A, task, smem_raw, dataflow, epoch);
  else
    run_task_f32<DIMS, SCHEME, TX, SKIP_IDLE>(A, task, smem_raw, dataflow, epoch);
}

// Threads of a full sweep CTA (16 pencils x the ordinate-group size) and the
// resident CTAs per SM the kernels are compiled for, which cap the registers
// of the single-precision body (its unrolled wavefront would otherwise take
// every register it can).  Measured on GB300:
//   * FP32 DD (128-thread CTAs) has two bodies.  At 8 CTAs per SM (64
//     registers) the 48^3 and 64^3 sweeps with 16 ordinates per octant (two
//     ordinate groups) take 115 and 196 us, against 143 and 219 us at 12 per
//     SM (40 registers).  The 100^3 duct with 36 ordinates per octant (five
//     groups: more independent tasks per wavefront level) is the other way
//     round, 1542 against 1369 us, and so is the multigroup solve with eight
//     groups in flight (415 against 374 ms).
//   * FP32 TW-DD (128-thread CTAs), with more live values per cell: compiled
//     for 5 per SM (it takes 80 registers, so 6 fit) for one group in flight,
//     244 us at 64^3 against 246 us compiled for 4; for 6 with many tasks per
//     level.
//   * FP64 (one-warp CTAs): 1, which leaves the registers to the compiler (154;
//     12 CTAs fit).  With 256-thread CTAs, 2 and 3 per SM had been 19 % and
//     38 % slower than 1: the FP64 pipe is the limit.
// MANY selects the body for many tasks per wavefront level; solvers take it
// from three (ordinate group, group in flight) slots per octant up
// (sweep_many_ctas).  Both bodies of a scheme run the same instructions on the
// same values: the same bits.
template <typename T, int SCHEME>
constexpr int sweep_cta_threads()
{
  return 16 * ordinate_group(std::is_same<T, double>::value ? DOMA_PREC_FP64 : DOMA_PREC_FP32, SCHEME);
}

template <typename T, int SCHEME, bool MANY = false>
constexpr int sweep_min_ctas()
{
  return std::is_same<T, double>::value ? DOMA_SWEEP_MIN_CTAS_FP64
         : SCHEME == DOMA_SCHEME_DD     ? (MANY ? DOMA_SWEEP_MIN_CTAS_DD_MANY : DOMA_SWEEP_MIN_CTAS_DD)
                                        : (MANY ? DOMA_SWEEP_MIN_CTAS_MANY : DOMA_SWEEP_MIN_CTAS);
}

// The batched kernel holds every block length's body; at 40 registers its DD
// form spills, and 8 CTAs per SM (64 registers) solved the 256-problem mix
// 2.4 % faster than 12.
template <typename T, int SCHEME>
constexpr int sweep_batch_min_ctas()
{
  return SCHEME == DOMA_SCHEME_DD ? DOMA_SWEEP_BATCH_MIN_CTAS_DD : sweep_min_ctas<T, SCHEME, true>();
}

// Only the FP32 modes have a second body.
template <typename T, int SCHEME>
constexpr bool has_many_body()
{
  return !std::is_same<T, double>::value;
}

template <typename T, int DIMS, int SCHEME, int TX>
constexpr size_t task_smem_bytes()
{
  if constexpr (std::is_same<T, double>::value) return TaskSmemExact<DIMS, TX>::bytes;
  else return TaskSmemF32<DIMS, TX, ordinate_group(DOMA_PREC_FP32, SCHEME)>::bytes;
}

// Persistent dataflow sweep: CTAs claim tasks in topological order from a
// ticket counter; a claimed task waits only on tasks with smaller tickets,
// which running CTAs already hold, so progress never depends on residency.
template <typename T, int DIMS, int SCHEME, int TX, bool MANY>
__global__ void __launch_bounds__(sweep_cta_threads<T, SCHEME>(), sweep_min_ctas<T, SCHEME, MANY>())
    sweep_persistent_kernel(const SweepArgs<T> A)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ unsigned s_next;
  const unsigned epoch = *A.epoch + 1u;
  const unsigned claimer = blockDim.x - 1;   // not thread 0, which does the waits
  if (threadIdx.x == claimer) s_next = atomicAdd(A.ticket, 1u);
  __syncthreads();
  for (;;) {
    const unsigned tk = s_next;
    __syncthreads();  // everyone has read the ticket; the previous task's smem is free
    if (tk >= (unsigned)A.num_tasks) break;
    // claim the following ticket now: its round trip overlaps this task (the
    // task's internal barriers order the write before the next read)
    if (threadIdx.x == claimer) s_next = atomicAdd(A.ticket, 1u);
    run_task<T, DIMS, SCHEME, TX>(A, A.tasks[tk], smem_raw, true, epoch);
  }
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(A.exit_count, 1u) == gridDim.x - 1) {
      // last CTA out: re-arm the counters for the next sweep
      *A.ticket = 0u;
      *A.exit_count = 0u;
      __threadfence();
      *A.epoch = epoch;
    }
  }
}

// Batched persistent sweep: one grid works through the level-merged tasks of
// every problem of a batch.  Tasks of problems that have converged publish
// their done flag and return, so a batch keeps one static task list.
template <typename T, int DIMS, int SCHEME>
__global__ void __launch_bounds__(sweep_cta_threads<T, SCHEME>(), sweep_batch_min_ctas<T, SCHEME>())
    sweep_batch_kernel(const SweepArgs<T> * args, const BatchTask * tasks, int num_tasks,
                       unsigned * ticket, unsigned * exit_count, unsigned * epoch_ctr,
                       const BatchLoop * loops)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ unsigned s_next;
  const unsigned epoch = *epoch_ctr + 1u;
  const unsigned claimer = blockDim.x - 1;
  if (threadIdx.x == claimer) s_next = atomicAdd(ticket, 1u);
  __syncthreads();
  for (;;) {
    const unsigned tk = s_next;
    __syncthreads();
    if (tk >= (unsigned)num_tasks) break;
    if (threadIdx.x == claimer) s_next = atomicAdd(ticket, 1u);
    const BatchTask bt = tasks[tk];
    const SweepArgs<T> & A = args[bt.prob];
    if (!loops[bt.prob].active) {  // uniform across the CTA: the flag changes between launches
      if (threadIdx.x == 0) {
        const size_t slot = (size_t)(bt.t.grp * 8 + bt.t.oct) * A.ngroups + bt.t.og;
        st_release(A.done + ((slot * A.nbz + bt.t.bk) * A.nby + bt.t.bj) * A.nbx + bt.t.bi, epoch);
      }
      // the claimer's write of s_next must be ordered before everyone's next
      // read of it (run_task's barriers do this on the other path)
      __syncthreads();
      continue;
    }
    // each problem has its own block length (uniform across the CTA)
    if (A.tx <= 8) run_task<T, DIMS, SCHEME, 8, true>(A, bt.t, smem_raw, true, epoch);
    else if (A.tx <= 16) run_task<T, DIMS, SCHEME, 16, true>(A, bt.t, smem_raw, true, epoch);
    else run_task<T, DIMS, SCHEME, 32, true>(A, bt.t, smem_raw, true, epoch);
  }
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(exit_count, 1u) == gridDim.x - 1) {
      *ticket = 0u;
      *exit_count = 0u;
      __threadfence();
      *epoch_ctr = epoch;
    }
  }
}

// One launch per level (level = bi + bj + bk): ordering by kernel boundaries.
template <typename T, int DIMS, int SCHEME, int TX, bool MANY>
__global__ void __launch_bounds__(sweep_cta_threads<T, SCHEME>(), sweep_min_ctas<T, SCHEME, MANY>())
    sweep_level_kernel(const SweepArgs<T> A)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  run_task<T, DIMS, SCHEME, TX>(A, A.tasks[A.task_offset + blockIdx.x], smem_raw, false, 0u);
}

template <typename T, int DIMS, int SCHEME, int TX, bool MANY>
doma_status launch_impl(const Schedule & s, const SweepArgs<T> & args, cudaStream_t stream,
                        uint64_t * launches)
{
  if (s.persistent) {
    sweep_persistent_kernel<T, DIMS, SCHEME, TX, MANY><<<s.grid, s.threads, s.smem, stream>>>(args);
    if (launches) ++*launches;
  } else {
    SweepArgs<T> a = args;
    const int levels = (int)s.level_begin.size() - 1;
    for (int L = 0; L < levels; ++L) {
      const int count = s.level_begin[L + 1] - s.level_begin[L];
      if (count == 0) continue;
      a.task_offset = s.level_begin[L];
      sweep_level_kernel<T, DIMS, SCHEME, TX, MANY><<<count, s.threads, s.smem, stream>>>(a);
      if (launches) ++*launches;
    }
  }
  DOMA_CUDA_TRY(cudaGetLastError());
  return DOMA_OK;
}

template <typename T>
struct TypeTag {
  using type = T;
};

// Dispatch over the compile-time choices: precision, dimension, scheme, TX.
template <typename F>
auto dispatch(int dims, int precision, int scheme, int tx, F && f)
{
  auto by_tx = [&](auto tag_t, auto dims_c, auto scheme_c) {
    using T = typename decltype(tag_t)::type;
    constexpr int D = decltype(dims_c)::value, S = decltype(scheme_c)::value;
    if (tx <= 8) return f(tag_t, dims_c, scheme_c, std::integral_constant<int, 8>{});
    if (tx <= 16) return f(tag_t, dims_c, scheme_c, std::integral_constant<int, 16>{});
    (void)sizeof(T); (void)D; (void)S;
    return f(tag_t, dims_c, scheme_c, std::integral_constant<int, 32>{});
  };
  auto by_scheme = [&](auto tag_t, auto dims_c) {
    if (scheme == DOMA_SCHEME_TW_DD)
      return by_tx(tag_t, dims_c, std::integral_constant<int, DOMA_SCHEME_TW_DD>{});
    return by_tx(tag_t, dims_c, std::integral_constant<int, DOMA_SCHEME_DD>{});
  };
  auto by_dims = [&](auto tag_t) {
    if (dims == 2) return by_scheme(tag_t, std::integral_constant<int, 2>{});
    return by_scheme(tag_t, std::integral_constant<int, 3>{});
  };
  if (precision == DOMA_PREC_FP64) return by_dims(TypeTag<double>{});
  return by_dims(TypeTag<float>{});
}

// Calls g with std::true_type for an FP32 mode's many-task body when `many`
// asks for it, else with std::false_type (the only body of the FP64 mode).
template <typename T, int S, typename G>
auto with_many(bool many, G && g)
{
  if constexpr (has_many_body<T, S>())
    if (many) return g(std::true_type{});
  return g(std::false_type{});
}

}  // namespace

int sweep_threads(int gs)
{
  return ((16 * gs + 31) / 32) * 32;
}

int sweep_tile_x(int requested)
{
  return requested <= 8 ? 8 : requested <= 16 ? 16 : 32;
}

size_t sweep_smem_bytes(int dims, int precision, int scheme, int tx)
{
  return dispatch(dims, precision, scheme, tx, [](auto tag_t, auto dims_c, auto sch_c, auto tx_c) {
    using T = typename decltype(tag_t)::type;
    return task_smem_bytes<T, decltype(dims_c)::value, decltype(sch_c)::value, decltype(tx_c)::value>();
  });
}

bool sweep_many_ctas(int precision, int ngroups, int groups_in_flight)
{
  return precision == DOMA_PREC_FP32 && ngroups * groups_in_flight >= 3;
}

doma_status sweep_prepare(int dims, int precision, int scheme, int tx, size_t smem, bool many)
{
  cudaError_t e = dispatch(dims, precision, scheme, tx, [&](auto tag_t, auto dims_c, auto sch_c, auto tx_c) {
    using T = typename decltype(tag_t)::type;
    constexpr int D = decltype(dims_c)::value, S = decltype(sch_c)::value, X = decltype(tx_c)::value;
    return with_many<T, S>(many, [&](auto many_c) {
      constexpr bool MN = decltype(many_c)::value;
      cudaError_t r = cudaFuncSetAttribute(sweep_persistent_kernel<T, D, S, X, MN>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (r != cudaSuccess) return r;
      return cudaFuncSetAttribute(sweep_level_kernel<T, D, S, X, MN>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    });
  });
  DOMA_CUDA_TRY(e);
  return DOMA_OK;
}

int sweep_resident_ctas(int dims, int precision, int scheme, int tx, int threads, size_t smem, bool many)
{
  return dispatch(dims, precision, scheme, tx, [&](auto tag_t, auto dims_c, auto sch_c, auto tx_c) {
    using T = typename decltype(tag_t)::type;
    constexpr int D = decltype(dims_c)::value, S = decltype(sch_c)::value, X = decltype(tx_c)::value;
    int per_sm = 0;
    const cudaError_t r = with_many<T, S>(many, [&](auto many_c) {
      return cudaOccupancyMaxActiveBlocksPerMultiprocessor(
          &per_sm, sweep_persistent_kernel<T, D, S, X, decltype(many_c)::value>, threads, smem);
    });
    if (r != cudaSuccess) return 0;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return per_sm * sms;
  });
}

// Dispatch over dimension and scheme only (the batched kernel holds every
// block length).
template <typename F>
auto dispatch_batch(int dims, int scheme, F && f)
{
  auto by_scheme = [&](auto dims_c) {
    if (scheme == DOMA_SCHEME_TW_DD) return f(dims_c, std::integral_constant<int, DOMA_SCHEME_TW_DD>{});
    return f(dims_c, std::integral_constant<int, DOMA_SCHEME_DD>{});
  };
  if (dims == 2) return by_scheme(std::integral_constant<int, 2>{});
  return by_scheme(std::integral_constant<int, 3>{});
}

size_t sweep_batch_smem_bytes(int dims, int scheme)
{
  // the largest block length's layout serves all three
  return dispatch_batch(dims, scheme, [](auto dims_c, auto sch_c) {
    return task_smem_bytes<float, decltype(dims_c)::value, decltype(sch_c)::value, 32>();
  });
}

doma_status launch_sweep_batch(int dims, int scheme, int grid, int threads, size_t smem,
                               const SweepArgs<float> * args, const BatchTask * tasks,
                               int num_tasks, unsigned * ticket, unsigned * exit_count,
                               unsigned * epoch, const BatchLoop * loops, cudaStream_t stream)
{
  cudaError_t e = dispatch_batch(dims, scheme, [&](auto dims_c, auto sch_c) {
    constexpr int D = decltype(dims_c)::value, S = decltype(sch_c)::value;
    cudaError_t r = cudaFuncSetAttribute(sweep_batch_kernel<float, D, S>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (r != cudaSuccess) return r;
    sweep_batch_kernel<float, D, S><<<grid, threads, smem, stream>>>(args, tasks, num_tasks, ticket,
                                                                    exit_count, epoch, loops);
    return cudaGetLastError();
  });
  DOMA_CUDA_TRY(e);
  return DOMA_OK;
}

int sweep_batch_resident_ctas(int dims, int scheme, int threads, size_t smem)
{
  return dispatch_batch(dims, scheme, [&](auto dims_c, auto sch_c) {
    constexpr int D = decltype(dims_c)::value, S = decltype(sch_c)::value;
    if (cudaFuncSetAttribute(sweep_batch_kernel<float, D, S>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
      return 0;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sweep_batch_kernel<float, D, S>,
                                                      threads, smem) != cudaSuccess)
      return 0;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return per_sm * sms;
  });
}

doma_status launch_sweep(int dims, int precision, int scheme, const Schedule & s,
                         const SweepArgs<double> * a64, const SweepArgs<float> * a32,
                         cudaStream_t stream, uint64_t * launches)
{
  return dispatch(dims, precision, scheme, s.tx, [&](auto tag_t, auto dims_c, auto sch_c, auto tx_c) {
    using T = typename decltype(tag_t)::type;
    constexpr int D = decltype(dims_c)::value, S = decltype(sch_c)::value, X = decltype(tx_c)::value;
    return with_many<T, S>(s.many, [&](auto many_c) {
      constexpr bool MN = decltype(many_c)::value;
      if constexpr (std::is_same<T, double>::value)
        return launch_impl<T, D, S, X, MN>(s, *a64, stream, launches);
      else
        return launch_impl<T, D, S, X, MN>(s, *a32, stream, launches);
    });
  });
}

}  // namespace doma
