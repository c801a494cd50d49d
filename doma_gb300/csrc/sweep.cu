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

__device__ __forceinline__ float fA(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fS(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fM(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fF(float a, float b, float c) { return __fmaf_rn(a, b, c); }
// Approximate reciprocal (one MUFU op); the TW-DD weights it inverts lie in [0.5, 1].
__device__ __forceinline__ float fR(float a) { return __fdividef(1.0f, a); }

// DD with cx = 2|mu|/lx etc.: psi = (q + cx x + cy y + cz z) / (cx + cy + cz + st).
__device__ __forceinline__ float dd_f32(float q, float st, float cx, float cy, float cz,
                                        float & x, float & y, float & z)
{
  const float num = fF(cz, z, fF(cy, y, fF(cx, x, q)));
  const float c = __fdividef(num, fA(fA(fA(cx, cy), cz), st));
  x = fF(2.0f, c, -x);
  y = fF(2.0f, c, -y);
  z = fF(2.0f, c, -z);
  return c;
}

// TW-DD weight: 1 - num / (den * flux), clamped to [0.5, 1]; 0.5 when the
// upwind flux is <= 1e-8 (include/TWDiamondDifference3D.h:43-75).
__device__ __forceinline__ float tw_weight(float num, float den_in, float flux)
{
  float a = 0.5f;
  if (flux > 1e-8f) a = fS(1.0f, __fdividef(num, fM(den_in, flux)));
  return fminf(fmaxf(a, 0.5f), 1.0f);
}

__device__ __forceinline__ float twdd3_f32(float q, float st, float amu, float aeta, float axi,
                                           float lx, float ly, float lz, float th, float & x,
                                           float & y, float & z)
{
  const float A = fM(ly, lz), B = fM(lx, lz), C = fM(lx, ly), V = fM(fM(lx, ly), lz);
  const float muA = fM(amu, A), etB = fM(aeta, B), xiC = fM(axi, C);
  const float qV = fM(q, V), qVt = fM(qV, th), sV = fM(st, V);
  const float mx = fM(muA, x), ey = fM(etB, y), xz = fM(xiC, z);
  const float a = tw_weight(fF(fA(ey, xz), th, fA(qVt, mx)), fF(2.0f, fA(etB, xiC), sV), x);
  const float b = tw_weight(fF(fA(mx, xz), th, fA(qVt, ey)), fF(2.0f, fA(muA, xiC), sV), y);
  const float c3 = tw_weight(fF(fA(mx, ey), th, fA(qVt, xz)), fF(2.0f, fA(muA, etB), sV), z);
  const float ra = fR(a), rb = fR(b), rc = fR(c3);
  const float ta = fM(muA, ra), tb = fM(etB, rb), tc = fM(xiC, rc);
  const float c = __fdividef(fF(tc, z, fF(tb, y, fF(ta, x, qV))), fA(fA(fA(sV, ta), tb), tc));
  x = fM(fF(fS(a, 1.0f), x, c), ra);   // (c - (1 - a) x) / a
  y = fM(fF(fS(b, 1.0f), y, c), rb);
  z = fM(fF(fS(c3, 1.0f), z, c), rc);
  return c;
}

__device__ __forceinline__ float dd2_f32(float q, float st, float cx, float cy, float & x,
                                         float & y)
{
  const float c = __fdividef(fF(cy, y, fF(cx, x, q)), fA(fA(cx, cy), st));
  x = fF(2.0f, c, -x);
  y = fF(2.0f, c, -y);
  return c;
}

__device__ __forceinline__ float twdd2_f32(float q, float st, float amu, float aeta, float axi,
                                           float lx, float ly, float th, float & x, float & y)
{
  const float A = ly, B = lx, V = fM(lx, ly);
  const float muA = fM(amu, A), etB = fM(aeta, B);
  const float qV = fM(q, V), qVt = fM(qV, th), sV = fM(st, V);
  const float mx = fM(muA, x), ey = fM(etB, y);
  const float a = tw_weight(fF(ey, th, fA(qVt, mx)), fF(2.0f, etB, sV), x);
  const float b = tw_weight(fF(fA(mx, axi), th, fA(qVt, ey)), fF(2.0f, muA, sV), y);
  const float ra = fR(a), rb = fR(b);
  const float ta = fM(muA, ra), tb = fM(etB, rb);
  const float c = __fdividef(fF(tb, y, fF(ta, x, qV)), fA(fA(sV, ta), tb));
  x = fM(fF(fS(a, 1.0f), x, c), ra);
  y = fM(fF(fS(b, 1.0f), y, c), rb);
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

// Wait until *flag == epoch.  Bounded: the first polls are back to back,
// then exponential back-off up to ~0.5 us; after `limit` polls it records
// DOMA_DEVICE_WAIT_TIMEOUT in *error and returns false.  It also gives up at
// once when another CTA has already failed.
__device__ bool wait_for(const unsigned * flag, unsigned epoch, unsigned limit, int * error)
{
  unsigned ns = 32;
  for (unsigned it = 0; it < limit; ++it) {
    if (ld_acquire(flag) == epoch) return true;
    if (ld_relaxed(error) != 0) return false;
    if (it >= 8) {
      __nanosleep(ns);
      if (ns < 512) ns *= 2;
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
// Shared memory carries only the block-boundary faces (staged in and out
// coalesced) and, in fp32 mode, the w*psi values for the angular reduction.

template <int DIMS> struct Pencils;
template <> struct Pencils<3> { static constexpr int PY = 4, PZ = 4; };
template <> struct Pencils<2> { static constexpr int PY = 16, PZ = 1; };

template <typename T, int DIMS, int TX>
struct TaskSmem {
  static constexpr int PY = Pencils<DIMS>::PY, PZ = Pencils<DIMS>::PZ;
  static constexpr int CELLS = TX * PY * PZ;
  static constexpr int YF = PZ * TX * kGroup;                  // y faces [PZ][TX][kGroup]
  static constexpr int ZF = DIMS == 3 ? PY * TX * kGroup : 0;  // z faces [PY][TX][kGroup]
  static constexpr int NT = 2 * YF + 2 * ZF + 2 * CELLS + TX + PY + PZ + kGroup * (TX + PY + PZ);
  static constexpr bool EXACT = std::is_same<T, double>::value;
  static constexpr size_t bytes = NT * sizeof(T) + (EXACT ? 0 : (size_t)(kGroup / 2) * CELLS * sizeof(float));
};

template <typename T, int DIMS, int SCHEME, int TX>
__device__ __forceinline__ void run_task(const SweepArgs<T> & A, const Task task,
                                         unsigned char * smem_raw, bool dataflow, unsigned epoch)
{
  using SM = TaskSmem<T, DIMS, TX>;
  constexpr bool EXACT = SM::EXACT;
  constexpr int PY = SM::PY, PZ = SM::PZ, CELLS = SM::CELLS;
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
  const int n0 = og * kGroup;
  const int gs = min(kGroup, Do - n0);
  const int i0 = task.bi * TX, j0 = task.bj * PY, k0 = task.bk * PZ;
  const int vx = min(TX, nx - i0), vy = min(PY, ny - j0), vz = min(PZ, nz - k0);

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
  T * cxs = lzs + PZ;                 // [kGroup][TX]
  T * cys = cxs + kGroup * TX;        // [kGroup][PY]
  T * czs = cys + kGroup * PY;        // [kGroup][PZ]
  float * P = reinterpret_cast<float *>(czs + kGroup * PZ);  // fp32: [kGroup / 2][CELLS] pair sums

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
  for (int e = t; e < kGroup * TX; e += blockDim.x) {
    const int nn = e / TX, il = e % TX;
    cxs[e] = (nn < gs && il < vx) ? A.cx[(size_t)(ob + nn) * nx + phys_i(il)] : (T)0;
  }
  for (int e = t; e < kGroup * PY; e += blockDim.x) {
    const int nn = e / PY, jj = e % PY;
    cys[e] = (nn < gs && jj < vy) ? A.cy[(size_t)(ob + nn) * ny + phys_j(jj)] : (T)0;
  }
  if (DIMS == 3)
    for (int e = t; e < kGroup * PZ; e += blockDim.x) {
      const int nn = e / PZ, kk = e % PZ;
      czs[e] = (nn < gs && kk < vz) ? A.cz[(size_t)(ob + nn) * nz + phys_k(kk)] : (T)0;
    }
  T amu, aeta, axi;
  if (EXACT) {
    amu = (T)A.amu[ord]; aeta = (T)A.aeta[ord]; axi = (T)A.axi[ord];
  } else {
    amu = (T)A.amu_f[ord]; aeta = (T)A.aeta_f[ord]; axi = (T)A.axi_f[ord];
  }
  const double wgt = A.wgt[ord];
  const float wgt_f = (float)wgt;
  const T th = (T)A.theta;
  const size_t slot = (size_t)of * A.ngroups + og;   // (group, octant, ordinate group) slot

  // -- wait for the upstream blocks (dataflow mode) --------------------------------
  if (dataflow) {
    if (t == 0) {
      const int nbx = A.nbx, nby = A.nby, nbz = A.nbz;
      const size_t base = slot * nbz;
      const unsigned want = epoch + A.wait_bias;
      if (task.bi > 0)
        wait_for(A.done + ((base + task.bk) * nby + task.bj) * nbx + task.bi - 1, want,
                 A.spin_limit, A.error);
      if (task.bj > 0)
        wait_for(A.done + ((base + task.bk) * nby + task.bj - 1) * nbx + task.bi, want,
                 A.spin_limit, A.error);
      if (DIMS == 3 && task.bk > 0)
        wait_for(A.done + ((base + task.bk - 1) * nby + task.bj) * nbx + task.bi, want,
                 A.spin_limit, A.error);
    }
    __syncthreads();
  }

  // -- incoming faces (written by other CTAs: read through L2) -----------------------
  for (int e = t; e < SM::YF; e += blockDim.x) {
    const int nn = e % kGroup, r = e / kGroup, il = r % TX, kk = r / TX;
    T v = (T)0;
    if (task.bj > 0 && nn < gs && il < vx && kk < vz)
      v = __ldcg(A.yf + (((size_t)of * nz + (k0 + kk)) * nx + (i0 + il)) * Do + n0 + nn);
    yin[e] = v;
  }
  if (DIMS == 3)
    for (int e = t; e < SM::ZF; e += blockDim.x) {
      const int nn = e % kGroup, r = e / kGroup, il = r % TX, jj = r / TX;
      T v = (T)0;
      if (task.bk > 0 && nn < gs && il < vx && jj < vy)
        v = __ldcg(A.zf + (((size_t)of * ny + (j0 + jj)) * nx + (i0 + il)) * Do + n0 + nn);
      zin[e] = v;
    }
  T xin = (T)0;
  const size_t xslot = (((size_t)of * nz + (k0 + kl)) * ny + (j0 + jl)) * Do + n0 + nl;
  if (active && task.bi > 0) xin = __ldcg(A.xf + xslot);
  __syncthreads();

  // -- wavefront: step s solves the cells with il + jl + kl == s, warp-synchronously --
  // per-thread constants of the pencil (valid for every active thread)
  const int ebase = (kl * PY + jl) * TX;          // cell index of il = 0
  const int ybase = kl * TX * kGroup + nl;        // y-face slot of il = 0
  const int zbase = jl * TX * kGroup + nl;        // z-face slot of il = 0
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
    float wp = 0.0f;
    int e = 0;
    if (valid) {
      T y = jl == 0 ? yin[ybase + il * kGroup] : ysh;
      T z = (T)0;
      if (DIMS == 3) z = kl == 0 ? zin[zbase + il * kGroup] : zsh;
      e = ebase + il;
      const T q = qs[e], st = ss[e];
      T psi;
      if constexpr (EXACT) {
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
      } else {
        if constexpr (DIMS == 3) {
          if constexpr (SCHEME == DOMA_SCHEME_DD)
            psi = dd_f32(q, st, cxs[cxbase + il], cy_t, cz_t, xin, y, z);
          else
            psi = twdd3_f32(q, st, amu, aeta, axi, lxs[il], ly_t, lz_t, th, xin, y, z);
        } else {
          if constexpr (SCHEME == DOMA_SCHEME_DD)
            psi = dd2_f32(q, st, cxs[cxbase + il], cy_t, xin, y);
          else
            psi = twdd2_f32(q, st, amu, aeta, axi, lxs[il], ly_t, th, xin, y);
        }
        wp = fM(wgt_f, psi);
      }
      yo = y;
      zo = z;
      if (jl == vy - 1) yout[ybase + il * kGroup] = y;
      if (DIMS == 3 && kl == vz - 1) zout[zbase + il * kGroup] = z;
    }
    if constexpr (!EXACT) {
      // lanes l and l + 16 hold the same cell for ordinates nl and nl + 1:
      // sum the pair in-warp, store one value per pair
      const float pair = fA(wp, __shfl_xor_sync(FULL, wp, 16));
      if (valid && lane < 16) P[(nl >> 1) * CELLS + e] = pair;
    }
    ysh = __shfl_up_sync(FULL, yo, 1);
    if (DIMS == 3) zsh = __shfl_up_sync(FULL, zo, PY);
  }
  __syncthreads();

  // -- outgoing faces and (fp32) the group's scalar-flux partial ------------------------
  if (active) A.xf[xslot] = xin;
  for (int e = t; e < SM::YF; e += blockDim.x) {
    const int nn = e % kGroup, r = e / kGroup, il = r % TX, kk = r / TX;
    if (nn < gs && il < vx && kk < vz)
      A.yf[(((size_t)of * nz + (k0 + kk)) * nx + (i0 + il)) * Do + n0 + nn] = yout[e];
  }
  if (DIMS == 3)
    for (int e = t; e < SM::ZF; e += blockDim.x) {
      const int nn = e % kGroup, r = e / kGroup, il = r % TX, jj = r / TX;
      if (nn < gs && il < vx && jj < vy)
        A.zf[(((size_t)of * ny + (j0 + jj)) * nx + (i0 + il)) * Do + n0 + nn] = zout[e];
    }
  if constexpr (!EXACT) {
    for (int e = t; e < CELLS; e += blockDim.x) {
      const int il = e % TX, r = e / TX, jj = r % PY, kk = r / PY;
      if (il < vx && jj < vy && kk < vz) {
        float sum = 0.0f, comp = 0.0f;
        const int npairs = (gs + 1) >> 1;
        for (int nn = 0; nn < npairs; ++nn) {  // Kahan over ordinate pairs, fixed order
          const float yv = fS(P[nn * CELLS + e], comp);
          const float tv = fA(sum, yv);
          comp = fS(fS(tv, sum), yv);
          sum = tv;
        }
        const size_t cg = ((size_t)phys_k(kk) * ny + phys_j(jj)) * nx + phys_i(il);
        A.octphi[slot * N + cg] = (double)sum - (double)comp;
      }
    }
  }

  // -- publish completion (dataflow mode) ---------------------------------------------
  if (dataflow) {
    __threadfence();
    __syncthreads();
    if (t == 0)
      st_release(A.done + ((slot * A.nbz + task.bk) * A.nby + task.bj) * A.nbx + task.bi, epoch);
  }
}

// Persistent dataflow sweep: CTAs claim tasks in topological order from a
// ticket counter; a claimed task waits only on tasks with smaller tickets,
// which running CTAs already hold, so progress never depends on residency.
template <typename T, int DIMS, int SCHEME, int TX>
__global__ void __launch_bounds__(kMaxSweepThreads) sweep_persistent_kernel(const SweepArgs<T> A)
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
template <typename T, int DIMS, int SCHEME, int TX>
__global__ void __launch_bounds__(kMaxSweepThreads)
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
    run_task<T, DIMS, SCHEME, TX>(A, bt.t, smem_raw, true, epoch);
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
template <typename T, int DIMS, int SCHEME, int TX>
__global__ void __launch_bounds__(kMaxSweepThreads) sweep_level_kernel(const SweepArgs<T> A)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  run_task<T, DIMS, SCHEME, TX>(A, A.tasks[A.task_offset + blockIdx.x], smem_raw, false, 0u);
}

template <typename T, int DIMS, int SCHEME, int TX>
doma_status launch_impl(const Schedule & s, const SweepArgs<T> & args, cudaStream_t stream,
                        uint64_t * launches)
{
  if (s.persistent) {
    sweep_persistent_kernel<T, DIMS, SCHEME, TX><<<s.grid, s.threads, s.smem, stream>>>(args);
    if (launches) ++*launches;
  } else {
    SweepArgs<T> a = args;
    const int levels = (int)s.level_begin.size() - 1;
    for (int L = 0; L < levels; ++L) {
      const int count = s.level_begin[L + 1] - s.level_begin[L];
      if (count == 0) continue;
      a.task_offset = s.level_begin[L];
      sweep_level_kernel<T, DIMS, SCHEME, TX><<<count, s.threads, s.smem, stream>>>(a);
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

}  // namespace

int sweep_tile_x(int requested)
{
  return requested <= 8 ? 8 : requested <= 16 ? 16 : 32;
}

size_t sweep_smem_bytes(int dims, int precision, int scheme, int tx)
{
  return dispatch(dims, precision, scheme, tx, [](auto tag_t, auto dims_c, auto, auto tx_c) {
    using T = typename decltype(tag_t)::type;
    return TaskSmem<T, decltype(dims_c)::value, decltype(tx_c)::value>::bytes;
  });
}

doma_status sweep_prepare(int dims, int precision, int scheme, int tx, size_t smem)
{
  cudaError_t e = dispatch(dims, precision, scheme, tx, [&](auto tag_t, auto dims_c, auto sch_c, auto tx_c) {
    using T = typename decltype(tag_t)::type;
    constexpr int D = decltype(dims_c)::value, S = decltype(sch_c)::value, X = decltype(tx_c)::value;
    cudaError_t r = cudaFuncSetAttribute(sweep_persistent_kernel<T, D, S, X>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (r != cudaSuccess) return r;
    return cudaFuncSetAttribute(sweep_level_kernel<T, D, S, X>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  });
  DOMA_CUDA_TRY(e);
  return DOMA_OK;
}

int sweep_resident_ctas(int dims, int precision, int scheme, int tx, int threads, size_t smem)
{
  return dispatch(dims, precision, scheme, tx, [&](auto tag_t, auto dims_c, auto sch_c, auto tx_c) {
    using T = typename decltype(tag_t)::type;
    constexpr int D = decltype(dims_c)::value, S = decltype(sch_c)::value, X = decltype(tx_c)::value;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sweep_persistent_kernel<T, D, S, X>,
                                                      threads, smem) != cudaSuccess)
      return 0;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return per_sm * sms;
  });
}

doma_status launch_sweep_batch(int dims, int scheme, int tx, int grid, int threads, size_t smem,
                               const SweepArgs<float> * args, const BatchTask * tasks,
                               int num_tasks, unsigned * ticket, unsigned * exit_count,
                               unsigned * epoch, const BatchLoop * loops, cudaStream_t stream)
{
  cudaError_t e = dispatch(dims, DOMA_PREC_FP32, scheme, tx, [&](auto, auto dims_c, auto sch_c, auto tx_c) {
    constexpr int D = decltype(dims_c)::value, S = decltype(sch_c)::value, X = decltype(tx_c)::value;
    cudaError_t r = cudaFuncSetAttribute(sweep_batch_kernel<float, D, S, X>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (r != cudaSuccess) return r;
    sweep_batch_kernel<float, D, S, X><<<grid, threads, smem, stream>>>(args, tasks, num_tasks, ticket,
                                                                       exit_count, epoch, loops);
    return cudaGetLastError();
  });
  DOMA_CUDA_TRY(e);
  return DOMA_OK;
}

int sweep_batch_resident_ctas(int dims, int scheme, int tx, int threads, size_t smem)
{
  return dispatch(dims, DOMA_PREC_FP32, scheme, tx, [&](auto, auto dims_c, auto sch_c, auto tx_c) {
    constexpr int D = decltype(dims_c)::value, S = decltype(sch_c)::value, X = decltype(tx_c)::value;
    if (cudaFuncSetAttribute(sweep_batch_kernel<float, D, S, X>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
      return 0;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sweep_batch_kernel<float, D, S, X>,
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
    if constexpr (std::is_same<T, double>::value)
      return launch_impl<T, D, S, X>(s, *a64, stream, launches);
    else
      return launch_impl<T, D, S, X>(s, *a32, stream, launches);
  });
}

}  // namespace doma
