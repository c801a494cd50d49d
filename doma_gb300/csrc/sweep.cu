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
// position: the next block along that axis reads it only after this block's
// launch has finished.  Tasks are launched level by level (level =
// bi + bj + bk); a level holds every independent task of all octants.
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

// DD with cx = 2|mu|/lx etc.: psi = (q + cx x + cy y + cz z) / (cx + cy + cz + st).
__device__ __forceinline__ float dd_f32(float q, float st, float cx, float cy, float cz,
                                        float & x, float & y, float & z)
{
  const float num = fmaf(cz, z, fmaf(cy, y, fmaf(cx, x, q)));
  const float c = __fdividef(num, cx + cy + cz + st);
  x = fmaf(2.0f, c, -x);
  y = fmaf(2.0f, c, -y);
  z = fmaf(2.0f, c, -z);
  return c;
}

__device__ __forceinline__ float tw_weight(float num, float den_in, float flux)
{
  // 1 - num / (den_in * flux), clamped to [0.5, 1]; 0.5 when the upwind flux is <= 1e-8.
  float a = 0.5f;
  if (flux > 1e-8f) a = 1.0f - __fdividef(num, den_in * flux);
  return fminf(fmaxf(a, 0.5f), 1.0f);
}

__device__ __forceinline__ float twdd3_f32(float q, float st, float amu, float aeta, float axi,
                                           float lx, float ly, float lz, float th, float & x,
                                           float & y, float & z)
{
  const float A = ly * lz, B = lx * lz, C = lx * ly, V = lx * ly * lz;
  const float muA = amu * A, etB = aeta * B, xiC = axi * C;
  const float qVt = q * V * th, sV = st * V;
  const float mx = muA * x, ey = etB * y, xz = xiC * z;
  const float a = tw_weight(qVt + (ey + xz) * th + mx, sV + 2.0f * (etB + xiC), x);
  const float b = tw_weight(qVt + (mx + xz) * th + ey, sV + 2.0f * (muA + xiC), y);
  const float c3 = tw_weight(qVt + (mx + ey) * th + xz, sV + 2.0f * (muA + etB), z);
  const float ra = __frcp_rn(a), rb = __frcp_rn(b), rc = __frcp_rn(c3);
  const float ta = muA * ra, tb = etB * rb, tc = xiC * rc;
  const float c = __fdividef(fmaf(tc, z, fmaf(tb, y, fmaf(ta, x, q * V))), sV + ta + tb + tc);
  x = (c - (1.0f - a) * x) * ra;
  y = (c - (1.0f - b) * y) * rb;
  z = (c - (1.0f - c3) * z) * rc;
  return c;
}

__device__ __forceinline__ float dd2_f32(float q, float st, float cx, float cy, float & x,
                                         float & y)
{
  const float c = __fdividef(fmaf(cy, y, fmaf(cx, x, q)), cx + cy + st);
  x = fmaf(2.0f, c, -x);
  y = fmaf(2.0f, c, -y);
  return c;
}

__device__ __forceinline__ float twdd2_f32(float q, float st, float amu, float aeta, float axi,
                                           float lx, float ly, float th, float & x, float & y)
{
  const float A = ly, B = lx, V = lx * ly;
  const float muA = amu * A, etB = aeta * B;
  const float qVt = q * V * th, sV = st * V;
  const float mx = muA * x, ey = etB * y;
  const float a = tw_weight(qVt + ey * th + mx, sV + 2.0f * etB, x);
  const float b = tw_weight(qVt + (mx + axi) * th + ey, sV + 2.0f * muA, y);
  const float ra = __frcp_rn(a), rb = __frcp_rn(b);
  const float ta = muA * ra, tb = etB * rb;
  const float c = __fdividef(fmaf(tb, y, fmaf(ta, x, q * V)), sV + ta + tb);
  x = (c - (1.0f - a) * x) * ra;
  y = (c - (1.0f - b) * y) * rb;
  return c;
}

// ---- the sweep kernel ------------------------------------------------------

template <typename T, int DIMS, int SCHEME>
__global__ void __launch_bounds__(kMaxSweepThreads) sweep_kernel(const SweepArgs<T> A)
{
  constexpr bool EXACT = std::is_same<T, double>::value;
  extern __shared__ __align__(16) unsigned char smem_raw[];

  const Task task = A.tasks[A.task_offset + blockIdx.x];
  const int o = task.oct;
  const bool rx = (o & 4) != 0, ry = (o & 2) != 0, rz = (o & 1) != 0;
  const int TX = A.tx, TY = A.ty, TZ = DIMS == 3 ? A.tz : 1;
  const int Do = A.d_oct;
  const int nx = A.nx, ny = A.ny, nz = DIMS == 3 ? A.nz : 1;
  const int i0 = task.bi * TX, j0 = task.bj * TY, k0 = task.bk * TZ;
  const int vx = min(TX, nx - i0), vy = min(TY, ny - j0), vz = min(TZ, nz - k0);
  const int cells = TX * TY * TZ;

  const int t = threadIdx.x;
  const int n = t % Do;
  const int pen = t / Do;
  const int jl = pen % TY;
  const int kl = pen / TY;
  const bool active = jl < vy && kl < vz;
  const int ord = A.oct_offset[o] + n;

  // shared memory carve-up (all T-sized arrays first, then the float buffer)
  T * yface = reinterpret_cast<T *>(smem_raw);     // [TZ][TX][Do]
  T * zface = yface + TZ * TX * Do;                // [TY][TX][Do] (3D)
  T * qs = zface + (DIMS == 3 ? TY * TX * Do : 0); // [TZ][TY][TX]
  T * ss = qs + cells;                             // [TZ][TY][TX]
  T * lxs = ss + cells;                            // [TX]
  T * lys = lxs + TX;                              // [TY]
  T * lzs = lys + TY;                              // [TZ]
  T * cxs = lzs + TZ;                              // [Do][TX]  2|mu|/lx
  T * cys = cxs + Do * TX;                         // [Do][TY]  2|eta|/ly
  T * czs = cys + Do * TY;                         // [Do][TZ]  2|xi|/lz
  float * P = reinterpret_cast<float *>(czs + Do * TZ);  // fp32: [cells][Do]

  auto phys_i = [&](int il) { return rx ? nx - 1 - (i0 + il) : i0 + il; };
  auto phys_j = [&](int jj) { return ry ? ny - 1 - (j0 + jj) : j0 + jj; };
  auto phys_k = [&](int kk) { return rz ? nz - 1 - (k0 + kk) : k0 + kk; };

  // -- prologue: stage cell data, widths, coefficients and incoming faces --
  for (int e = t; e < cells; e += blockDim.x) {
    const int il = e % TX, r = e / TX, jj = r % TY, kk = r / TY;
    if (il < vx && jj < vy && kk < vz) {
      const size_t c = ((size_t)phys_k(kk) * ny + phys_j(jj)) * nx + phys_i(il);
      qs[e] = A.q[c];
      ss[e] = A.sigt[c];
    }
  }
  for (int e = t; e < TX; e += blockDim.x) lxs[e] = e < vx ? (T)A.dx[phys_i(e)] : (T)1;
  for (int e = t; e < TY; e += blockDim.x) lys[e] = e < vy ? (T)A.dy[phys_j(e)] : (T)1;
  if (DIMS == 3)
    for (int e = t; e < TZ; e += blockDim.x) lzs[e] = e < vz ? (T)A.dz[phys_k(e)] : (T)1;
  const int ob = A.oct_offset[o];
  for (int e = t; e < Do * TX; e += blockDim.x) {
    const int nn = e / TX, il = e % TX;
    const double lx = il < vx ? A.dx[phys_i(il)] : 1.0;
    cxs[e] = EXACT ? (T)dD(dM(2.0, A.amu[ob + nn]), lx) : (T)(2.0 * A.amu[ob + nn] / lx);
  }
  for (int e = t; e < Do * TY; e += blockDim.x) {
    const int nn = e / TY, jj = e % TY;
    const double ly = jj < vy ? A.dy[phys_j(jj)] : 1.0;
    cys[e] = EXACT ? (T)dD(dM(2.0, A.aeta[ob + nn]), ly) : (T)(2.0 * A.aeta[ob + nn] / ly);
  }
  if (DIMS == 3)
    for (int e = t; e < Do * TZ; e += blockDim.x) {
      const int nn = e / TZ, kk = e % TZ;
      const double lz = kk < vz ? A.dz[phys_k(kk)] : 1.0;
      czs[e] = EXACT ? (T)dD(dM(2.0, A.axi[ob + nn]), lz) : (T)(2.0 * A.axi[ob + nn] / lz);
    }
  // y faces: smem [kk][il][nn] <- global yf[o][k'][i'][nn]
  for (int e = t; e < TZ * TX * Do; e += blockDim.x) {
    const int nn = e % Do, r = e / Do, il = r % TX, kk = r / TX;
    T v = (T)0;
    if (task.bj > 0 && il < vx && kk < vz)
      v = A.yf[(((size_t)o * nz + (k0 + kk)) * nx + (i0 + il)) * Do + nn];
    yface[e] = v;
  }
  if (DIMS == 3) {
    // z faces: smem [jj][il][nn] <- global zf[o][j'][i'][nn]
    for (int e = t; e < TY * TX * Do; e += blockDim.x) {
      const int nn = e % Do, r = e / Do, il = r % TX, jj = r / TX;
      T v = (T)0;
      if (task.bk > 0 && il < vx && jj < vy)
        v = A.zf[(((size_t)o * ny + (j0 + jj)) * nx + (i0 + il)) * Do + nn];
      zface[e] = v;
    }
  }
  T xin = (T)0;
  const size_t xslot = (((size_t)o * nz + (k0 + kl)) * ny + (j0 + jl)) * Do + n;
  if (active && task.bi > 0) xin = A.xf[xslot];

  T amu, aeta, axi;
  if (EXACT) {
    amu = (T)A.amu[ord]; aeta = (T)A.aeta[ord]; axi = (T)A.axi[ord];
  } else {
    amu = (T)A.amu_f[ord]; aeta = (T)A.aeta_f[ord]; axi = (T)A.axi_f[ord];
  }
  const double wgt = A.wgt[ord];
  const float wgt_f = (float)wgt;
  const T th = (T)A.theta;
  const size_t N = (size_t)nx * ny * nz;
  __syncthreads();

  // -- wavefront: step s solves the cells with il + jl + kl == s ------------
  const int steps = TX + TY + TZ - 2;
  for (int s = 0; s < steps; ++s) {
    const int il = s - jl - kl;
    if (active && il >= 0 && il < vx) {
      const int e = (kl * TY + jl) * TX + il;
      T & yref = yface[(kl * TX + il) * Do + n];
      T y = yref;
      T z = (T)0;
      if (DIMS == 3) z = zface[(jl * TX + il) * Do + n];
      const T q = qs[e], st = ss[e];
      T psi;
      if constexpr (EXACT) {
        if constexpr (DIMS == 3) {
          if constexpr (SCHEME == DOMA_SCHEME_DD) {
            const double geo = dA(dA(cxs[n * TX + il], cys[n * TY + jl]), czs[n * TZ + kl]);
            psi = dd3_exact(q, st, amu, aeta, axi, lxs[il], lys[jl], lzs[kl], geo, xin, y, z);
          } else {
            psi = twdd3_exact(q, st, amu, aeta, axi, lxs[il], lys[jl], lzs[kl], th, xin, y, z);
          }
        } else {
          if constexpr (SCHEME == DOMA_SCHEME_DD) {
            const double geo = dA(cxs[n * TX + il], cys[n * TY + jl]);
            psi = dd2_exact(q, st, amu, aeta, lxs[il], lys[jl], geo, xin, y);
          } else {
            psi = twdd2_exact(q, st, amu, aeta, axi, lxs[il], lys[jl], th, xin, y);
          }
        }
        const size_t cg = ((size_t)phys_k(kl) * ny + phys_j(jl)) * nx + phys_i(il);
        A.wpsi[cg * A.d_total + ord] = dM(wgt, psi);
      } else {
        if constexpr (DIMS == 3) {
          if constexpr (SCHEME == DOMA_SCHEME_DD)
            psi = dd_f32(q, st, cxs[n * TX + il], cys[n * TY + jl], czs[n * TZ + kl], xin, y, z);
          else
            psi = twdd3_f32(q, st, amu, aeta, axi, lxs[il], lys[jl], lzs[kl], th, xin, y, z);
        } else {
          if constexpr (SCHEME == DOMA_SCHEME_DD)
            psi = dd2_f32(q, st, cxs[n * TX + il], cys[n * TY + jl], xin, y);
          else
            psi = twdd2_f32(q, st, amu, aeta, axi, lxs[il], lys[jl], th, xin, y);
        }
        P[e * Do + n] = wgt_f * psi;
      }
      yref = y;
      if (DIMS == 3) zface[(jl * TX + il) * Do + n] = z;
    }
    __syncthreads();
  }

  // -- epilogue: outgoing faces and (fp32) the per-octant scalar flux ---------
  if (active) A.xf[xslot] = xin;
  for (int e = t; e < TZ * TX * Do; e += blockDim.x) {
    const int nn = e % Do, r = e / Do, il = r % TX, kk = r / TX;
    if (il < vx && kk < vz) A.yf[(((size_t)o * nz + (k0 + kk)) * nx + (i0 + il)) * Do + nn] = yface[e];
  }
  if (DIMS == 3) {
    for (int e = t; e < TY * TX * Do; e += blockDim.x) {
      const int nn = e % Do, r = e / Do, il = r % TX, jj = r / TX;
      if (il < vx && jj < vy)
        A.zf[(((size_t)o * ny + (j0 + jj)) * nx + (i0 + il)) * Do + nn] = zface[e];
    }
  }
  if constexpr (!EXACT) {
    for (int e = t; e < cells; e += blockDim.x) {
      const int il = e % TX, r = e / TX, jj = r % TY, kk = r / TY;
      if (il < vx && jj < vy && kk < vz) {
        float s = 0.0f, comp = 0.0f;
        const float * pv = P + (size_t)e * Do;
        for (int nn = 0; nn < Do; ++nn) {  // Kahan, fixed ordinate order
          const float yv = pv[nn] - comp;
          const float tv = s + yv;
          comp = (tv - s) - yv;
          s = tv;
        }
        const size_t cg = ((size_t)phys_k(kk) * ny + phys_j(jj)) * nx + phys_i(il);
        A.octphi[(size_t)o * N + cg] = (double)s - (double)comp;
      }
    }
  }
}

template <typename T, int DIMS, int SCHEME>
doma_status launch_levels(const Schedule & s, const SweepArgs<T> & args, cudaStream_t stream,
                          uint64_t * launches)
{
  SweepArgs<T> a = args;
  const int levels = (int)s.level_begin.size() - 1;
  for (int L = 0; L < levels; ++L) {
    const int count = s.level_begin[L + 1] - s.level_begin[L];
    if (count == 0) continue;
    a.task_offset = s.level_begin[L];
    sweep_kernel<T, DIMS, SCHEME><<<count, s.threads, s.smem, stream>>>(a);
    if (launches) ++*launches;
  }
  DOMA_CUDA_TRY(cudaGetLastError());
  return DOMA_OK;
}

template <typename T, int DIMS, int SCHEME>
cudaError_t set_smem_attr(size_t smem)
{
  return cudaFuncSetAttribute(sweep_kernel<T, DIMS, SCHEME>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

}  // namespace

size_t sweep_smem_bytes(int dims, int precision, int scheme, int tx, int ty, int tz, int d_oct)
{
  (void)scheme;
  const size_t ts = precision == DOMA_PREC_FP64 ? 8 : 4;
  const size_t tzz = dims == 3 ? tz : 1;
  const size_t cells = (size_t)tx * ty * tzz;
  size_t n = tzz * tx * d_oct;                       // y faces
  if (dims == 3) n += (size_t)ty * tx * d_oct;       // z faces
  n += 2 * cells + tx + ty + tzz;                    // q, sigma_t, widths
  n += (size_t)d_oct * (tx + ty + tzz);              // coefficients
  size_t bytes = n * ts;
  if (precision == DOMA_PREC_FP32) bytes += cells * d_oct * 4;  // P
  return bytes;
}

doma_status sweep_prepare(size_t smem)
{
  if (smem <= 48 * 1024) return DOMA_OK;
  cudaError_t e = cudaSuccess;
  cudaError_t r;
#define DOMA_SET(T, D, S) if ((r = set_smem_attr<T, D, S>(smem)) != cudaSuccess) e = r;
  DOMA_SET(double, 3, DOMA_SCHEME_DD) DOMA_SET(double, 3, DOMA_SCHEME_TW_DD)
  DOMA_SET(double, 2, DOMA_SCHEME_DD) DOMA_SET(double, 2, DOMA_SCHEME_TW_DD)
  DOMA_SET(float, 3, DOMA_SCHEME_DD) DOMA_SET(float, 3, DOMA_SCHEME_TW_DD)
  DOMA_SET(float, 2, DOMA_SCHEME_DD) DOMA_SET(float, 2, DOMA_SCHEME_TW_DD)
#undef DOMA_SET
  DOMA_CUDA_TRY(e);
  return DOMA_OK;
}

doma_status launch_sweep(int dims, int precision, int scheme, const Schedule & s,
                         const SweepArgs<double> * a64, const SweepArgs<float> * a32,
                         cudaStream_t stream, uint64_t * launches)
{
  const bool tw = scheme == DOMA_SCHEME_TW_DD;
  if (precision == DOMA_PREC_FP64) {
    if (dims == 3)
      return tw ? launch_levels<double, 3, DOMA_SCHEME_TW_DD>(s, *a64, stream, launches)
                : launch_levels<double, 3, DOMA_SCHEME_DD>(s, *a64, stream, launches);
    return tw ? launch_levels<double, 2, DOMA_SCHEME_TW_DD>(s, *a64, stream, launches)
              : launch_levels<double, 2, DOMA_SCHEME_DD>(s, *a64, stream, launches);
  }
  if (dims == 3)
    return tw ? launch_levels<float, 3, DOMA_SCHEME_TW_DD>(s, *a32, stream, launches)
              : launch_levels<float, 3, DOMA_SCHEME_DD>(s, *a32, stream, launches);
  return tw ? launch_levels<float, 2, DOMA_SCHEME_TW_DD>(s, *a32, stream, launches)
            : launch_levels<float, 2, DOMA_SCHEME_DD>(s, *a32, stream, launches);
}

}  // namespace doma
