// noalloc.cu -- one FP32 transport sweep that allocates no memory.
//
// Some callers cannot call cudaMalloc: code running inside another
// framework's memory pool, under a strict allocator budget, or in a process
// that must not change its device-memory footprint after start-up.
// doma_sweep_noalloc gives them one sweep of one group (all octants and
// ordinates, the same persistent dataflow kernel as the solver's FP32 mode)
// with every piece of device scratch -- geometry and quadrature tables, the
// task list, the dataflow flags, the face planes and the per-(octant, group)
// scalar-flux partials -- carved from the fixed array below.  Host-side
// staging uses fixed static buffers as well, so a call performs no heap or
// device allocation.
//
// Limits: the scratch array holds DOMA_NOALLOC_SCRATCH_BYTES (64 MiB; enough
// for a 64^3 mesh with 16 ordinates per octant); np and na are at most 8;
// larger problems are rejected with DOMA_BAD_INPUT and a message that gives
// the bytes needed.  Every GPU that loads this library holds the array until
// the process exits.
//
// Sharing: all calls use the same array and it keeps the last call's
// contents.  Each call re-initialises what must start at zero (scheduling
// counters and flags) before its sweep.  Calls that overlap on the GPU (from
// different streams or threads) race on the array and give wrong results;
// the host-side part of a call is serialised by a mutex, the device side is
// the caller's to order.
//
// Set-up: every call resolves the array's device address on the current
// device with cudaGetSymbolAddress (host code cannot use the array's name as
// a device address).  A call copies small tables from host memory and
// synchronises its stream before returning, to report a timed-out device
// wait, so it must not be issued on a stream that is being captured into a
// CUDA graph; it returns DOMA_BAD_INPUT there.
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

#include "common.cuh"

namespace doma {
namespace {

static __device__ __align__(256) unsigned char g_noalloc_scratch[DOMA_NOALLOC_SCRATCH_BYTES];

constexpr unsigned kMaxPolar = 8, kMaxAzimuthal = 8;
constexpr int kMaxOrdinates = 8 * kMaxPolar * kMaxAzimuthal;  // 512
constexpr int kMaxAxisCells = 4096;
constexpr size_t kMaxTasks = 1u << 17;

std::mutex g_lock;

// Host staging (static storage, reused by every call under g_lock).
Task g_tasks[kMaxTasks];
double g_quad[4][kMaxOrdinates];   // |mu|, |eta|, |xi|, w  (octant-major)
double g_quad_flat[4 * kMaxOrdinates];
double g_widths[3 * kMaxAxisCells];

struct NoallocCtl {
  unsigned ticket, exit_count, epoch;
  int error;
};

doma_status fail(const std::string & msg)
{
  set_error(msg);
  return DOMA_BAD_INPUT;
}

// The device address of the scratch array on the current device.  It is
// resolved on every call (cheap next to a sweep), so a device reset or a
// re-created primary context never leaves a stale address behind.
doma_status scratch_address(unsigned char ** out)
{
  void * p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess) {
    set_error(std::string("cudaGetSymbolAddress(no-alloc scratch): ") + cudaGetErrorString(e));
    return DOMA_CUDA_ERROR;
  }
  *out = static_cast<unsigned char *>(p);
  return DOMA_OK;
}

// Gauss-Legendre x Chebyshev quadrature into the fixed host tables, with
// absolute direction cosines: the solver's own construction (gc_quadrature,
// quadrature.cpp), which allocates nothing.
int quadrature_fixed(unsigned np, unsigned na, unsigned dims, int counts[8])
{
  unsigned c[8];
  const int D = gc_quadrature(np, na, dims, g_quad[0], g_quad[1], g_quad[2], g_quad[3], c);
  if (D < 0) return D;
  for (int k = 0; k < D; ++k)
    for (int a = 0; a < 3; ++a) g_quad[a][k] = std::abs(g_quad[a][k]);
  for (int o = 0; o < 8; ++o) counts[o] = (int)c[o];
  return D;
}

// Float tables for the FP32 sweep: 2|cosine|/width formed in double exactly
// as the solver forms them on the host, then rounded once.
__global__ void noalloc_tables(const double * quad, int D, const double * w, int nx, int ny,
                               int nz, float * amu_f, float * aeta_f, float * axi_f, float * cx,
                               float * cy, float * cz, float * wx, float * wy, float * wz)
{
  const double * amu = quad;
  const double * aeta = quad + D;
  const double * axi = quad + 2 * D;
  const double * dx = w;
  const double * dy = w + nx;
  const double * dz = w + nx + ny;
  const int total = D * (nx + ny + nz);
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
    if (e < D * nx) {
      const int n = e / nx, i = e % nx;
      cx[e] = (float)__ddiv_rn(__dmul_rn(2.0, amu[n]), dx[i]);
    } else if (e < D * (nx + ny)) {
      const int r = e - D * nx, n = r / ny, j = r % ny;
      cy[r] = (float)__ddiv_rn(__dmul_rn(2.0, aeta[n]), dy[j]);
    } else {
      const int r = e - D * (nx + ny), n = r / nz, k = r % nz;
      cz[r] = (float)__ddiv_rn(__dmul_rn(2.0, axi[n]), dz[k]);
    }
    if (e < D) {
      amu_f[e] = (float)amu[e];
      aeta_f[e] = (float)aeta[e];
      axi_f[e] = (float)axi[e];
    }
    if (e < nx) wx[e] = (float)dx[e];
    if (e < ny) wy[e] = (float)dy[e];
    if (e < nz) wz[e] = (float)dz[e];
  }
}

// phi = sum of the (octant, ordinate group) partials, in slot order: the
// same order as the solver's source-iteration epilogue.
__global__ void noalloc_reduce(const float2 * octphi, size_t N, unsigned oct_mask, int ngroups,
                               double * phi)
{
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < N;
       c += (size_t)gridDim.x * blockDim.x) {
    PartialSum ps;
    for (int o = 0; o < 8; ++o)
      if (oct_mask & (1u << o))
        for (int g = 0; g < ngroups; ++g) ps.add(octphi[((size_t)o * ngroups + g) * N + c]);
    phi[c] = __dadd_rn(0.0, ps.value());
  }
}

// Bump allocation inside the scratch array (256-byte aligned regions).
struct Carver {
  size_t off = 0;
  size_t take(size_t bytes)
  {
    const size_t at = (off + 255) & ~(size_t)255;
    off = at + bytes;
    return at;
  }
};

}  // namespace
}  // namespace doma

using namespace doma;

extern "C" doma_status doma_sweep_noalloc(const doma_problem * p, uint32_t scheme, double theta,
                                          const float * q, const float * sigma_t, double * phi_out,
                                          void * stream)
{
  if (!p || !q || !sigma_t || !phi_out) return fail("null argument");
  if (p->num_dims != 2 && p->num_dims != 3) return fail("num_dims must be 2 or 3");
  const int dims = (int)p->num_dims;
  const int nx = (int)p->nx, ny = (int)p->ny, nz = dims == 3 ? (int)p->nz : 1;
  if (nx <= 0 || ny <= 0 || nz <= 0 || (dims == 2 && p->nz != 1)) return fail("bad mesh size");
  if (nx > kMaxAxisCells || ny > kMaxAxisCells || nz > kMaxAxisCells)
    return fail("the no-alloc sweep takes at most 4096 cells per axis");
  if (!p->dx || !p->dy || (dims == 3 && !p->dz)) return fail("missing cell widths");
  if (p->num_polar == 0 || p->num_azimuthal == 0 || p->num_polar > kMaxPolar ||
      p->num_azimuthal > kMaxAzimuthal)
    return fail("the no-alloc sweep takes 1 <= np, na <= 8");
  if (scheme != DOMA_SCHEME_DD && scheme != DOMA_SCHEME_TW_DD) return fail("unknown scheme");
  if (!(theta >= 0.0 && theta <= 1.0)) return fail("theta must lie in [0, 1]");
  for (int i = 0; i < nx; ++i) if (!(p->dx[i] > 0.0)) return fail("cell widths must be positive");
  for (int j = 0; j < ny; ++j) if (!(p->dy[j] > 0.0)) return fail("cell widths must be positive");
  if (dims == 3) for (int k = 0; k < nz; ++k) if (!(p->dz[k] > 0.0)) return fail("cell widths must be positive");

  cudaStream_t s = static_cast<cudaStream_t>(stream);
  {
    // the call copies from host buffers and synchronises: never inside a capture
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    DOMA_CUDA_TRY(cudaStreamIsCapturing(s, &cap));
    if (cap != cudaStreamCaptureStatusNone)
      return fail("doma_sweep_noalloc cannot run on a stream that is being captured");
  }

  std::lock_guard<std::mutex> guard(g_lock);
  int counts[8];
  const int D = quadrature_fixed(p->num_polar, p->num_azimuthal, (unsigned)dims, counts);
  if (D <= 0) return fail("bad quadrature order");
  const int d_oct = (int)(p->num_polar * p->num_azimuthal);
  const int kg = ordinate_group(DOMA_PREC_FP32, (int)scheme);
  const int ngroups = (d_oct + kg - 1) / kg;
  unsigned oct_mask = 0;
  int offs[8];
  for (int o = 0, acc = 0; o < 8; ++o) {
    offs[o] = acc;
    acc += counts[o];
    if (counts[o]) oct_mask |= 1u << o;
  }

  // block shape and task list (level order) in static host storage
  // the solver's block lengths (pick_tile): TW-DD 16, DD 16 with many tasks per level, else 8
  const int tx = sweep_tile_x(dims == 3 ? (scheme == DOMA_SCHEME_TW_DD || ngroups >= 3 ? 16 : 8) : 32);
  const int py = dims == 3 ? 4 : 16, pz = dims == 3 ? 4 : 1;
  const int nbx = (nx + tx - 1) / tx, nby = (ny + py - 1) / py, nbz = (nz + pz - 1) / pz;
  const int levels = nbx + nby + nbz - 2;
  const size_t num_tasks = (size_t)__builtin_popcount(oct_mask) * ngroups * nbx * nby * nbz;
  if (num_tasks > kMaxTasks) return fail("the no-alloc sweep takes at most 131072 blocks");
  {
    size_t t = 0;
    for (int L = 0; L < levels; ++L)
      for (int o = 0; o < 8; ++o) {
        if (!(oct_mask & (1u << o))) continue;
        for (int og = 0; og < ngroups; ++og)
          for (int bk = 0; bk < nbz; ++bk)
            for (int bj = 0; bj < nby; ++bj) {
              const int bi = L - bj - bk;
              if (bi >= 0 && bi < nbx) g_tasks[t++] = Task{o, og, bi, bj, bk, 0};
            }
      }
    if (t != num_tasks) return fail("internal task count mismatch");
  }

  // scratch layout
  const size_t N = (size_t)nx * ny * nz;
  Carver cv;
  const size_t o_ctl = cv.take(sizeof(NoallocCtl));
  const size_t o_done = cv.take(sizeof(unsigned) * 8 * (size_t)ngroups * nbx * nby * nbz);
  const size_t o_tasks = cv.take(sizeof(Task) * num_tasks);
  const size_t o_offs = cv.take(sizeof(int) * 8);
  const size_t o_quad = cv.take(sizeof(double) * 4 * (size_t)D);
  const size_t o_w = cv.take(sizeof(double) * (size_t)(nx + ny + nz));
  const size_t o_qf = cv.take(sizeof(float) * 3 * (size_t)D);
  const size_t o_cx = cv.take(sizeof(float) * (size_t)D * nx);
  const size_t o_cy = cv.take(sizeof(float) * (size_t)D * ny);
  const size_t o_cz = cv.take(sizeof(float) * (size_t)D * nz);
  const size_t o_wf = cv.take(sizeof(float) * (size_t)(nx + ny + nz));
  const size_t slots = (size_t)ngroups * kg;  // face slots per face (padded ordinate groups)
  const size_t o_xf = cv.take(sizeof(float) * 8 * (size_t)nz * ny * slots);
  const size_t o_yf = cv.take(sizeof(float) * 8 * (size_t)nz * nx * slots);
  const size_t o_zf = cv.take(sizeof(float) * 8 * (size_t)ny * nx * slots);
  const size_t o_oct = cv.take(sizeof(float2) * 8 * (size_t)ngroups * N);
  if (cv.off > (size_t)DOMA_NOALLOC_SCRATCH_BYTES)
    return fail("the no-alloc sweep needs " + std::to_string(cv.off) + " bytes of scratch; it has " +
                std::to_string((size_t)DOMA_NOALLOC_SCRATCH_BYTES));

  unsigned char * base = nullptr;
  doma_status st = scratch_address(&base);
  if (st != DOMA_OK) return st;

  // upload the small host tables; zero what must start at zero
  std::memcpy(g_widths, p->dx, sizeof(double) * nx);
  std::memcpy(g_widths + nx, p->dy, sizeof(double) * ny);
  if (dims == 3) std::memcpy(g_widths + nx + ny, p->dz, sizeof(double) * nz);
  else g_widths[nx + ny] = 1.0;
  for (int a = 0; a < 4; ++a) std::memcpy(g_quad_flat + a * D, g_quad[a], sizeof(double) * D);
  DOMA_CUDA_TRY(cudaMemsetAsync(base + o_ctl, 0, sizeof(NoallocCtl), s));
  DOMA_CUDA_TRY(cudaMemsetAsync(base + o_done, 0, sizeof(unsigned) * 8 * (size_t)ngroups * nbx * nby * nbz, s));
  DOMA_CUDA_TRY(cudaMemcpyAsync(base + o_tasks, g_tasks, sizeof(Task) * num_tasks, cudaMemcpyHostToDevice, s));
  DOMA_CUDA_TRY(cudaMemcpyAsync(base + o_offs, offs, sizeof(offs), cudaMemcpyHostToDevice, s));
  // (pageable sources: each copy has read its host buffer when it returns)
  DOMA_CUDA_TRY(cudaMemcpyAsync(base + o_quad, g_quad_flat, sizeof(double) * 4 * D, cudaMemcpyHostToDevice, s));
  DOMA_CUDA_TRY(cudaMemcpyAsync(base + o_w, g_widths, sizeof(double) * (nx + ny + nz), cudaMemcpyHostToDevice, s));

  float * qf = reinterpret_cast<float *>(base + o_qf);
  float * wf = reinterpret_cast<float *>(base + o_wf);
  noalloc_tables<<<64, 256, 0, s>>>(reinterpret_cast<const double *>(base + o_quad), D,
                                    reinterpret_cast<const double *>(base + o_w), nx, ny, nz, qf,
                                    qf + D, qf + 2 * D, reinterpret_cast<float *>(base + o_cx),
                                    reinterpret_cast<float *>(base + o_cy),
                                    reinterpret_cast<float *>(base + o_cz), wf, wf + nx, wf + nx + ny);
  DOMA_CUDA_TRY(cudaGetLastError());

  SweepArgs<float> a{};
  a.nx = nx; a.ny = ny; a.nz = nz;
  a.d_oct = d_oct; a.d_total = D; a.ngroups = ngroups;
  a.nbx = nbx; a.nby = nby; a.nbz = nbz;
  a.num_tasks = (int)num_tasks;
  a.tasks = reinterpret_cast<const Task *>(base + o_tasks);
  a.task_offset = 0;
  a.oct_offset = reinterpret_cast<const int *>(base + o_offs);
  a.amu = reinterpret_cast<const double *>(base + o_quad);
  a.aeta = a.amu + D;
  a.axi = a.amu + 2 * D;
  a.wgt = a.amu + 3 * D;
  a.amu_f = qf; a.aeta_f = qf + D; a.axi_f = qf + 2 * D;
  a.wx = wf; a.wy = wf + nx; a.wz = wf + nx + ny;
  a.cx = reinterpret_cast<const float *>(base + o_cx);
  a.cy = reinterpret_cast<const float *>(base + o_cy);
  a.cz = reinterpret_cast<const float *>(base + o_cz);
  a.q = q;
  a.sigt = sigma_t;
  a.xf = reinterpret_cast<float *>(base + o_xf);
  a.yf = reinterpret_cast<float *>(base + o_yf);
  a.zf = reinterpret_cast<float *>(base + o_zf);
  a.wpsi = nullptr;
  a.octphi = reinterpret_cast<float2 *>(base + o_oct);
  a.theta = theta;
  NoallocCtl * ctl = reinterpret_cast<NoallocCtl *>(base + o_ctl);
  a.ticket = &ctl->ticket;
  a.exit_count = &ctl->exit_count;
  a.epoch = &ctl->epoch;
  a.done = reinterpret_cast<unsigned *>(base + o_done);
  a.error = &ctl->error;
  a.spin_limit = 1u << 22;
  a.wait_bias = 0u;

  Schedule sc;  // persistent mode: only the launch shape is used
  sc.tx = tx;
  sc.persistent = true;
  sc.threads = sweep_threads(std::min(kg, d_oct));
  sc.smem = sweep_smem_bytes(dims, DOMA_PREC_FP32, (int)scheme, tx);
  sc.many = sweep_many_ctas(DOMA_PREC_FP32, ngroups, 1);
  st = sweep_prepare(dims, DOMA_PREC_FP32, (int)scheme, tx, sc.smem, sc.many);
  if (st != DOMA_OK) return st;
  const int fit = sweep_resident_ctas(dims, DOMA_PREC_FP32, (int)scheme, tx, sc.threads, sc.smem,
                                      sc.many);
  if (fit <= 0) return fail("the sweep block does not fit on this device");
  sc.grid = std::max(1, std::min<int>(fit, (int)num_tasks));
  st = launch_sweep(dims, DOMA_PREC_FP32, (int)scheme, sc, nullptr, &a, s, nullptr);
  if (st != DOMA_OK) return st;
  noalloc_reduce<<<256, 256, 0, s>>>(a.octphi, N, oct_mask, ngroups, phi_out);
  DOMA_CUDA_TRY(cudaGetLastError());

  int err = 0;
  DOMA_CUDA_TRY(cudaMemcpyAsync(&err, &ctl->error, sizeof(int), cudaMemcpyDeviceToHost, s));
  DOMA_CUDA_TRY(cudaStreamSynchronize(s));
  if (err) {
    set_error("a sweep wait for an upstream block timed out");
    return DOMA_DEVICE_WAIT_TIMEOUT;
  }
  return DOMA_OK;
}
