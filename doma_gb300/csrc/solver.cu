// solver.cu -- the C ABI: solver handle, device buffers, and the
// Gauss-Seidel / source-iteration driver.
//
// The driver follows TransportSolver3D::solveFixedSource
// (src/TransportSolver3D.cpp:262-316) and ::sourceIteration (:458-497) step by
// step, including their exit rules: SI stops when it reaches fs_max_it or the
// residual is <= fs_tol and succeeds iff it < fs_max_it; the Gauss-Seidel loop
// runs once for one group and succeeds iff mg_it < mg_max_it; a norm whose
// total is <= 1e-8 gives residual 0.  One deliberate difference: a NaN or
// infinite norm stops the solve with DOMA_NUMERIC_ERROR (DOMA would report
// convergence, because `tol < NaN` is false).
//
// Device layout (one solver = one problem, all resident in HBM):
//   per cell   : material index, volume, q and sigma_t of the current group
//                (sweep precision), the increment's octant partials (fp32:
//                [8][N] double) or the weighted angular flux (exact: [N][D] double)
//   per group  : phi and the previous Gauss-Seidel iterate, [G][N] double
//   per octant : face planes x [nz][ny][Do], y [nz][nx][Do], z [ny][nx][Do]
//   materials  : total [M][G], scatter [M][G][G], source, fission data
#include <chrono>
#include <cmath>
#include <cstddef>
#include <cstdlib>
#include <type_traits>
#include <cstdio>
#include <cstring>
#include <map>
#include <new>
#include <tuple>
#include <array>
#include <string>
#include <vector>

#include "accel.cuh"
#include "common.cuh"
#include "iteration.cuh"
#include "unet.cuh"

namespace doma {

namespace {
thread_local std::string g_error;
}

void set_error(const std::string & msg) { g_error = msg; }
const char * get_error() { return g_error.c_str(); }

}  // namespace doma

using namespace doma;

using DevCtl = LoopCtl;

struct doma_solver {
  int dims = 3, nx = 1, ny = 1, nz = 1, G = 1, M = 1;
  size_t N = 0;
  int D = 0, d_oct = 0;
  unsigned oct_mask = 0;
  bool mgi = false;     // multigroup iteration: every group in flight
  int gif = 1;          // groups in flight per sweep (G in multigroup mode, else 1)
  double * d_dscratch = nullptr;   // multigroup mode: [G][N] increments
  cudaGraph_t mgi_graph = nullptr;
  cudaGraphExec_t mgi_exec = nullptr;
  doma_options opts{};
  int offs[8] = {0};

  // device buffers
  double *d_dx = nullptr, *d_dy = nullptr, *d_dz = nullptr, *d_vol = nullptr;
  uint32_t * d_mat = nullptr;
  double *d_total = nullptr, *d_scatter = nullptr, *d_source = nullptr;
  uint8_t * d_fis = nullptr;
  double *d_chi = nullptr, *d_nsf = nullptr;
  double *d_amu = nullptr, *d_aeta = nullptr, *d_axi = nullptr, *d_w = nullptr;
  float *d_amu_f = nullptr, *d_aeta_f = nullptr, *d_axi_f = nullptr;
  int * d_oct_offset = nullptr;
  double *d_phi = nullptr, *d_prev = nullptr;
  void *d_q = nullptr, *d_sigt = nullptr;
  void *d_xf = nullptr, *d_yf = nullptr, *d_zf = nullptr;
  double * d_wpsi = nullptr;
  float2 * d_octphi = nullptr;
  void *d_wx = nullptr, *d_wy = nullptr, *d_wz = nullptr;   // widths, sweep precision
  void *d_cx = nullptr, *d_cy = nullptr, *d_cz = nullptr;   // 2|cosine|/width tables
  double * d_partials = nullptr;
  unsigned * d_ticket = nullptr;
  DevCtl * d_ctl = nullptr;
  unsigned * d_done = nullptr;  // [tasks] persistent-sweep done epochs
  Task * d_tasks = nullptr;
  DevCtl * h_ctl = nullptr;     // pinned mirror

  // graph-driven solve
  unsigned * d_pair_counts = nullptr;
  double * d_pair_res = nullptr;
  double * d_mg_hist = nullptr;
  double * d_si_hist = nullptr;
  unsigned pair_cap = 0, mg_cap = 0;
  unsigned long long hist_cap = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t graph_exec = nullptr;
  bool use_graph = true;

  Schedule sched;
  cudaStream_t stream = nullptr;
  cudaStream_t own_stream = nullptr;
  uint64_t launches = 0;
  int device = 0;

  SweepArgs<double> a64{};
  SweepArgs<float> a32{};
  IterArgs it{};
  std::vector<void *> allocations;

  // learned accelerator and reference-error stop (multigroup mode)
  doma_unet * accel = nullptr;
  doma_accel_options accel_opts{};
  float *d_fsig = nullptr, *d_fabs = nullptr, *d_kappa = nullptr;   // [G][N]
  float *d_corr = nullptr;                                            // [G][N]
  float *d_r = nullptr, *d_ya = nullptr, *d_yb = nullptr, *d_nn_out = nullptr;  // [N]
  void * d_nn_in = nullptr;                                           // [N][16] bf16
  double * d_rms = nullptr;                                           // [G]
  double *d_phi_save = nullptr, *d_delta_save = nullptr;              // [G][N]
  double * d_acc_partials = nullptr;                                  // [grid]
  unsigned * d_acc_ticket = nullptr;
  double * d_ref = nullptr;                                           // [G][N]
  // a correction's kernels (per group: residual, input, U-Net forward,
  // correction) captured as one graph after a first, eager correction
  cudaGraph_t acc_graph = nullptr;
  cudaGraphExec_t acc_exec = nullptr;
  const doma_unet * acc_net = nullptr;   // the net and workspace it was captured over
  unsigned long long acc_gen = 0;
  bool acc_warm = false;
  double ref_norm2 = 0.0, ref_target = 0.0;
  doma_accel_stats stats{};

  // k-eigenvalue mode: host copies of the flux and the previous iterate for
  // the k update, which sums in DOMA's order (pinned, allocated on first use),
  // and of the per-cell data that update reads
  double *h_phi = nullptr, *h_prev = nullptr;
  bool fissile = false;
  std::vector<uint32_t> h_mat;   // [N]
  std::vector<double> h_vol;     // [N] cell volume (area in 2D)
  std::vector<uint8_t> h_fis;    // [M]
  std::vector<double> h_nsf;     // [M][G]

  // transient mode: device tables and state, allocated on first use for
  // tr_D delayed groups (grown, with the graph rebuilt, when a call needs
  // more); the captured Gauss-Seidel graph of a transient step
  cudaGraph_t eg_graph = nullptr;        // k-eigenvalue: one power iteration's group loop
  cudaGraphExec_t eg_exec = nullptr;
  double * d_k = nullptr;                 // the k that graph reads
  double * h_k = nullptr;                 // pinned staging of k
  TransientArgs tr{};
  int tr_D = 0;
  std::vector<void *> tr_allocs;
  double * h_dnps = nullptr;     // pinned [tr_D][N], for the step callback
  cudaGraph_t tr_graph = nullptr;
  cudaGraphExec_t tr_exec = nullptr;
};

namespace {

template <typename T>
doma_status dalloc(doma_solver * s, T ** p, size_t count)
{
  *p = nullptr;
  if (count == 0) return DOMA_OK;
  void * v = nullptr;
  cudaError_t e = cudaMalloc(&v, count * sizeof(T));
  if (e != cudaSuccess) {
    set_error(std::string("cudaMalloc(") + std::to_string(count * sizeof(T)) +
              " bytes): " + cudaGetErrorString(e));
    return DOMA_CUDA_ERROR;
  }
  s->allocations.push_back(v);
  *p = static_cast<T *>(v);
  return DOMA_OK;
}

template <typename T>
doma_status upload(doma_solver * s, T ** p, const T * host, size_t count)
{
  doma_status st = dalloc(s, p, count);
  if (st != DOMA_OK || count == 0) return st;
  DOMA_CUDA_TRY(cudaMemcpy(*p, host, count * sizeof(T), cudaMemcpyHostToDevice));
  return DOMA_OK;
}

doma_status bad(const std::string & msg)
{
  set_error(msg);
  return DOMA_BAD_INPUT;
}

doma_status validate(const doma_problem * p, const doma_options * o)
{
  if (!p || !o) return bad("null problem or options");
  if (p->num_dims != 2 && p->num_dims != 3) return bad("num_dims must be 2 or 3");
  if (p->nx == 0 || p->ny == 0 || p->nz == 0) return bad("empty mesh");
  if (p->num_dims == 2 && p->nz != 1) return bad("a 2D problem needs nz == 1");
  if (!p->dx || !p->dy || (p->num_dims == 3 && !p->dz)) return bad("missing cell widths");
  if (p->num_groups == 0) return bad("num_groups must be positive");
  if (p->num_materials == 0) return bad("num_materials must be positive");
  if (!p->cell_material || !p->total || !p->scatter) return bad("missing material data");
  if (p->has_fission && (!p->chi_p || !p->nu_sigma_f))
    return bad("has_fission given without chi_p / nu_sigma_f");
  if (p->num_polar == 0 || p->num_azimuthal == 0) return bad("np and na must be positive");
  if ((uint64_t)p->num_polar * p->num_azimuthal > 4096u)
    return bad("np*na (ordinates per octant) must be <= 4096");
  const uint64_t N = (uint64_t)p->nx * p->ny * p->nz;
  if (N > (1ull << 31)) return bad("too many cells");
  for (uint64_t c = 0; c < N; ++c)
    if (p->cell_material[c] >= p->num_materials)
      return bad("cell " + std::to_string(c) + " has material " +
                 std::to_string(p->cell_material[c]) + " >= num_materials");
  auto positive = [](const double * v, size_t n) {
    for (size_t i = 0; i < n; ++i)
      if (!(v[i] > 0.0) || !std::isfinite(v[i])) return false;
    return true;
  };
  if (!positive(p->dx, p->nx) || !positive(p->dy, p->ny) ||
      (p->num_dims == 3 && !positive(p->dz, p->nz)))
    return bad("cell widths must be positive and finite");
  if (o->scheme != DOMA_SCHEME_DD && o->scheme != DOMA_SCHEME_TW_DD) return bad("unknown scheme");
  if (o->precision != DOMA_PREC_FP64 && o->precision != DOMA_PREC_FP32)
    return bad("unknown precision");
  if (!(o->theta >= 0.0 && o->theta <= 1.0)) return bad("theta must lie in [0, 1]");
  if (o->iteration != DOMA_ITER_GAUSS_SEIDEL && o->iteration != DOMA_ITER_MULTIGROUP)
    return bad("unknown iteration");
  return DOMA_OK;
}

// Block shape: tx cells along x (8, 16 or 32) by the kernel's fixed 16-pencil
// cross-section; ordinates split into groups of at most ordinate_group(precision,
// scheme) per task.
void pick_tile(doma_solver * s, const doma_options * o)
{
  const int kg = ordinate_group((int)o->precision, (int)o->scheme);
  s->sched.ngroups = (s->d_oct + kg - 1) / kg;
  s->sched.gs = std::min(kg, s->d_oct);
  // Measured on GB300 with the present bodies (3D): TW-DD 64^3 347, 261, 291 us
  // for 8, 16, 32-cell blocks.  DD wants 8-cell blocks when a wavefront level
  // holds few tasks (64^3 and 48^3 with 16 ordinates: 186 against 193 us, 110
  // against 121 us) and 16 when it holds many (the 100^3 duct with 36
  // ordinates: 1253 against 1312 us; the FP64 duct 0.96 against 1.21 s), the
  // criterion of the register bodies (sweep_many_ctas, counted here with the
  // mode's own ordinate groups).  2D takes 32.
  const bool many = s->sched.ngroups * s->gif >= 3;
  const int want3 = o->scheme == DOMA_SCHEME_TW_DD ? 16 : (many ? 16 : 8);
  const int want = o->tile_x ? (int)o->tile_x : (s->dims == 3 ? want3 : 32);
  s->sched.tx = sweep_tile_x(want);
  s->sched.ty = s->dims == 3 ? 4 : 16;
  s->sched.tz = s->dims == 3 ? 4 : 1;
}

void build_schedule(doma_solver * s)
{
  Schedule & sc = s->sched;
  sc.nbx = (s->nx + sc.tx - 1) / sc.tx;
  sc.nby = (s->ny + sc.ty - 1) / sc.ty;
  sc.nbz = (s->nz + sc.tz - 1) / sc.tz;
  sc.threads = sweep_threads(sc.gs);
  sc.smem = sweep_smem_bytes(s->dims, s->opts.precision, s->opts.scheme, sc.tx);
  sc.many = sweep_many_ctas(s->opts.precision, sc.ngroups, s->gif);
  {
    // DOMA_SWEEP_MANY=0/1 picks the FP32 body by hand (the tests run both)
    const char * env = std::getenv("DOMA_SWEEP_MANY");
    if (env && s->opts.precision == DOMA_PREC_FP32) sc.many = std::string(env) == "1";
  }
  const int levels = sc.nbx + sc.nby + sc.nbz - 2;
  std::vector<std::vector<Task>> by_level(levels);
  for (int g = 0; g < s->gif; ++g)
    for (int o = 0; o < 8; ++o) {
      if (!(s->oct_mask & (1u << o))) continue;
      for (int og = 0; og < sc.ngroups; ++og)
        for (int bk = 0; bk < sc.nbz; ++bk)
          for (int bj = 0; bj < sc.nby; ++bj)
            for (int bi = 0; bi < sc.nbx; ++bi)
              by_level[bi + bj + bk].push_back(Task{o, og, bi, bj, bk, g});
    }
  sc.tasks.clear();
  sc.level_begin.assign(1, 0);
  for (auto & lv : by_level) {
    sc.tasks.insert(sc.tasks.end(), lv.begin(), lv.end());
    sc.level_begin.push_back((int)sc.tasks.size());
  }
}

doma_status create_impl(const doma_problem * p, const doma_options * o, doma_solver * s)
{
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    set_error("no CUDA device is visible");
    return DOMA_NO_DEVICE;
  }
  DOMA_CUDA_TRY(cudaGetDevice(&s->device));
  s->opts = *o;
  s->dims = (int)p->num_dims;
  s->nx = (int)p->nx;
  s->ny = (int)p->ny;
  s->nz = s->dims == 3 ? (int)p->nz : 1;
  s->G = (int)p->num_groups;
  s->M = (int)p->num_materials;
  s->N = (size_t)s->nx * s->ny * s->nz;
  s->d_oct = (int)(p->num_polar * p->num_azimuthal);
  s->D = (s->dims == 3 ? 8 : 4) * s->d_oct;
  s->mgi = o->iteration == DOMA_ITER_MULTIGROUP;
  s->gif = s->mgi ? s->G : 1;

  std::vector<double> mu(s->D), eta(s->D), xi(s->D), w(s->D);
  unsigned counts[8];
  if (gc_quadrature(p->num_polar, p->num_azimuthal, p->num_dims, mu.data(), eta.data(),
                    xi.data(), w.data(), counts) != s->D)
    return bad("quadrature construction failed");
  int off = 0;
  for (int oc = 0; oc < 8; ++oc) {
    s->offs[oc] = off;
    off += (int)counts[oc];
    if (counts[oc]) {
      s->oct_mask |= 1u << oc;
      if ((int)counts[oc] != s->d_oct) return bad("unexpected octant size");
    }
  }
  std::vector<double> amu(s->D), aeta(s->D), axi(s->D);
  std::vector<float> amu_f(s->D), aeta_f(s->D), axi_f(s->D);
  for (int n = 0; n < s->D; ++n) {
    amu[n] = std::abs(mu[n]);
    aeta[n] = std::abs(eta[n]);
    axi[n] = std::abs(xi[n]);
    amu_f[n] = (float)amu[n];
    aeta_f[n] = (float)aeta[n];
    axi_f[n] = (float)axi[n];
  }

  // geometry and materials
  const size_t N = s->N, G = s->G, M = s->M;
  std::vector<double> dz(s->nz, 1.0);
  if (s->dims == 3) dz.assign(p->dz, p->dz + s->nz);
  std::vector<double> vol(N);
  for (int k = 0; k < s->nz; ++k)
    for (int j = 0; j < s->ny; ++j)
      for (int i = 0; i < s->nx; ++i) {
        const size_t c = ((size_t)k * s->ny + j) * s->nx + i;
        vol[c] = s->dims == 3 ? p->dx[i] * p->dy[j] * dz[k] : p->dx[i] * p->dy[j];
      }
  DOMA_TRY(upload(s, &s->d_dx, p->dx, (size_t)s->nx));
  DOMA_TRY(upload(s, &s->d_dy, p->dy, (size_t)s->ny));
  DOMA_TRY(upload(s, &s->d_dz, dz.data(), (size_t)s->nz));
  DOMA_TRY(upload(s, &s->d_vol, vol.data(), N));
  DOMA_TRY(upload(s, &s->d_mat, p->cell_material, N));
  DOMA_TRY(upload(s, &s->d_total, p->total, M * G));
  DOMA_TRY(upload(s, &s->d_scatter, p->scatter, M * G * G));
  if (p->source) DOMA_TRY(upload(s, &s->d_source, p->source, M * G));
  if (p->has_fission) {
    DOMA_TRY(upload(s, &s->d_fis, p->has_fission, M));
    DOMA_TRY(upload(s, &s->d_chi, p->chi_p, M * G));
    DOMA_TRY(upload(s, &s->d_nsf, p->nu_sigma_f, M * G));
  }
  s->h_mat.assign(p->cell_material, p->cell_material + N);
  s->h_vol = vol;
  s->h_fis.assign(M, 0u);
  s->h_nsf.assign(M * G, 0.0);
  if (p->has_fission) {
    s->h_fis.assign(p->has_fission, p->has_fission + M);
    s->h_nsf.assign(p->nu_sigma_f, p->nu_sigma_f + M * G);
    for (size_t m = 0; m < M; ++m) s->fissile = s->fissile || s->h_fis[m] != 0u;
  }
  DOMA_TRY(upload(s, &s->d_amu, amu.data(), (size_t)s->D));
  DOMA_TRY(upload(s, &s->d_aeta, aeta.data(), (size_t)s->D));
  DOMA_TRY(upload(s, &s->d_axi, axi.data(), (size_t)s->D));
  DOMA_TRY(upload(s, &s->d_w, w.data(), (size_t)s->D));
  DOMA_TRY(upload(s, &s->d_amu_f, amu_f.data(), (size_t)s->D));
  DOMA_TRY(upload(s, &s->d_aeta_f, aeta_f.data(), (size_t)s->D));
  DOMA_TRY(upload(s, &s->d_axi_f, axi_f.data(), (size_t)s->D));
  DOMA_TRY(upload(s, &s->d_oct_offset, s->offs, 8));

  // state
  const bool exact = o->precision == DOMA_PREC_FP64;
  const size_t ts = exact ? sizeof(double) : sizeof(float);

  // Sweep-precision geometry tables.  The coefficient 2|mu|/dx is formed on
  // the host exactly as DOMA forms it per cell solve ((2.0 * |mu|) / l_x,
  // include/DiamondDifference3D.h:36), so the exact mode sees the same bits.
  {
    const int D = s->D;
    std::vector<double> cx((size_t)D * s->nx), cy((size_t)D * s->ny), cz((size_t)D * s->nz);
    for (int n = 0; n < D; ++n) {
      for (int i = 0; i < s->nx; ++i) cx[(size_t)n * s->nx + i] = (2.0 * amu[n]) / p->dx[i];
      for (int j = 0; j < s->ny; ++j) cy[(size_t)n * s->ny + j] = (2.0 * aeta[n]) / p->dy[j];
      for (int k = 0; k < s->nz; ++k) cz[(size_t)n * s->nz + k] = (2.0 * axi[n]) / dz[k];
    }
    std::vector<double> wx(p->dx, p->dx + s->nx), wy(p->dy, p->dy + s->ny), wz(dz);
    auto put = [&](void ** dst, const std::vector<double> & v) -> doma_status {
      if (exact) {
        double * d = nullptr;
        DOMA_TRY(upload(s, &d, v.data(), v.size()));
        *dst = d;
      } else {
        std::vector<float> f(v.begin(), v.end());
        float * d = nullptr;
        DOMA_TRY(upload(s, &d, f.data(), f.size()));
        *dst = d;
      }
      return DOMA_OK;
    };
    DOMA_TRY(put(&s->d_cx, cx));
    DOMA_TRY(put(&s->d_cy, cy));
    DOMA_TRY(put(&s->d_cz, cz));
    DOMA_TRY(put(&s->d_wx, wx));
    DOMA_TRY(put(&s->d_wy, wy));
    DOMA_TRY(put(&s->d_wz, wz));
  }
  DOMA_TRY(dalloc(s, &s->d_phi, G * N));
  DOMA_TRY(dalloc(s, &s->d_prev, G * N));
  const size_t gif = (size_t)s->gif;
  unsigned char * qb = nullptr;
  DOMA_TRY(dalloc(s, &qb, 2 * gif * N * ts));
  s->d_q = qb;
  s->d_sigt = qb + gif * N * ts;
  // face planes: ordinate_group slots per face for each ordinate group (the
  // last group padded), so a task's faces along a row are contiguous
  const int kg = ordinate_group((int)s->opts.precision, (int)s->opts.scheme);
  const size_t Do = (size_t)((s->d_oct + kg - 1) / kg) * kg;
  unsigned char * fb = nullptr;
  const size_t xf = gif * 8 * (size_t)s->nz * s->ny * Do, yf = gif * 8 * (size_t)s->nz * s->nx * Do,
               zf = gif * 8 * (size_t)s->ny * s->nx * Do;
  DOMA_TRY(dalloc(s, &fb, (xf + yf + zf) * ts));
  s->d_xf = fb;
  s->d_yf = fb + xf * ts;
  s->d_zf = fb + (xf + yf) * ts;
  if (exact)
    DOMA_TRY(dalloc(s, &s->d_wpsi, gif * N * (size_t)s->D));
  else
    DOMA_TRY(dalloc(s, &s->d_octphi, gif * 8 * (size_t)((s->d_oct + kg - 1) / kg) * N));
  if (s->mgi) DOMA_TRY(dalloc(s, &s->d_dscratch, (size_t)s->G * N));

  pick_tile(s, o);
  build_schedule(s);
  if (s->sched.smem > 227 * 1024) return bad("sweep block needs too much shared memory");
  DOMA_TRY(sweep_prepare(s->dims, o->precision, o->scheme, s->sched.tx, s->sched.smem, s->sched.many));
  DOMA_TRY(upload(s, &s->d_tasks, s->sched.tasks.data(), s->sched.tasks.size()));
  {
    const char * env = std::getenv("DOMA_SWEEP_SCHEDULE");
    s->sched.persistent = !(env && std::string(env) == "levels");
    const int fit = sweep_resident_ctas(s->dims, o->precision, o->scheme, s->sched.tx,
                                        s->sched.threads, s->sched.smem, s->sched.many);
    if (fit <= 0) return bad("the sweep block does not fit on this device");
    s->sched.grid = std::max(1, std::min<int>(fit, (int)s->sched.tasks.size()));
    // one flag per (octant slot, block): indexed by octant 0..7 even when
    // only four octants carry ordinates (2D)
    const size_t flags = (size_t)s->gif * 8 * s->sched.ngroups * s->sched.nbx * s->sched.nby * s->sched.nbz;
    DOMA_TRY(dalloc(s, &s->d_done, flags));
    DOMA_CUDA_TRY(cudaMemset(s->d_done, 0, flags * sizeof(unsigned)));
  }

  // per-cell kernels: fixed grid (determinism of the norms depends on it)
  int sms = 0;
  DOMA_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, s->device));
  const size_t blocks_needed = (N + iteration_block() - 1) / iteration_block();
  const int grid = (int)std::max<size_t>(1, std::min<size_t>(blocks_needed, (size_t)sms * 8));
  // the FP32 epilogue's grid: fewer, longer threads amortise its FP64 block reduction
  const int epi_grid = (int)std::max<size_t>(1, std::min<size_t>(blocks_needed, (size_t)sms * 3));
  DOMA_TRY(dalloc(s, &s->d_partials, 2 * (size_t)std::max(grid, epi_grid)));
  DOMA_TRY(dalloc(s, &s->d_ticket, 1));
  DOMA_CUDA_TRY(cudaMemset(s->d_ticket, 0, sizeof(unsigned)));
  DOMA_TRY(dalloc(s, &s->d_ctl, 1));
  DOMA_CUDA_TRY(cudaMemset(s->d_ctl, 0, sizeof(DevCtl)));
  DOMA_CUDA_TRY(cudaMallocHost(&s->h_ctl, sizeof(DevCtl)));
  std::memset(s->h_ctl, 0, sizeof(DevCtl));
  {
    // histories of the graph-driven solve: one entry per (MG iteration, group)
    // pair and per MG iteration; every SI residual only for verbose output
    const char * env = std::getenv("DOMA_SOLVE_LOOP");
    s->use_graph = !(env && std::string(env) == "host");
    s->pair_cap = (unsigned)std::min<uint64_t>((uint64_t)o->mg_max_it * s->G + s->G, 1u << 22);
    s->mg_cap = std::max(1u, o->mg_max_it);
    DOMA_TRY(dalloc(s, &s->d_pair_counts, s->pair_cap));
    DOMA_TRY(dalloc(s, &s->d_pair_res, s->pair_cap));
    DOMA_TRY(dalloc(s, &s->d_mg_hist, s->mg_cap));
    if (o->verbose >= 2) {
      s->hist_cap = std::min<uint64_t>((uint64_t)o->fs_max_it * s->pair_cap, 1ull << 24);
      DOMA_TRY(dalloc(s, &s->d_si_hist, (size_t)s->hist_cap));
    }
  }
  DOMA_CUDA_TRY(cudaStreamCreateWithFlags(&s->own_stream, cudaStreamNonBlocking));
  s->stream = s->own_stream;

  // kernel argument blocks
  auto fill = [&](auto & a, auto * tp) {
    using T = std::remove_pointer_t<decltype(tp)>;
    a.nx = s->nx; a.ny = s->ny; a.nz = s->nz;
    a.d_oct = s->d_oct; a.d_total = s->D; a.ngroups = s->sched.ngroups;
    a.nbx = s->sched.nbx; a.nby = s->sched.nby; a.nbz = s->sched.nbz;
    a.tx = s->sched.tx;
    a.num_tasks = (int)s->sched.tasks.size();
    a.tasks = s->d_tasks; a.task_offset = 0; a.oct_offset = s->d_oct_offset;
    a.amu = s->d_amu; a.aeta = s->d_aeta; a.axi = s->d_axi; a.wgt = s->d_w;
    a.amu_f = s->d_amu_f; a.aeta_f = s->d_aeta_f; a.axi_f = s->d_axi_f;
    a.wx = (const T *)s->d_wx; a.wy = (const T *)s->d_wy; a.wz = (const T *)s->d_wz;
    a.cx = (const T *)s->d_cx; a.cy = (const T *)s->d_cy; a.cz = (const T *)s->d_cz;
    a.q = (const T *)s->d_q; a.sigt = (const T *)s->d_sigt;
    a.xf = (T *)s->d_xf; a.yf = (T *)s->d_yf; a.zf = (T *)s->d_zf;
    a.wpsi = s->d_wpsi; a.octphi = s->d_octphi; a.theta = o->theta;
    a.ticket = &s->d_ctl->ticket; a.exit_count = &s->d_ctl->exit_count;
    a.epoch = &s->d_ctl->epoch; a.done = s->d_done; a.error = &s->d_ctl->error;
    a.spin_limit = 1u << 22;
    a.wait_bias = 0u;
    // Failure-detection test: every upstream wait targets an epoch nobody
    // publishes and gives up after 2000 polls, so the sweep reports
    // DOMA_DEVICE_WAIT_TIMEOUT without hanging or faulting.
    const char * wt = std::getenv("DOMA_SWEEP_WAIT_TEST");
    if (wt && std::string(wt) == "1") {
      a.spin_limit = 2000u;
      a.wait_bias = 0x40000000u;
    }
  };
  if (exact)
    fill(s->a64, (double *)nullptr);
  else
    fill(s->a32, (float *)nullptr);
  IterArgs & it = s->it;
  it.N = N; it.G = s->G; it.D = s->D; it.grid = grid; it.epi_grid = epi_grid;
  it.oct_mask = s->oct_mask;
  it.ngroups = s->sched.ngroups;
  it.exact = exact;
  it.src_scale = s->dims == 3 ? 0.25 : 0.5;
  it.vol = s->d_vol; it.mat = s->d_mat; it.total = s->d_total; it.scatter = s->d_scatter;
  it.source = s->d_source; it.fis = s->d_fis; it.chi = s->d_chi; it.nsf = s->d_nsf;
  it.phi = s->d_phi; it.prev = s->d_prev; it.wpsi = s->d_wpsi; it.octphi = s->d_octphi;
  it.partials = s->d_partials; it.ticket = s->d_ticket;
  {
    std::vector<double> qc(M * G);
    const double sc = it.src_scale;
    for (size_t m = 0; m < M; ++m)
      for (size_t g = 0; g < G; ++g)
        qc[m * G + g] = sc * p->scatter[(m * G + g) * G + g] / M_PI;
    double * d_qc = nullptr;
    DOMA_TRY(upload(s, &d_qc, qc.data(), M * G));
    it.qcoef = d_qc;
  }
  if (!exact && !s->mgi) {
    // the FP32 Gauss-Seidel mode's group-source tables (mg_source_kernel<float>)
    const double sc = it.src_scale;
    std::vector<double> mc(M * G * G, 0.0), sq(M * G, 0.0);
    for (size_t m = 0; m < M; ++m)
      for (size_t g = 0; g < G; ++g) {
        if (p->source) sq[m * G + g] = sc * p->source[m * G + g] / M_PI;
        const bool fis = p->has_fission && p->has_fission[m];
        for (size_t gp = 0; gp < G; ++gp) {
          double v = gp != g ? p->scatter[(m * G + g) * G + gp] : 0.0;
          if (fis) v += p->chi_p[m * G + g] * p->nu_sigma_f[m * G + gp];
          mc[(m * G + g) * G + gp] = sc * v / M_PI;
        }
      }
    double *d_mc = nullptr, *d_sq = nullptr;
    DOMA_TRY(upload(s, &d_mc, mc.data(), M * G * G));
    DOMA_TRY(upload(s, &d_sq, sq.data(), M * G));
    it.mgcoef = d_mc;
    it.srcq = d_sq;
  }

  DOMA_CUDA_TRY(cudaMemset(s->d_phi, 0, G * N * sizeof(double)));
  DOMA_CUDA_TRY(cudaMemset(s->d_prev, 0, G * N * sizeof(double)));
  DOMA_CUDA_TRY(cudaMemset(s->d_q, 0, 2 * gif * N * ts));
  DOMA_CUDA_TRY(cudaDeviceSynchronize());
  return DOMA_OK;
}

void release(doma_solver * s)
{
  if (!s) return;
  if (s->mgi_exec) cudaGraphExecDestroy(s->mgi_exec);
  if (s->mgi_graph) cudaGraphDestroy(s->mgi_graph);
  if (s->graph_exec) cudaGraphExecDestroy(s->graph_exec);
  if (s->graph) cudaGraphDestroy(s->graph);
  for (void * p : s->allocations) cudaFree(p);
  if (s->h_ctl) cudaFreeHost(s->h_ctl);
  if (s->h_phi) cudaFreeHost(s->h_phi);
  if (s->h_prev) cudaFreeHost(s->h_prev);
  if (s->eg_exec) cudaGraphExecDestroy(s->eg_exec);
  if (s->eg_graph) cudaGraphDestroy(s->eg_graph);
  if (s->h_k) cudaFreeHost(s->h_k);
  if (s->tr_exec) cudaGraphExecDestroy(s->tr_exec);
  if (s->tr_graph) cudaGraphDestroy(s->tr_graph);
  if (s->acc_exec) cudaGraphExecDestroy(s->acc_exec);
  if (s->acc_graph) cudaGraphDestroy(s->acc_graph);
  for (void * p : s->tr_allocs) cudaFree(p);
  if (s->h_dnps) cudaFreeHost(s->h_dnps);
  if (s->own_stream) cudaStreamDestroy(s->own_stream);
  delete s;
}

doma_status sweep_once(doma_solver * s)
{
  return launch_sweep(s->dims, s->opts.precision, s->opts.scheme, s->sched, &s->a64, &s->a32,
                      s->stream, &s->launches);
}

// One source iteration: sweep, epilogue; norms land in d_ctl->norms[0..1].
doma_status source_iteration(doma_solver * s, int g)
{
  DOMA_TRY(sweep_once(s));
  DOMA_TRY(launch_si_epilogue(s->it, g, s->opts.precision, s->d_q, s->d_ctl->norms, LoopParams{}, s->stream));
  ++s->launches;
  return DOMA_OK;
}

// Read a norm pair and the sweep error flag (synchronises the stream).
doma_status read_norms(doma_solver * s, int first, double * diff, double * tot)
{
  DOMA_CUDA_TRY(cudaMemcpyAsync(s->h_ctl, s->d_ctl, offsetof(DevCtl, ticket),
                                cudaMemcpyDeviceToHost, s->stream));
  DOMA_CUDA_TRY(cudaStreamSynchronize(s->stream));
  if (s->h_ctl->error) {
    set_error("a sweep wait for an upstream block timed out");
    return DOMA_DEVICE_WAIT_TIMEOUT;
  }
  *diff = s->h_ctl->norms[first];
  *tot = s->h_ctl->norms[first + 1];
  return DOMA_OK;
}

double ratio(double diff, double tot)
{
  return tot > 1e-8 ? std::sqrt(diff) / std::sqrt(tot) : 0.0;
}

// Tallies of a host-driven solve.
struct Tally {
  uint64_t sweeps = 0;
  size_t si_len = 0;
  unsigned mg = 0;
  double mg_res = 0.0, si_res = 0.0;
};

// True for the statuses after which a solve still reports (the iteration
// stopped); false for errors that end the call at once.
bool reportable(doma_status st)
{
  return st == DOMA_OK || st == DOMA_NOT_CONVERGED || st == DOMA_NUMERIC_ERROR;
}

// sourceIteration (src/TransportSolver3D.cpp:458-497) for group g, its source
// already staged: sweep + epilogue until the SI residual is at most fs_tol or
// fs_max_it is reached, with DOMA's progress lines.  The count goes to
// r->si_counts.  Returns DOMA_OK, DOMA_NOT_CONVERGED (fs_max_it reached),
// DOMA_NUMERIC_ERROR or the error that stopped it.
doma_status group_source_iteration(doma_solver * s, int g, doma_report * r, Tally & t)
{
  const doma_options & o = s->opts;
  const int verbose = (int)o.verbose;
  unsigned it = 0;
  t.si_res = 0.0;
  doma_status status = DOMA_OK;
  do {
    if (verbose >= 2) {
      if (it != 0u)
        std::printf("Performing SI %u for G%d, residual = %g\n", it, g, t.si_res);
      else
        std::printf("Performing SI %u for G%d\n", it, g);
    }
    DOMA_TRY(source_iteration(s, g));
    ++t.sweeps;
    double diff, tot;
    DOMA_TRY(read_norms(s, 0, &diff, &tot));
    if (!std::isfinite(diff) || !std::isfinite(tot)) {
      set_error("source iteration norm is not finite (group " + std::to_string(g) + ")");
      status = DOMA_NUMERIC_ERROR;
      break;
    }
    t.si_res = ratio(diff, tot);
    ++it;
  } while (it < o.fs_max_it && o.fs_tol < t.si_res);
  if (r && r->si_counts && t.si_len < r->si_counts_capacity) r->si_counts[t.si_len] = it;
  ++t.si_len;
  if (status != DOMA_OK) return status;
  if (it < o.fs_max_it) {
    if (verbose)
      std::printf("SI converged after %u iterations with a residual of %g for G%d\n", it,
                  t.si_res, g);
    return DOMA_OK;
  }
  if (verbose)
    std::printf("SI failed to converge after %u iterations with a residual of %g for G%d\n", it,
                t.si_res, g);
  return DOMA_NOT_CONVERGED;
}

// The Gauss-Seidel loop of solveFixedSource (src/TransportSolver3D.cpp:271-315),
// host-driven: stage(g) sets up group g's source, then its source iteration;
// the MG residual after each pass over the groups; DOMA's progress lines.
template <typename Stage>
doma_status gs_host_loop(doma_solver * s, Stage && stage, doma_report * r, Tally & t)
{
  const doma_options & o = s->opts;
  const int verbose = (int)o.verbose;
  doma_status status = DOMA_OK;
  t.mg = 0;
  t.mg_res = 0.0;
  do {
    if (verbose) {
      if (t.mg != 0u)
        std::printf("Performing MGI %u, residual = %g\n", t.mg, t.mg_res);
      else
        std::printf("Performing MGI %u\n", t.mg);
      std::printf("----------------------------------------------------------------------------------\n");
    }
    for (int g = 0; g < s->G && status == DOMA_OK; ++g) {
      DOMA_TRY(stage(g));
      ++s->launches;
      status = group_source_iteration(s, g, r, t);
      if (!reportable(status)) return status;
    }
    if (status != DOMA_OK) break;
    DOMA_TRY(launch_mg_residual(s->it, s->d_ctl->norms + 2, LoopParams{}, s->stream));
    ++s->launches;
    double diff, tot;
    DOMA_TRY(read_norms(s, 2, &diff, &tot));
    if (!std::isfinite(diff) || !std::isfinite(tot)) {
      set_error("Gauss-Seidel norm is not finite");
      status = DOMA_NUMERIC_ERROR;
      break;
    }
    t.mg_res = ratio(diff, tot);
    ++t.mg;
  } while (t.mg < o.mg_max_it && o.mg_tol < t.mg_res && s->G > 1);

  if (status == DOMA_OK) {
    if (t.mg < o.mg_max_it) {
      if (verbose && s->G > 1)
        std::printf("MGI converged after %u iterations with a residual of %g\n", t.mg, t.mg_res);
    } else {
      if (verbose)
        std::printf("MGI failed to converge after %u iterations with a residual of %g\n", t.mg,
                    t.mg_res);
      status = DOMA_NOT_CONVERGED;
      set_error("Gauss-Seidel iteration reached mg_max_it");
    }
  } else if (status == DOMA_NOT_CONVERGED) {
    set_error("source iteration reached fs_max_it");
  }
  return status;
}

void fill_report(const doma_solver * s, doma_report * r, doma_status status, const Tally & t,
                 std::chrono::steady_clock::time_point t0, uint64_t launches0)
{
  if (!r) return;
  const auto t1 = std::chrono::steady_clock::now();
  r->status = status;
  r->mg_iterations = t.mg;
  r->si_iterations = t.sweeps;
  r->updates = t.sweeps * (uint64_t)s->N * (uint64_t)s->D;
  r->kernel_launches = s->launches - launches0;
  r->mg_residual = t.mg_res;
  r->si_residual = t.si_res;
  r->solve_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
  r->si_counts_len = t.si_len;
}

LoopParams loop_params(doma_solver * s, int G)
{
  LoopParams L;
  L.ctl = s->d_ctl;
  L.pair_counts = s->d_pair_counts;
  L.pair_res = s->d_pair_res;
  L.pair_cap = s->pair_cap;
  L.si_hist = s->d_si_hist;
  L.hist_cap = s->hist_cap;
  L.mg_hist = s->d_mg_hist;
  L.mg_cap = s->mg_cap;
  L.fs_tol = s->opts.fs_tol;
  L.mg_tol = s->opts.mg_tol;
  L.fs_max_it = s->opts.fs_max_it;
  L.mg_max_it = s->opts.mg_max_it;
  L.G = G;
  L.graph = 1;
  return L;
}

// Insert a WHILE conditional node at the current position of a capture and
// return its (empty) body graph.
doma_status add_while(cudaStream_t cap, cudaGraphConditionalHandle h, cudaGraph_t * body)
{
  cudaStreamCaptureStatus st;
  cudaGraph_t g = nullptr;
  const cudaGraphNode_t * deps = nullptr;
  size_t ndeps = 0;
  DOMA_CUDA_TRY(cudaStreamGetCaptureInfo(cap, &st, nullptr, &g, &deps, nullptr, &ndeps));
  if (st != cudaStreamCaptureStatusActive) {
    set_error("stream is not capturing");
    return DOMA_CUDA_ERROR;
  }
  cudaGraphNodeParams np{};
  np.type = cudaGraphNodeTypeConditional;
  np.conditional.handle = h;
  np.conditional.type = cudaGraphCondTypeWhile;
  np.conditional.size = 1;
  cudaGraphNode_t node;
  DOMA_CUDA_TRY(cudaGraphAddNode(&node, g, deps, nullptr, ndeps, &np));
  DOMA_CUDA_TRY(cudaStreamUpdateCaptureDependencies(cap, &node, nullptr, 1,
                                                    cudaStreamSetCaptureDependencies));
  *body = np.conditional.phGraph_out[0];
  return DOMA_OK;
}

// The whole fixed-source solve as one graph:
//   WHILE(mg) { for g: mg_source(g) ; WHILE(si_g) { sweep ; si_epilogue(g) } ;
//               mg_residual }
// mg_source arms its group's SI loop, the epilogue decides whether the SI
// loop goes on, the Gauss-Seidel residual kernel decides the outer loop.
// Capture the Gauss-Seidel / source-iteration loop as one graph with WHILE
// nodes: the fixed-source solve, or (transient) one time step, whose source
// kernel reads t and dt from the device clock.
doma_status build_graph(doma_solver * s, bool transient)
{
  cudaStream_t c0 = nullptr, c1 = nullptr, c2 = nullptr;
  DOMA_CUDA_TRY(cudaStreamCreateWithFlags(&c0, cudaStreamNonBlocking));
  DOMA_CUDA_TRY(cudaStreamCreateWithFlags(&c1, cudaStreamNonBlocking));
  DOMA_CUDA_TRY(cudaStreamCreateWithFlags(&c2, cudaStreamNonBlocking));
  doma_status status = DOMA_OK;
  auto fail = [&](doma_status st) {
    status = st;
    return st;
  };
  auto run = [&]() -> doma_status {
    cudaGraph_t root = nullptr;
    if (cudaGraphCreate(&root, 0) != cudaSuccess) return fail(DOMA_CUDA_ERROR);
    (transient ? s->tr_graph : s->graph) = root;
    cudaGraphConditionalHandle mg_h;
    DOMA_CUDA_TRY(cudaGraphConditionalHandleCreate(&mg_h, root, 1u, cudaGraphCondAssignDefault));
    std::vector<cudaGraphConditionalHandle> si_h(s->G);
    for (int g = 0; g < s->G; ++g)
      DOMA_CUDA_TRY(cudaGraphConditionalHandleCreate(&si_h[g], root, 0u, 0u));

    DOMA_CUDA_TRY(cudaStreamBeginCaptureToGraph(c0, root, nullptr, nullptr, 0,
                                                cudaStreamCaptureModeThreadLocal));
    cudaGraph_t mg_body = nullptr;
    doma_status st = add_while(c0, mg_h, &mg_body);
    if (st == DOMA_OK) {
      DOMA_CUDA_TRY(cudaStreamBeginCaptureToGraph(c1, mg_body, nullptr, nullptr, 0,
                                                  cudaStreamCaptureModeThreadLocal));
      for (int g = 0; g < s->G && st == DOMA_OK; ++g) {
        LoopParams L = loop_params(s, s->G);
        L.si_handle = si_h[g];
        L.mg_handle = mg_h;
        st = transient ? launch_mg_source_transient(s->it, s->tr, g, s->opts.precision, s->d_q,
                                                    s->d_sigt, L, c1)
                       : launch_mg_source(s->it, g, s->opts.precision, s->d_q, s->d_sigt, L, c1);
        cudaGraph_t si_body = nullptr;
        if (st == DOMA_OK) st = add_while(c1, si_h[g], &si_body);
        if (st == DOMA_OK) {
          DOMA_CUDA_TRY(cudaStreamBeginCaptureToGraph(c2, si_body, nullptr, nullptr, 0,
                                                      cudaStreamCaptureModeThreadLocal));
          st = launch_sweep(s->dims, s->opts.precision, s->opts.scheme, s->sched, &s->a64,
                            &s->a32, c2, nullptr);
          if (st == DOMA_OK)
            st = launch_si_epilogue(s->it, g, s->opts.precision, s->d_q, s->d_ctl->norms, L, c2);
          cudaGraph_t out = nullptr;
          DOMA_CUDA_TRY(cudaStreamEndCapture(c2, &out));
        }
      }
      if (st == DOMA_OK) {
        LoopParams L = loop_params(s, s->G);
        L.mg_handle = mg_h;
        st = launch_mg_residual(s->it, s->d_ctl->norms + 2, L, c1);
      }
      cudaGraph_t out = nullptr;
      DOMA_CUDA_TRY(cudaStreamEndCapture(c1, &out));
    }
    cudaGraph_t out = nullptr;
    DOMA_CUDA_TRY(cudaStreamEndCapture(c0, &out));
    if (st != DOMA_OK) return fail(st);
    DOMA_CUDA_TRY(cudaGraphInstantiate(transient ? &s->tr_exec : &s->graph_exec, root, 0));
    return DOMA_OK;
  };
  doma_status st = run();
  cudaStreamDestroy(c0);
  cudaStreamDestroy(c1);
  cudaStreamDestroy(c2);
  if (st != DOMA_OK && status == DOMA_OK) status = st;
  return status;
}

// Print DOMA's progress lines (src/TransportSolver3D.cpp:268-315,466-494)
// from the histories the graph recorded.
// One launch of a captured Gauss-Seidel graph, read back: the loop state and
// the per-(MG iteration, group) SI counts and residual histories.
struct GraphRun {
  DevCtl c{};
  std::vector<unsigned> counts;
  std::vector<double> pres, mgh, sih;
};

// sourceIteration's lines (src/TransportSolver3D.cpp:466-494) for one pass over
// the groups, from a graph run's history starting at (pair, hist); false when
// a group failed (the solve stops there).
bool print_si_pass(doma_solver * s, const GraphRun & run, size_t & pair, size_t & hist)
{
  const DevCtl & c = run.c;
  const std::vector<unsigned> & counts = run.counts;
  const std::vector<double> &pres = run.pres, &sih = run.sih;
  const int verbose = (int)s->opts.verbose;
  for (int g = 0; g < s->G && pair < c.pairs; ++g, ++pair) {
    const unsigned n = pair < counts.size() ? counts[pair] : 0u;
    const double r = pair < pres.size() ? pres[pair] : 0.0;
    if (verbose >= 2)
      for (unsigned k = 0; k < n; ++k, ++hist) {
        if (k != 0u && hist - 1 < sih.size())
          std::printf("Performing SI %u for G%d, residual = %g\n", k, g, sih[hist - 1]);
        else
          std::printf("Performing SI %u for G%d\n", k, g);
      }
    if (n < s->opts.fs_max_it && !(c.failed && pair + 1 == c.pairs)) {
      std::printf("SI converged after %u iterations with a residual of %g for G%d\n", n, r, g);
    } else {
      std::printf("SI failed to converge after %u iterations with a residual of %g for G%d\n", n, r, g);
      return false;
    }
  }
  return true;
}

void print_history(doma_solver * s, const GraphRun & run, bool banner)
{
  const DevCtl & c = run.c;
  const std::vector<double> & mgh = run.mgh;
  const int G = s->G;
  if (banner) std::printf("Solving...\nInitializing the solver...\n");
  size_t pair = 0, hist = 0;
  for (unsigned m = 0;; ++m) {
    if (pair >= c.pairs) break;
    if (m != 0u)
      std::printf("Performing MGI %u, residual = %g\n", m, mgh[m - 1]);
    else
      std::printf("Performing MGI %u\n", m);
    std::printf("----------------------------------------------------------------------------------\n");
    if (!print_si_pass(s, run, pair, hist)) break;
  }
  if (!c.failed) {
    if (c.mg_it < s->opts.mg_max_it) {
      if (G > 1)
        std::printf("MGI converged after %u iterations with a residual of %g\n", c.mg_it, c.mg_res);
    } else {
      std::printf("MGI failed to converge after %u iterations with a residual of %g\n", c.mg_it,
                  c.mg_res);
    }
  }
  std::fflush(stdout);
}

doma_status graph_run(doma_solver * s, cudaGraphExec_t exec, GraphRun & out)
{
  // clear error and loop state; keep the persistent-sweep counters
  DOMA_CUDA_TRY(cudaMemsetAsync(&s->d_ctl->error, 0, sizeof(int), s->stream));
  DOMA_CUDA_TRY(cudaMemsetAsync(&s->d_ctl->si_it, 0, sizeof(DevCtl) - offsetof(DevCtl, si_it),
                                s->stream));
  DOMA_CUDA_TRY(cudaGraphLaunch(exec, s->stream));
  DOMA_CUDA_TRY(cudaMemcpyAsync(s->h_ctl, s->d_ctl, sizeof(DevCtl), cudaMemcpyDeviceToHost, s->stream));
  DOMA_CUDA_TRY(cudaStreamSynchronize(s->stream));
  out.c = *s->h_ctl;
  const DevCtl & c = out.c;
  const size_t npairs = std::min<size_t>(c.pairs, s->pair_cap);
  out.counts.assign(npairs, 0u);
  out.pres.assign(npairs, 0.0);
  out.mgh.assign(std::min<size_t>(c.mg_it, s->mg_cap), 0.0);
  out.sih.clear();
  if (npairs) {
    DOMA_CUDA_TRY(cudaMemcpy(out.counts.data(), s->d_pair_counts, npairs * sizeof(unsigned),
                             cudaMemcpyDeviceToHost));
    DOMA_CUDA_TRY(cudaMemcpy(out.pres.data(), s->d_pair_res, npairs * sizeof(double),
                             cudaMemcpyDeviceToHost));
  }
  if (!out.mgh.empty())
    DOMA_CUDA_TRY(cudaMemcpy(out.mgh.data(), s->d_mg_hist, out.mgh.size() * sizeof(double),
                             cudaMemcpyDeviceToHost));
  if (s->d_si_hist && c.hist_len) {
    out.sih.resize(std::min<unsigned long long>(c.hist_len, s->hist_cap));
    DOMA_CUDA_TRY(cudaMemcpy(out.sih.data(), s->d_si_hist, out.sih.size() * sizeof(double),
                             cudaMemcpyDeviceToHost));
  }
  return DOMA_OK;
}

// The status a graph run ended with (and its error message).
doma_status graph_status(const doma_solver * s, const DevCtl & c)
{
  if (c.failed == DOMA_DEVICE_WAIT_TIMEOUT) {
    set_error("a sweep wait for an upstream block timed out");
    return DOMA_DEVICE_WAIT_TIMEOUT;
  }
  if (c.failed == DOMA_NUMERIC_ERROR) {
    set_error("a residual norm is not finite");
    return DOMA_NUMERIC_ERROR;
  }
  if (c.failed == DOMA_NOT_CONVERGED) {
    set_error("source iteration reached fs_max_it");
    return DOMA_NOT_CONVERGED;
  }
  if (!(c.mg_it < s->opts.mg_max_it)) {
    set_error("Gauss-Seidel iteration reached mg_max_it");
    return DOMA_NOT_CONVERGED;
  }
  return DOMA_OK;
}

// Kernel launches of a graph run: G sources + one MG residual per MG
// iteration and (sweep launches + 1) per source iteration.
uint64_t graph_launches(const doma_solver * s, const DevCtl & c)
{
  uint64_t per_sweep = s->sched.persistent ? 1 : 0;
  if (!s->sched.persistent)
    for (size_t L = 0; L + 1 < s->sched.level_begin.size(); ++L)
      per_sweep += s->sched.level_begin[L + 1] > s->sched.level_begin[L];
  return c.sweeps * (per_sweep + 1) +
         (uint64_t)(c.mg_it + (c.failed ? 1 : 0)) * (uint64_t)(s->G + 1);
}

// One power iteration's group loop as a graph: per group the eigen source
// (k read from the device) and the source-iteration WHILE loop; the power
// iteration itself, with DOMA's host-side k update, stays on the host.
doma_status build_eigen_graph(doma_solver * s)
{
  cudaStream_t c0 = nullptr, c2 = nullptr;
  DOMA_CUDA_TRY(cudaStreamCreateWithFlags(&c0, cudaStreamNonBlocking));
  DOMA_CUDA_TRY(cudaStreamCreateWithFlags(&c2, cudaStreamNonBlocking));
  auto run = [&]() -> doma_status {
    cudaGraph_t root = nullptr;
    DOMA_CUDA_TRY(cudaGraphCreate(&root, 0));
    s->eg_graph = root;
    std::vector<cudaGraphConditionalHandle> si_h(s->G);
    for (int g = 0; g < s->G; ++g)
      DOMA_CUDA_TRY(cudaGraphConditionalHandleCreate(&si_h[g], root, 0u, 0u));
    DOMA_CUDA_TRY(cudaStreamBeginCaptureToGraph(c0, root, nullptr, nullptr, 0,
                                                cudaStreamCaptureModeThreadLocal));
    doma_status st = DOMA_OK;
    for (int g = 0; g < s->G && st == DOMA_OK; ++g) {
      LoopParams L = loop_params(s, s->G);
      L.si_handle = si_h[g];
      st = launch_mg_source_eigen(s->it, g, s->opts.precision, 0.0, s->d_k, s->d_q, s->d_sigt, L, c0);
      cudaGraph_t si_body = nullptr;
      if (st == DOMA_OK) st = add_while(c0, si_h[g], &si_body);
      if (st == DOMA_OK) {
        DOMA_CUDA_TRY(cudaStreamBeginCaptureToGraph(c2, si_body, nullptr, nullptr, 0,
                                                    cudaStreamCaptureModeThreadLocal));
        st = launch_sweep(s->dims, s->opts.precision, s->opts.scheme, s->sched, &s->a64, &s->a32,
                          c2, nullptr);
        if (st == DOMA_OK)
          st = launch_si_epilogue(s->it, g, s->opts.precision, s->d_q, s->d_ctl->norms, L, c2);
        cudaGraph_t out = nullptr;
        DOMA_CUDA_TRY(cudaStreamEndCapture(c2, &out));
      }
    }
    cudaGraph_t out = nullptr;
    DOMA_CUDA_TRY(cudaStreamEndCapture(c0, &out));
    if (st != DOMA_OK) return st;
    DOMA_CUDA_TRY(cudaGraphInstantiate(&s->eg_exec, root, 0));
    return DOMA_OK;
  };
  const doma_status st = run();
  cudaStreamDestroy(c0);
  cudaStreamDestroy(c2);
  return st;
}

doma_status solve_graph(doma_solver * s, doma_report * r)
{
  const size_t G = s->G, N = s->N;
  const auto t0 = std::chrono::steady_clock::now();
  if (!s->graph_exec) DOMA_TRY(build_graph(s, false));
  DOMA_CUDA_TRY(cudaMemsetAsync(s->d_phi, 0, G * N * sizeof(double), s->stream));
  DOMA_CUDA_TRY(cudaMemsetAsync(s->d_prev, 0, G * N * sizeof(double), s->stream));
  GraphRun run;
  DOMA_TRY(graph_run(s, s->graph_exec, run));
  const DevCtl & c = run.c;
  if (s->opts.verbose) print_history(s, run, true);
  const doma_status status = graph_status(s, c);
  const uint64_t launches = graph_launches(s, c);
  s->launches += launches;
  const auto t1 = std::chrono::steady_clock::now();
  if (r) {
    r->status = status;
    r->mg_iterations = c.mg_it;
    r->si_iterations = c.sweeps;
    r->updates = c.sweeps * (uint64_t)s->N * (uint64_t)s->D;
    r->kernel_launches = launches;
    r->mg_residual = c.mg_res;
    r->si_residual = c.si_res;
    r->solve_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
    r->si_counts_len = c.pairs;
    if (r->si_counts)
      for (size_t k = 0; k < run.counts.size() && k < r->si_counts_capacity; ++k)
        r->si_counts[k] = run.counts[k];
  }
  return status;
}

// ---- multigroup mode (every group in flight) ------------------------------

// One multigroup iteration: all-group sweep, then the epilogue that forms the
// next increment's source for every group.
doma_status mgi_iteration(doma_solver * s, const LoopParams & L, cudaStream_t st)
{
  DOMA_TRY(launch_sweep(s->dims, s->opts.precision, s->opts.scheme, s->sched, &s->a64, &s->a32,
                        st, &s->launches));
  DOMA_TRY(launch_mgi_epilogue(s->it, s->opts.precision, s->d_q, s->d_dscratch, s->d_ctl->norms, L,
                               st));
  ++s->launches;
  return DOMA_OK;
}

// WHILE(si) { sweep(all groups); mgi_epilogue } -- the epilogue decides.
doma_status build_mgi_graph(doma_solver * s)
{
  cudaStream_t c0 = nullptr, c1 = nullptr;
  DOMA_CUDA_TRY(cudaStreamCreateWithFlags(&c0, cudaStreamNonBlocking));
  DOMA_CUDA_TRY(cudaStreamCreateWithFlags(&c1, cudaStreamNonBlocking));
  auto run = [&]() -> doma_status {
    DOMA_CUDA_TRY(cudaGraphCreate(&s->mgi_graph, 0));
    cudaGraphConditionalHandle h;
    DOMA_CUDA_TRY(cudaGraphConditionalHandleCreate(&h, s->mgi_graph, 1u, cudaGraphCondAssignDefault));
    DOMA_CUDA_TRY(cudaStreamBeginCaptureToGraph(c0, s->mgi_graph, nullptr, nullptr, 0,
                                                cudaStreamCaptureModeThreadLocal));
    cudaGraph_t body = nullptr;
    doma_status st = add_while(c0, h, &body);
    if (st == DOMA_OK) {
      DOMA_CUDA_TRY(cudaStreamBeginCaptureToGraph(c1, body, nullptr, nullptr, 0,
                                                  cudaStreamCaptureModeThreadLocal));
      LoopParams L = loop_params(s, s->G);
      L.si_handle = h;
      const uint64_t before = s->launches;
      st = mgi_iteration(s, L, c1);
      s->launches = before;
      cudaGraph_t out = nullptr;
      DOMA_CUDA_TRY(cudaStreamEndCapture(c1, &out));
    }
    cudaGraph_t out = nullptr;
    DOMA_CUDA_TRY(cudaStreamEndCapture(c0, &out));
    if (st != DOMA_OK) return st;
    DOMA_CUDA_TRY(cudaGraphInstantiate(&s->mgi_exec, s->mgi_graph, 0));
    return DOMA_OK;
  };
  const doma_status st = run();
  cudaStreamDestroy(c0);
  cudaStreamDestroy(c1);
  return st;
}

doma_status solve_multigroup(doma_solver * s, doma_report * r)
{
  const auto t0 = std::chrono::steady_clock::now();
  const size_t G = s->G, N = s->N;
  const doma_options & o = s->opts;
  if (o.verbose) std::printf("Solving (multigroup source iteration, all %d groups in flight)...\n", s->G);
  DOMA_CUDA_TRY(cudaMemsetAsync(s->d_prev, 0, G * N * sizeof(double), s->stream));
  DOMA_CUDA_TRY(cudaMemsetAsync(&s->d_ctl->error, 0, sizeof(int), s->stream));
  DOMA_CUDA_TRY(cudaMemsetAsync(&s->d_ctl->si_it, 0, sizeof(DevCtl) - offsetof(DevCtl, si_it),
                                s->stream));
  DOMA_TRY(launch_mgi_init(s->it, o.precision, s->d_q, s->d_sigt, s->stream));
  uint64_t launches = 1;
  unsigned iters = 0;
  double res = 0.0;
  doma_status status = DOMA_OK;
  std::vector<double> hist;
  if (s->use_graph) {
    if (!s->mgi_exec) DOMA_TRY(build_mgi_graph(s));
    DOMA_CUDA_TRY(cudaGraphLaunch(s->mgi_exec, s->stream));
    DOMA_CUDA_TRY(cudaMemcpyAsync(s->h_ctl, s->d_ctl, sizeof(DevCtl), cudaMemcpyDeviceToHost, s->stream));
    DOMA_CUDA_TRY(cudaStreamSynchronize(s->stream));
    const DevCtl c = *s->h_ctl;
    iters = c.si_it;
    res = c.si_res;
    launches += 2ull * iters;
    if (c.failed) status = (doma_status)c.failed;
    if (s->d_si_hist && c.hist_len) {
      hist.resize(std::min<unsigned long long>(c.hist_len, s->hist_cap));
      DOMA_CUDA_TRY(cudaMemcpy(hist.data(), s->d_si_hist, hist.size() * sizeof(double),
                               cudaMemcpyDeviceToHost));
    }
  } else {
    const LoopParams L{};
    do {
      DOMA_TRY(mgi_iteration(s, L, s->stream));
      launches += 2;
      double diff, tot;
      DOMA_TRY(read_norms(s, 0, &diff, &tot));
      ++iters;
      if (!std::isfinite(diff) || !std::isfinite(tot)) {
        status = DOMA_NUMERIC_ERROR;
        break;
      }
      res = ratio(diff, tot);
      hist.push_back(res);
    } while (iters < o.fs_max_it && o.fs_tol < res);
    if (status == DOMA_OK && !(iters < o.fs_max_it)) status = DOMA_NOT_CONVERGED;
  }
  if (o.verbose >= 2)
    for (size_t k = 0; k < hist.size(); ++k)
      std::printf("Performing MGSI %zu, residual = %g\n", k, hist[k]);
  if (o.verbose) {
    std::printf("Multigroup source iteration %s after %u iterations with a residual of %g\n",
                status == DOMA_OK ? "converged" : "failed to converge", iters, res);
    std::fflush(stdout);
  }
  if (status == DOMA_NOT_CONVERGED) set_error("multigroup source iteration reached fs_max_it");
  else if (status == DOMA_NUMERIC_ERROR) set_error("a residual norm is not finite");
  else if (status == DOMA_DEVICE_WAIT_TIMEOUT) set_error("a sweep wait for an upstream block timed out");
  if (s->use_graph) s->launches += launches;  // (the host loop counted its own launches)
  const auto t1 = std::chrono::steady_clock::now();
  if (r) {
    r->status = status;
    r->mg_iterations = iters;
    r->si_iterations = (uint64_t)iters * G;
    r->updates = (uint64_t)iters * G * N * (uint64_t)s->D;
    r->kernel_launches = launches;
    r->mg_residual = res;
    r->si_residual = res;
    r->solve_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
    r->si_counts_len = 1;
    if (r->si_counts && r->si_counts_capacity) r->si_counts[0] = iters;
  }
  return status;
}

// ---- guided multigroup solve: learned corrections and/or a reference stop --

// Network corrections for every group in order (y chain), then the next
// sweep's source from delta + Delta.
// The kernels of one correction, in group order (the y chain).
doma_status accel_correction_kernels(doma_solver * s, cudaStream_t st)
{
  const size_t N = s->N;
  float * y_prev = nullptr;
  float * ya = s->d_ya;
  float * yb = s->d_yb;
  for (int g = 0; g < s->G; ++g) {
    DOMA_TRY(accel_residual(s->it, g, s->d_dscratch, s->d_kappa, y_prev, s->d_r, s->d_acc_partials,
                            s->d_acc_ticket, s->d_rms + g, st));
    DOMA_TRY(accel_input(N, g, s->d_r, s->d_rms + g, s->d_fsig, s->d_fabs,
                         static_cast<__nv_bfloat16 *>(s->d_nn_in), st));
    DOMA_TRY(unet_forward(s->accel, static_cast<const __nv_bfloat16 *>(s->d_nn_in), s->d_nn_out, 1,
                          s->nz, s->ny, s->nx, st));
    DOMA_TRY(accel_correct(N, g, s->d_nn_out, s->d_rms + g, s->d_r, s->d_kappa, y_prev, s->d_corr,
                           ya, st));
    y_prev = ya;
    std::swap(ya, yb);
  }
  return DOMA_OK;
}

// A correction is G U-Net forwards and 3G small kernels, about 250 short
// launches: after a first, eager correction (which sizes the network's
// workspace and configures its kernels) they are captured once as a graph and
// replayed.  The graph is rebuilt when the net or its workspace changed.
// DOMA_ACCEL_GRAPH=0 keeps the launches eager.
doma_status accel_correction_launch(doma_solver * s, cudaStream_t st)
{
  const char * env = std::getenv("DOMA_ACCEL_GRAPH");
  // (the legacy default stream cannot be captured)
  const bool use_graph = !(env && std::string(env) == "0") && st != nullptr && st != cudaStreamLegacy;
  const bool stale = s->acc_net != s->accel || s->acc_gen != s->accel->work_gen;
  if (stale) {
    if (s->acc_exec) cudaGraphExecDestroy(s->acc_exec);
    if (s->acc_graph) cudaGraphDestroy(s->acc_graph);
    s->acc_exec = nullptr;
    s->acc_graph = nullptr;
    s->acc_warm = false;
  }
  if (!use_graph || !s->acc_warm) {
    DOMA_TRY(accel_correction_kernels(s, st));
    s->acc_warm = true;
    s->acc_net = s->accel;
    s->acc_gen = s->accel->work_gen;
    return DOMA_OK;
  }
  if (!s->acc_exec) {
    DOMA_CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    const doma_status cst = accel_correction_kernels(s, st);
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(st, &g);
    if (cst != DOMA_OK) {
      if (g) cudaGraphDestroy(g);
      return cst;
    }
    DOMA_CUDA_TRY(e);
    s->acc_graph = g;
    DOMA_CUDA_TRY(cudaGraphInstantiate(&s->acc_exec, g, 0));
    if (s->acc_gen != s->accel->work_gen) {   // the capture itself resized the workspace
      set_error("the U-Net workspace changed while its correction graph was captured");
      return DOMA_CUDA_ERROR;
    }
  }
  DOMA_CUDA_TRY(cudaGraphLaunch(s->acc_exec, st));
  return DOMA_OK;
}

doma_status accel_correction(doma_solver * s, cudaStream_t st)
{
  DOMA_TRY(accel_correction_launch(s, st));
  // a tensor-memory convolution whose bounded wait gave up leaves garbage in
  // the correction: report it instead of sweeping from it
  DOMA_CUDA_TRY(cudaStreamSynchronize(st));
  int conv_err = 0;
  DOMA_TRY(conv3_tc_error(&conv_err));
  if (conv_err) {
    set_error("a convolution's wait for its tensor-memory pipeline timed out");
    return DOMA_DEVICE_WAIT_TIMEOUT;
  }
  return accel_source(s->it, s->opts.precision, s->d_dscratch, s->d_corr, s->d_q, st);
}

// Host-driven multigroup loop.  After iteration `first` and then every
// `interval` iterations the network proposes a correction; the iteration
// that follows is swept from it, and with the guard on a correction after
// which the relative increment norm rose is undone (flux, increment and
// source restored; that sweep is spent).  With a reference flux the loop
// stops on the relative L2 error against it instead of the increment norm.
doma_status solve_multigroup_guided(doma_solver * s, doma_report * r)
{
  const auto t0 = std::chrono::steady_clock::now();
  const size_t G = s->G, N = s->N;
  const size_t bytes = G * N * sizeof(double);
  const doma_options & o = s->opts;
  cudaStream_t st = s->stream;
  DOMA_CUDA_TRY(cudaMemsetAsync(s->d_prev, 0, bytes, st));
  DOMA_CUDA_TRY(cudaMemsetAsync(&s->d_ctl->error, 0, sizeof(int), st));
  DOMA_CUDA_TRY(cudaMemsetAsync(s->d_ctl->norms, 0, sizeof(s->d_ctl->norms), st));
  DOMA_TRY(launch_mgi_init(s->it, o.precision, s->d_q, s->d_sigt, st));
  const bool use_ref = s->d_ref != nullptr;
  const doma_accel_options A = s->accel_opts;
  uint64_t launches = 1;
  unsigned iters = 0, tries = 0, next_try = std::max(1u, A.first);
  unsigned accepted = 0, rejected = 0;
  double res = 0.0, err = -1.0, res_before = 0.0, err_before = -1.0;
  bool pending = false;
  doma_status status = DOMA_OK;
  for (;;) {
    s->it.corr = pending ? s->d_corr : nullptr;
    const doma_status ist = mgi_iteration(s, LoopParams{}, st);
    s->it.corr = nullptr;
    DOMA_TRY(ist);
    launches += 2;
    if (use_ref) {
      DOMA_TRY(ref_error(s->it, s->d_ref, s->d_acc_partials, s->d_acc_ticket, &s->d_ctl->norms[2], st));
      ++launches;
    }
    double diff, tot;
    DOMA_TRY(read_norms(s, 0, &diff, &tot));
    const double e2 = s->h_ctl->norms[2];
    ++iters;
    if (!std::isfinite(diff) || !std::isfinite(tot) || !std::isfinite(e2)) {
      status = DOMA_NUMERIC_ERROR;
      break;
    }
    res = ratio(diff, tot);
    if (use_ref) err = std::sqrt(e2 / s->ref_norm2);
    if (pending) {
      pending = false;
      const bool reached = use_ref && err <= s->ref_target;
      if (!reached && A.guard && res > res_before) {
        DOMA_CUDA_TRY(cudaMemcpyAsync(s->d_phi, s->d_phi_save, bytes, cudaMemcpyDeviceToDevice, st));
        DOMA_CUDA_TRY(cudaMemcpyAsync(s->d_dscratch, s->d_delta_save, bytes,
                                      cudaMemcpyDeviceToDevice, st));
        DOMA_TRY(accel_source(s->it, o.precision, s->d_dscratch, nullptr, s->d_q, st));
        ++launches;
        ++rejected;
        res = res_before;
        err = err_before;
      } else {
        ++accepted;
      }
    }
    if (use_ref ? err <= s->ref_target : !(o.fs_tol < res)) break;
    if (iters >= o.fs_max_it) {
      status = DOMA_NOT_CONVERGED;
      break;
    }
    if (s->accel && tries < A.max_corrections && iters >= next_try) {
      DOMA_CUDA_TRY(cudaMemcpyAsync(s->d_phi_save, s->d_phi, bytes, cudaMemcpyDeviceToDevice, st));
      DOMA_CUDA_TRY(cudaMemcpyAsync(s->d_delta_save, s->d_dscratch, bytes,
                                    cudaMemcpyDeviceToDevice, st));
      DOMA_TRY(accel_correction(s, st));
      launches += 1 + 4 * G;
      pending = true;
      res_before = res;
      err_before = err;
      ++tries;
      next_try = iters + 1 + A.interval;
    }
  }
  DOMA_CUDA_TRY(cudaStreamSynchronize(st));
  if (status == DOMA_NOT_CONVERGED) set_error("the guided multigroup solve reached fs_max_it");
  else if (status == DOMA_NUMERIC_ERROR) set_error("a residual norm is not finite");
  s->launches += launches;
  const auto t1 = std::chrono::steady_clock::now();
  const double ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
  s->stats.iterations = iters;
  s->stats.corrections_accepted = accepted;
  s->stats.corrections_rejected = rejected;
  s->stats.error = err;
  s->stats.solve_ms = ms;
  if (o.verbose)
    std::printf("Guided multigroup iteration %s after %u iterations (%u corrections kept, %u undone), "
                "residual %g, error %g\n",
                status == DOMA_OK ? "converged" : "failed to converge", iters, accepted, rejected, res,
                err);
  if (r) {
    r->status = status;
    r->mg_iterations = iters;
    r->si_iterations = (uint64_t)iters * G;
    r->updates = (uint64_t)iters * G * N * (uint64_t)s->D;
    r->kernel_launches = launches;
    r->mg_residual = res;
    r->si_residual = res;
    r->solve_ms = ms;
    r->si_counts_len = 1;
    if (r->si_counts && r->si_counts_capacity) r->si_counts[0] = iters;
  }
  return status;
}

doma_status solve_impl(doma_solver * s, doma_report * r)
{
  if (s->mgi && (s->accel || s->d_ref)) return solve_multigroup_guided(s, r);
  if (s->mgi) return solve_multigroup(s, r);
  if (s->use_graph) return solve_graph(s, r);
  const size_t G = s->G, N = s->N;
  const auto t0 = std::chrono::steady_clock::now();
  const uint64_t launches0 = s->launches;
  if (s->opts.verbose) std::printf("Solving...\nInitializing the solver...\n");
  DOMA_CUDA_TRY(cudaMemsetAsync(s->d_phi, 0, G * N * sizeof(double), s->stream));
  DOMA_CUDA_TRY(cudaMemsetAsync(s->d_prev, 0, G * N * sizeof(double), s->stream));
  DOMA_CUDA_TRY(cudaMemsetAsync(&s->d_ctl->error, 0, sizeof(int), s->stream));
  Tally t;
  auto stage = [&](int g) {
    return launch_mg_source(s->it, g, s->opts.precision, s->d_q, s->d_sigt, LoopParams{},
                            s->stream);
  };
  const doma_status status = gs_host_loop(s, stage, r, t);
  if (!reportable(status)) return status;
  if (s->opts.verbose) std::fflush(stdout);
  DOMA_CUDA_TRY(cudaStreamSynchronize(s->stream));
  fill_report(s, r, status, t, t0, launches0);
  return status;
}

// Pinned host copies of the flux and the previous iterate (first use).
doma_status ensure_host_flux(doma_solver * s)
{
  const size_t bytes = (size_t)s->G * s->N * sizeof(double);
  if (!s->h_phi) DOMA_CUDA_TRY(cudaMallocHost(&s->h_phi, bytes));
  if (!s->h_prev) DOMA_CUDA_TRY(cudaMallocHost(&s->h_prev, bytes));
  return DOMA_OK;
}

// ---- k-eigenvalue power iteration ------------------------------------------

// updateEigenvalue (src/TransportSolver3D.cpp:432-456): num and den summed on
// the host over cells in order, groups inner, cells without production
// skipped -- DOMA's single-thread order, so k carries DOMA's bits.
doma_status k_update(doma_solver * s, double k, double * k_new)
{
  const size_t G = s->G, N = s->N, bytes = G * N * sizeof(double);
  DOMA_TRY(ensure_host_flux(s));
  DOMA_CUDA_TRY(cudaMemcpyAsync(s->h_phi, s->d_phi, bytes, cudaMemcpyDeviceToHost, s->stream));
  DOMA_CUDA_TRY(cudaMemcpyAsync(s->h_prev, s->d_prev, bytes, cudaMemcpyDeviceToHost, s->stream));
  DOMA_CUDA_TRY(cudaStreamSynchronize(s->stream));
  double num = 0.0, den = 0.0;
  for (size_t c = 0; c < N; ++c) {
    const uint32_t m = s->h_mat[c];
    if (!s->h_fis[m]) continue;
    const double V = s->h_vol[c];
    for (size_t g = 0; g < G; ++g) {
      const double nsf = s->h_nsf[(size_t)m * G + g];
      num = num + V * nsf * s->h_phi[g * N + c];
      den = den + V * nsf * s->h_prev[g * N + c] / k;
    }
  }
  *k_new = num / den;
  return DOMA_OK;
}

// solveEigenvalue (src/TransportSolver3D.cpp:29-86; 2D :31-88), host-driven:
// the group loop and source iterations are the fixed-source ones.
doma_status solve_eigen_impl(doma_solver * s, double k_tol, doma_report * r, double * k_out)
{
  if (s->mgi) return bad("eigenvalue solves use Gauss-Seidel iteration");
  if (!s->fissile) return bad("an eigenvalue solve needs a fissile material");
  const doma_options & o = s->opts;
  const int verbose = (int)o.verbose;
  const size_t N = s->N;
  const auto t0 = std::chrono::steady_clock::now();
  const uint64_t launches0 = s->launches;
  if (s->use_graph && !s->eg_exec) {
    if (!s->d_k) DOMA_TRY(dalloc(s, &s->d_k, 1));
    if (!s->h_k) DOMA_CUDA_TRY(cudaMallocHost(&s->h_k, sizeof(double)));
    DOMA_TRY(build_eigen_graph(s));
  }
  if (verbose) std::printf("Solving...\nInitializing the solver...\n");
  DOMA_TRY(launch_eigen_init(s->it, s->stream));
  ++s->launches;
  DOMA_CUDA_TRY(cudaMemsetAsync(s->d_q, 0, N * (o.precision == DOMA_PREC_FP64 ? 8 : 4), s->stream));
  DOMA_CUDA_TRY(cudaMemsetAsync(&s->d_ctl->error, 0, sizeof(int), s->stream));

  Tally t;
  double k = 1.0, k_prev = 0.0, shape = 0.0, kdiff = 0.0;
  doma_status status = DOMA_OK;
  do {
    if (verbose) {
      if (t.mg != 0u)
        std::printf("Performing PI %u, shape residual = %g, k residual = %g\nk = %g\n", t.mg,
                    shape, kdiff, k);
      else
        std::printf("Performing PI %u\n", t.mg);
      std::printf("----------------------------------------------------------------------------------\n");
    }
    if (s->use_graph) {
      // the group loop as one graph launch; k reaches it through device memory
      *s->h_k = k;
      DOMA_CUDA_TRY(cudaMemcpyAsync(s->d_k, s->h_k, sizeof(double), cudaMemcpyHostToDevice,
                                    s->stream));
      GraphRun run;
      DOMA_TRY(graph_run(s, s->eg_exec, run));
      if (verbose) {
        size_t pair = 0, hist = 0;
        print_si_pass(s, run, pair, hist);
      }
      if (run.c.failed) status = graph_status(s, run.c);   // solveEigenvalue returns false
      uint64_t per_sweep = s->sched.persistent ? 1 : 0;
      if (!s->sched.persistent)
        for (size_t L = 0; L + 1 < s->sched.level_begin.size(); ++L)
          per_sweep += s->sched.level_begin[L + 1] > s->sched.level_begin[L];
      s->launches += run.c.sweeps * (per_sweep + 1) + (uint64_t)s->G;
      t.sweeps += run.c.sweeps;
      t.si_res = run.c.si_res;
      if (r && r->si_counts)
        for (size_t q = 0; q < run.counts.size(); ++q)
          if (t.si_len + q < r->si_counts_capacity) r->si_counts[t.si_len + q] = run.counts[q];
      t.si_len += run.c.pairs;
    } else {
      for (int g = 0; g < s->G && status == DOMA_OK; ++g) {
        DOMA_TRY(launch_mg_source_eigen(s->it, g, o.precision, k, nullptr, s->d_q, s->d_sigt,
                                        LoopParams{}, s->stream));
        ++s->launches;
        status = group_source_iteration(s, g, r, t);  // a failed group: solveEigenvalue returns false
        if (!reportable(status)) return status;
      }
    }
    if (status != DOMA_OK) break;
    k_prev = k;
    DOMA_TRY(k_update(s, k, &k));
    DOMA_TRY(launch_mg_residual(s->it, s->d_ctl->norms + 2, LoopParams{}, s->stream));
    ++s->launches;
    double diff, tot;
    DOMA_TRY(read_norms(s, 2, &diff, &tot));
    if (!std::isfinite(diff) || !std::isfinite(tot) || !std::isfinite(k)) {
      set_error("power iteration norm or k is not finite");
      status = DOMA_NUMERIC_ERROR;
      break;
    }
    shape = ratio(diff, tot);
    kdiff = std::abs(k - k_prev);
    ++t.mg;
  } while (t.mg < o.mg_max_it && (o.mg_tol < shape || k_tol < kdiff));

  if (status == DOMA_OK) {
    if (t.mg < o.mg_max_it) {
      if (verbose)
        std::printf("PI converged after %u iterations with a flux shape residual of %g and a k "
                    "residual of %g.\nConverged value of k = %g\n", t.mg, shape, kdiff, k);
    } else {
      if (verbose)
        std::printf("PI failed to converge after %u iterations with a flux shape residual of %g "
                    "and a k residual of %g.\n", t.mg, shape, kdiff);
      status = DOMA_NOT_CONVERGED;
      set_error("power iteration reached mg_max_it");
    }
  } else if (status == DOMA_NOT_CONVERGED) {
    set_error("source iteration reached fs_max_it");
  }
  if (verbose) std::fflush(stdout);
  DOMA_CUDA_TRY(cudaStreamSynchronize(s->stream));
  if (k_out) *k_out = k;
  t.mg_res = shape;
  fill_report(s, r, status, t, t0, launches0);
  return status;
}

// ---- transient (zero initial condition) ------------------------------------

// The checks DOMA's deck reader makes on transient data
// (src/InputParameters.cpp:286-500), plus what its solver assumes: a material
// with delayed groups has production cross sections (stepDNPs reads them) and
// positive decay constants (it divides by them).
doma_status transient_validate(const doma_solver * s, const doma_transient * tr)
{
  if (!tr) return bad("transient data is null");
  if (!(tr->dt > 0.0) || !std::isfinite(tr->dt)) return bad("transient dt must be positive and finite");
  if (!tr->inv_v) return bad("transient inv_v is required");
  const size_t M = s->M, G = s->G, D = tr->num_d_groups;
  for (size_t i = 0; i < M * G; ++i)
    if (!std::isfinite(tr->inv_v[i])) return bad("transient inv_v must be finite");
  if (D > 0 && (!tr->d_groups || !tr->chi_d || !tr->beta || !tr->lambda))
    return bad("delayed groups need d_groups, chi_d, beta and lambda");
  if (tr->d_groups)
    for (size_t m = 0; m < M; ++m) {
      const uint32_t Dm = tr->d_groups[m];
      if (Dm > D)
        return bad("material " + std::to_string(m) + " has more delayed groups than num_d_groups");
      if (Dm > 0 && !s->h_fis[m])
        return bad("material " + std::to_string(m) + " has delayed groups but no fission data");
      for (uint32_t d = 0; d < Dm; ++d)
        if (!(tr->lambda[m * D + d] > 0.0) || !std::isfinite(tr->lambda[m * D + d]))
          return bad("material " + std::to_string(m) + ": decay constants must be positive");
    }
  if (tr->step_type) {
    if (!tr->step_insert || !tr->step_remove || !tr->step_source)
      return bad("source steps need step_insert, step_remove and step_source");
    for (size_t m = 0; m < M; ++m) {
      const uint32_t st = tr->step_type[m];
      if (st > DOMA_STEP_REMOVE)
        return bad("material " + std::to_string(m) + ": unknown source step type");
      if (st == DOMA_STEP_BOTH && tr->step_remove[m] < tr->step_insert[m])
        return bad("The step source for block " + std::to_string(m) + " is being removed at " +
                   std::to_string(tr->step_remove[m]) +
                   ", which is less than the insertion time of " +
                   std::to_string(tr->step_insert[m]) + "!");
    }
  }
  return DOMA_OK;
}

template <typename T>
doma_status talloc(doma_solver * s, T ** p, size_t count)
{
  void * v = nullptr;
  cudaError_t e = cudaMalloc(&v, std::max<size_t>(count, 1) * sizeof(T));
  if (e != cudaSuccess) {
    set_error(std::string("cudaMalloc: ") + cudaGetErrorString(e));
    return DOMA_CUDA_ERROR;
  }
  s->tr_allocs.push_back(v);
  *p = static_cast<T *>(v);
  return DOMA_OK;
}

// Device tables of a transient call, padded to the allocated delayed-group
// count (absent arrays upload as zeros, so the captured graph's arguments
// never change), the clock (t = 0, dt) and the zero initial condition
// (initZeroIC, src/TransportSolver3D.cpp:142-157).
doma_status transient_upload(doma_solver * s, const doma_transient * tr)
{
  const size_t M = s->M, G = s->G, N = s->N, D = tr->num_d_groups;
  DOMA_CUDA_TRY(cudaStreamSynchronize(s->stream));
  if (s->tr_allocs.empty() || D > (size_t)s->tr_D) {
    if (s->tr_exec) cudaGraphExecDestroy(s->tr_exec);
    if (s->tr_graph) cudaGraphDestroy(s->tr_graph);
    s->tr_exec = nullptr;
    s->tr_graph = nullptr;
    for (void * p : s->tr_allocs) cudaFree(p);
    s->tr_allocs.clear();
    if (s->h_dnps) cudaFreeHost(s->h_dnps);
    s->h_dnps = nullptr;
    const size_t Dc = std::max<size_t>(D, 1);
    TransientArgs & x = s->tr;
    x = TransientArgs{};
    x.D = (int)Dc;
    x.dims2 = s->dims == 2;
    double *clock, *inv_v, *chi_d, *beta, *lambda, *decay, *ins, *rem, *ssrc, *last, *dnps;
    uint32_t *dg, *stype;
    DOMA_TRY(talloc(s, &clock, 2));
    DOMA_TRY(talloc(s, &inv_v, M * G));
    DOMA_TRY(talloc(s, &dg, M));
    DOMA_TRY(talloc(s, &chi_d, M * G * Dc));
    DOMA_TRY(talloc(s, &beta, M * G * Dc));
    DOMA_TRY(talloc(s, &lambda, M * Dc));
    DOMA_TRY(talloc(s, &decay, M * Dc));
    DOMA_TRY(talloc(s, &stype, M));
    DOMA_TRY(talloc(s, &ins, M));
    DOMA_TRY(talloc(s, &rem, M));
    DOMA_TRY(talloc(s, &ssrc, M * G));
    DOMA_TRY(talloc(s, &last, G * N));
    DOMA_TRY(talloc(s, &dnps, Dc * N));
    DOMA_CUDA_TRY(cudaMallocHost(&s->h_dnps, Dc * N * sizeof(double)));
    x.clock = clock; x.inv_v = inv_v; x.dg = dg; x.chi_d = chi_d; x.beta = beta;
    x.lambda = lambda; x.decay = decay; x.step_type = stype; x.step_insert = ins;
    x.step_remove = rem; x.step_source = ssrc; x.last = last; x.dnps = dnps;
    s->tr_D = (int)Dc;
  }
  const size_t Dc = (size_t)s->tr_D;
  std::vector<uint32_t> dg(M, 0u), stype(M, 0u);
  std::vector<double> chi_d(M * G * Dc, 0.0), beta(M * G * Dc, 0.0), lambda(M * Dc, 0.0),
      decay(M * Dc, 0.0), ins(M, 0.0), rem(M, 0.0), ssrc(M * G, 0.0);
  if (tr->d_groups)
    for (size_t m = 0; m < M; ++m) {
      dg[m] = tr->d_groups[m];
      for (size_t d = 0; d < dg[m]; ++d) {
        for (size_t g = 0; g < G; ++g) {
          chi_d[(m * G + g) * Dc + d] = tr->chi_d[(m * G + g) * D + d];
          beta[(m * G + g) * Dc + d] = tr->beta[(m * G + g) * D + d];
        }
        const double lam = tr->lambda[m * D + d];
        lambda[m * Dc + d] = lam;
        decay[m * Dc + d] = std::exp(-lam * tr->dt);  // stepDNPs: std::exp(-lambda * dt)
      }
    }
  if (tr->step_type) {
    stype.assign(tr->step_type, tr->step_type + M);
    ins.assign(tr->step_insert, tr->step_insert + M);
    rem.assign(tr->step_remove, tr->step_remove + M);
    ssrc.assign(tr->step_source, tr->step_source + M * G);
  }
  const double clock[2] = {0.0, tr->dt};
  const TransientArgs & x = s->tr;
  DOMA_CUDA_TRY(cudaMemcpy(x.clock, clock, sizeof(clock), cudaMemcpyHostToDevice));
  DOMA_CUDA_TRY(cudaMemcpy((void *)x.inv_v, tr->inv_v, M * G * sizeof(double), cudaMemcpyHostToDevice));
  DOMA_CUDA_TRY(cudaMemcpy((void *)x.dg, dg.data(), M * sizeof(uint32_t), cudaMemcpyHostToDevice));
  DOMA_CUDA_TRY(cudaMemcpy((void *)x.chi_d, chi_d.data(), chi_d.size() * sizeof(double), cudaMemcpyHostToDevice));
  DOMA_CUDA_TRY(cudaMemcpy((void *)x.beta, beta.data(), beta.size() * sizeof(double), cudaMemcpyHostToDevice));
  DOMA_CUDA_TRY(cudaMemcpy((void *)x.lambda, lambda.data(), lambda.size() * sizeof(double), cudaMemcpyHostToDevice));
  DOMA_CUDA_TRY(cudaMemcpy((void *)x.decay, decay.data(), decay.size() * sizeof(double), cudaMemcpyHostToDevice));
  DOMA_CUDA_TRY(cudaMemcpy((void *)x.step_type, stype.data(), M * sizeof(uint32_t), cudaMemcpyHostToDevice));
  DOMA_CUDA_TRY(cudaMemcpy((void *)x.step_insert, ins.data(), M * sizeof(double), cudaMemcpyHostToDevice));
  DOMA_CUDA_TRY(cudaMemcpy((void *)x.step_remove, rem.data(), M * sizeof(double), cudaMemcpyHostToDevice));
  DOMA_CUDA_TRY(cudaMemcpy((void *)x.step_source, ssrc.data(), M * G * sizeof(double), cudaMemcpyHostToDevice));
  DOMA_CUDA_TRY(cudaMemsetAsync(x.last, 0, G * N * sizeof(double), s->stream));
  DOMA_CUDA_TRY(cudaMemsetAsync(x.dnps, 0, Dc * N * sizeof(double), s->stream));
  DOMA_CUDA_TRY(cudaMemsetAsync(s->d_phi, 0, G * N * sizeof(double), s->stream));
  DOMA_CUDA_TRY(cudaMemsetAsync(s->d_prev, 0, G * N * sizeof(double), s->stream));
  DOMA_CUDA_TRY(cudaMemsetAsync(&s->d_ctl->error, 0, sizeof(int), s->stream));
  return DOMA_OK;
}

// solveTransient with TransientIC::Zero (src/TransportSolver3D.cpp:88-140):
// per step the Gauss-Seidel solve with the transient source (one graph
// launch, or the host loop), stepDNPs, the callback, updateStepFluxes.
doma_status solve_transient_impl(doma_solver * s, const doma_transient * tr,
                                 doma_step_callback callback, void * user, doma_report * r)
{
  if (s->mgi) return bad("transient solves use Gauss-Seidel iteration");
  DOMA_TRY(transient_validate(s, tr));
  const int verbose = (int)s->opts.verbose;
  const size_t G = s->G, N = s->N, D = tr->num_d_groups;
  const auto t0 = std::chrono::steady_clock::now();
  const uint64_t launches0 = s->launches;
  DOMA_TRY(transient_upload(s, tr));
  if (s->use_graph && !s->tr_exec) DOMA_TRY(build_graph(s, true));
  if (callback) DOMA_TRY(ensure_host_flux(s));
  if (verbose) std::printf("Setting up initial conditions...\n");
  Tally t;
  doma_status status = DOMA_OK;
  double time = 0.0;
  for (uint32_t step = 0; step < tr->num_steps; ++step) {
    if (verbose) std::printf("Solving timestep %u...\n", step);
    if (s->use_graph) {
      GraphRun run;
      DOMA_TRY(graph_run(s, s->tr_exec, run));
      if (verbose) print_history(s, run, false);
      status = graph_status(s, run.c);
      s->launches += graph_launches(s, run.c);
      t.sweeps += run.c.sweeps;
      t.mg = run.c.mg_it;
      t.mg_res = run.c.mg_res;
      t.si_res = run.c.si_res;
      if (r && r->si_counts)
        for (size_t k = 0; k < run.counts.size(); ++k)
          if (t.si_len + k < r->si_counts_capacity) r->si_counts[t.si_len + k] = run.counts[k];
      t.si_len += run.c.pairs;
    } else {
      auto stage = [&](int g) {
        return launch_mg_source_transient(s->it, s->tr, g, s->opts.precision, s->d_q, s->d_sigt,
                                          LoopParams{}, s->stream);
      };
      status = gs_host_loop(s, stage, r, t);
      if (!reportable(status)) return status;
    }
    if (status != DOMA_OK) break;  // solveTransient returns false at once
    DOMA_TRY(launch_step_dnps(s->it, s->tr, s->stream));
    ++s->launches;
    if (callback) {
      DOMA_CUDA_TRY(cudaMemcpyAsync(s->h_phi, s->d_phi, G * N * sizeof(double),
                                    cudaMemcpyDeviceToHost, s->stream));
      if (D)
        DOMA_CUDA_TRY(cudaMemcpyAsync(s->h_dnps, s->tr.dnps, D * N * sizeof(double),
                                      cudaMemcpyDeviceToHost, s->stream));
      DOMA_CUDA_TRY(cudaStreamSynchronize(s->stream));
      if (verbose) std::fflush(stdout);
      if (callback(user, step, time, s->h_phi, D ? s->h_dnps : nullptr) != 0) {
        status = bad("the step callback stopped the transient after step " + std::to_string(step));
        break;
      }
    }
    if (step + 1 != tr->num_steps) {
      DOMA_TRY(launch_step_rollover(s->it, s->tr, s->stream));
      ++s->launches;
    }
    time += tr->dt;
  }
  if (verbose) std::fflush(stdout);
  DOMA_CUDA_TRY(cudaStreamSynchronize(s->stream));
  fill_report(s, r, status, t, t0, launches0);
  return status;
}

}  // namespace

extern "C" {

void doma_default_options(doma_options * o)
{
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->scheme = DOMA_SCHEME_DD;
  o->theta = 0.9;
  o->precision = DOMA_PREC_FP64;
  o->fs_tol = 1e-8;
  o->fs_max_it = 1000;
  o->mg_tol = 1e-8;
  o->mg_max_it = 100;
}

const char * doma_last_error(void) { return get_error(); }

uint32_t doma_abi_version(void) { return DOMA_ABI_VERSION; }

doma_status doma_quadrature(uint32_t np, uint32_t na, uint32_t dims, double * mu, double * eta,
                            double * xi, double * w, uint32_t counts[8])
{
  if (!mu || !eta || !xi || !w || !counts) return bad("null output pointer");
  unsigned c[8];
  const int n = gc_quadrature(np, na, dims, mu, eta, xi, w, c);
  if (n < 0) return bad("invalid quadrature order");
  for (int o = 0; o < 8; ++o) counts[o] = c[o];
  return DOMA_OK;
}

doma_status doma_solver_create(const doma_problem * problem, const doma_options * opts,
                               doma_solver ** out)
{
  if (!out) return bad("null output handle");
  *out = nullptr;
  doma_status st = validate(problem, opts);
  if (st != DOMA_OK) return st;
  doma_solver * s = new (std::nothrow) doma_solver();
  if (!s) return bad("out of host memory");
  st = create_impl(problem, opts, s);
  if (st != DOMA_OK) {
    release(s);
    return st;
  }
  *out = s;
  return DOMA_OK;
}

doma_status doma_solver_set_stream(doma_solver * s, void * stream)
{
  if (!s) return bad("null solver");
  s->stream = stream ? static_cast<cudaStream_t>(stream) : s->own_stream;
  return DOMA_OK;
}

doma_status doma_solver_solve_fixed_source(doma_solver * s, doma_report * report)
{
  if (!s) return bad("null solver");
  return solve_impl(s, report);
}

doma_status doma_solver_solve_eigenvalue(doma_solver * s, double k_tol, doma_report * report,
                                         double * k)
{
  if (!s) return bad("null solver");
  if (!(k_tol >= 0.0)) return bad("k_tol must be >= 0");
  return solve_eigen_impl(s, k_tol, report, k);
}

doma_status doma_solver_solve_transient(doma_solver * s, const doma_transient * tr,
                                        doma_step_callback callback, void * user,
                                        doma_report * report)
{
  if (!s) return bad("null solver");
  return solve_transient_impl(s, tr, callback, user, report);
}

doma_status doma_solver_get_scalar_flux(doma_solver * s, double * out, size_t count)
{
  if (!s || !out) return bad("null solver or output");
  if (count < (size_t)s->G * s->N) return bad("output buffer too small");
  DOMA_CUDA_TRY(cudaMemcpyAsync(out, s->d_phi, (size_t)s->G * s->N * sizeof(double),
                                cudaMemcpyDeviceToHost, s->stream));
  DOMA_CUDA_TRY(cudaStreamSynchronize(s->stream));
  return DOMA_OK;
}

doma_status doma_solver_source_iterations(doma_solver * s, uint32_t group, uint32_t count)
{
  if (!s) return bad("null solver");
  if ((int)group >= s->G) return bad("group out of range");
  if (s->mgi) {
    // multigroup mode: `count` iterations of all groups from the external source
    DOMA_TRY(launch_mgi_init(s->it, s->opts.precision, s->d_q, s->d_sigt, s->stream));
    ++s->launches;
    for (uint32_t i = 0; i < count; ++i) DOMA_TRY(mgi_iteration(s, LoopParams{}, s->stream));
    return DOMA_OK;
  }
  DOMA_TRY(launch_mg_source(s->it, (int)group, s->opts.precision, s->d_q, s->d_sigt, LoopParams{},
                            s->stream));
  ++s->launches;
  for (uint32_t i = 0; i < count; ++i) DOMA_TRY(source_iteration(s, (int)group));
  return DOMA_OK;
}

doma_status doma_solver_sweeps(doma_solver * s, uint32_t group, uint32_t count)
{
  if (!s) return bad("null solver");
  if ((int)group >= s->G) return bad("group out of range");
  for (uint32_t i = 0; i < count; ++i) DOMA_TRY(sweep_once(s));
  return DOMA_OK;
}

doma_status doma_solver_describe(const doma_solver * s, uint32_t tile[3],
                                 uint32_t * launches_per_sweep, uint64_t * kernel_launches)
{
  if (!s) return bad("null solver");
  if (tile) {
    tile[0] = (uint32_t)s->sched.tx;
    tile[1] = (uint32_t)s->sched.ty;
    tile[2] = (uint32_t)s->sched.tz;
  }
  if (launches_per_sweep) {
    uint32_t n = 0;
    if (s->sched.persistent) {
      n = 1;
    } else {
      for (size_t L = 0; L + 1 < s->sched.level_begin.size(); ++L)
        if (s->sched.level_begin[L + 1] > s->sched.level_begin[L]) ++n;
    }
    *launches_per_sweep = n;
  }
  if (kernel_launches) *kernel_launches = s->launches;
  return DOMA_OK;
}

doma_status doma_solver_set_accelerator(doma_solver * s, doma_unet * net,
                                        const doma_accel_options * opts)
{
  if (!s) return bad("null solver");
  // a correction graph captured over the previous net is dropped (a new net
  // may even reuse the old one's address)
  if (s->acc_exec) cudaGraphExecDestroy(s->acc_exec);
  if (s->acc_graph) cudaGraphDestroy(s->acc_graph);
  s->acc_exec = nullptr;
  s->acc_graph = nullptr;
  s->acc_net = nullptr;
  s->acc_warm = false;
  if (!net) {
    s->accel = nullptr;
    return DOMA_OK;
  }
  if (!opts) return bad("null accelerator options");
  if (!s->mgi) return bad("the accelerator works in multigroup iteration (DOMA_ITER_MULTIGROUP)");
  if (s->dims != 3 || s->nx % 8 || s->ny % 8 || s->nz % 8)
    return bad("the accelerator needs a 3D mesh with extents that are multiples of 8");
  if (s->opts.scheme != DOMA_SCHEME_DD)
    return bad("the accelerator needs the linear diamond-difference scheme (DOMA_SCHEME_DD)");
  const size_t G = s->G, N = s->N;
  if (!s->d_fsig) {
    DOMA_TRY(dalloc(s, &s->d_fsig, G * N));
    DOMA_TRY(dalloc(s, &s->d_fabs, G * N));
    DOMA_TRY(dalloc(s, &s->d_kappa, G * N));
    DOMA_TRY(dalloc(s, &s->d_corr, G * N));
    DOMA_TRY(dalloc(s, &s->d_r, N));
    DOMA_TRY(dalloc(s, &s->d_ya, N));
    DOMA_TRY(dalloc(s, &s->d_yb, N));
    DOMA_TRY(dalloc(s, &s->d_nn_out, N));
    uint16_t * in = nullptr;
    DOMA_TRY(dalloc(s, &in, N * 16));
    s->d_nn_in = in;
    DOMA_TRY(dalloc(s, &s->d_rms, G));
    DOMA_TRY(dalloc(s, &s->d_phi_save, G * N));
    DOMA_TRY(dalloc(s, &s->d_delta_save, G * N));
  }
  if (!s->d_acc_partials) {
    DOMA_TRY(dalloc(s, &s->d_acc_partials, (size_t)s->it.grid));
    DOMA_TRY(dalloc(s, &s->d_acc_ticket, 1));
    DOMA_CUDA_TRY(cudaMemset(s->d_acc_ticket, 0, sizeof(unsigned)));
  }
  DOMA_TRY(accel_features(s->it, s->d_fsig, s->d_fabs, s->d_kappa, s->stream));
  DOMA_CUDA_TRY(cudaStreamSynchronize(s->stream));
  s->accel = net;
  s->accel_opts = *opts;
  return DOMA_OK;
}

doma_status doma_solver_set_reference(doma_solver * s, const double * phi_ref, size_t count,
                                      double target_error)
{
  if (!s) return bad("null solver");
  if (!phi_ref) {
    s->d_ref = nullptr;
    return DOMA_OK;
  }
  if (!s->mgi) return bad("the reference stop works in multigroup iteration (DOMA_ITER_MULTIGROUP)");
  const size_t n = (size_t)s->G * s->N;
  if (count != n) return bad("reference flux must hold num_groups * num_cells values");
  if (!(target_error > 0.0)) return bad("target error must be positive");
  double norm2 = 0.0;
  for (size_t i = 0; i < n; ++i) norm2 += phi_ref[i] * phi_ref[i];
  if (!(norm2 > 0.0) || !std::isfinite(norm2)) return bad("reference flux is zero or not finite");
  if (!s->d_acc_partials) {
    DOMA_TRY(dalloc(s, &s->d_acc_partials, (size_t)s->it.grid));
    DOMA_TRY(dalloc(s, &s->d_acc_ticket, 1));
    DOMA_CUDA_TRY(cudaMemset(s->d_acc_ticket, 0, sizeof(unsigned)));
  }
  double * ref = nullptr;
  DOMA_TRY(upload(s, &ref, phi_ref, n));
  s->d_ref = ref;
  s->ref_norm2 = norm2;
  s->ref_target = target_error;
  return DOMA_OK;
}

doma_status doma_solver_accel_stats(const doma_solver * s, doma_accel_stats * out)
{
  if (!s || !out) return bad("null solver or output");
  *out = s->stats;
  return DOMA_OK;
}

void doma_solver_destroy(doma_solver * s) { release(s); }

}  // extern "C"


// ============================================================================
// Batched solve (C ABI doma_batch_*): many independent problems share one
// persistent sweep launch per iteration.
// ============================================================================

namespace {

struct BatchCtl {
  unsigned ticket, exit_count, epoch;
  int error;
  unsigned still_active;  // problems still iterating after this iteration
  unsigned iters;         // batched iterations run (graph loop)
};

}  // namespace

struct doma_batch {
  std::vector<doma_solver *> solvers;
  doma_options opts{};
  int dims = 3;
  int tx = 8, threads = kMaxSweepThreads, grid = 0;
  size_t smem = 0;
  int num_tasks = 0, epi_blocks = 0;
  SweepArgs<float> * d_args = nullptr;
  BatchTask * d_tasks = nullptr;
  BatchSlot * d_slots = nullptr;
  int * d_block_prob = nullptr;
  BatchLoop * d_loops = nullptr;
  BatchCtl * d_ctl = nullptr;
  BatchCtl * h_ctl = nullptr;
  cudaStream_t stream = nullptr, own_stream = nullptr;
  bool use_graph = true;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  unsigned iters = 0;   // batched iterations since doma_batch_begin
  // the last doma_batch_tune: ms of two batched sweeps per uniform block
  // length (8, 16, 32) and with the per-class lengths; number of classes
  float tune_uniform_ms[3] = {0.f, 0.f, 0.f};
  float tune_mixed_ms = 0.f;
  unsigned tune_classes = 0;
  std::chrono::steady_clock::time_point t_begin{};
  std::vector<void *> allocs;
};

namespace {

template <typename T>
doma_status balloc(doma_batch * b, T ** p, size_t count)
{
  void * v = nullptr;
  DOMA_CUDA_TRY(cudaMalloc(&v, std::max<size_t>(1, count) * sizeof(T)));
  b->allocs.push_back(v);
  *p = static_cast<T *>(v);
  return DOMA_OK;
}

void bfree(doma_batch * b, void * p)
{
  if (!p) return;
  for (auto it = b->allocs.begin(); it != b->allocs.end(); ++it)
    if (*it == p) {
      b->allocs.erase(it);
      break;
    }
  cudaFree(p);
}

void drop_batch_graph(doma_batch * b)
{
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->exec = nullptr;
  b->graph = nullptr;
}

void sfree(doma_solver * s, void * p)
{
  if (!p) return;
  for (auto it = s->allocations.begin(); it != s->allocations.end(); ++it)
    if (*it == p) {
      s->allocations.erase(it);
      break;
    }
  cudaFree(p);
}

// Rebuild one solver's sweep schedule for block length tx (fresh task list
// and done flags; its single-problem launches follow the new shape too).
doma_status reschedule(doma_solver * s, int tx)
{
  s->opts.tile_x = (uint32_t)tx;
  pick_tile(s, &s->opts);
  build_schedule(s);
  DOMA_TRY(sweep_prepare(s->dims, s->opts.precision, s->opts.scheme, s->sched.tx, s->sched.smem,
                         s->sched.many));
  sfree(s, s->d_tasks);
  sfree(s, s->d_done);
  DOMA_TRY(upload(s, &s->d_tasks, s->sched.tasks.data(), s->sched.tasks.size()));
  const size_t flags = (size_t)s->gif * 8 * s->sched.ngroups * s->sched.nbx * s->sched.nby * s->sched.nbz;
  DOMA_TRY(dalloc(s, &s->d_done, flags));
  DOMA_CUDA_TRY(cudaMemset(s->d_done, 0, flags * sizeof(unsigned)));
  const int fit = sweep_resident_ctas(s->dims, s->opts.precision, s->opts.scheme, s->sched.tx,
                                      s->sched.threads, s->sched.smem, s->sched.many);
  s->sched.grid = std::max(1, std::min<int>(fit, (int)s->sched.tasks.size()));
  for (auto * a : {&s->a32}) {
    a->nbx = s->sched.nbx; a->nby = s->sched.nby; a->nbz = s->sched.nbz;
    a->tx = s->sched.tx;
    a->num_tasks = (int)s->sched.tasks.size();
    a->tasks = s->d_tasks;
    a->done = s->d_done;
  }
  return DOMA_OK;
}

// The batch's merged task list, sweep arguments and epilogue layout for the
// current block length.
doma_status build_batch_schedule(doma_batch * b)
{
  const size_t P = b->solvers.size();
  b->smem = sweep_batch_smem_bytes(b->dims, (int)b->opts.scheme);
  b->threads = sweep_threads(ordinate_group(DOMA_PREC_FP32, (int)b->opts.scheme));
  std::vector<BatchTask> tasks;
  int max_levels = 0;
  for (auto * s : b->solvers) max_levels = std::max(max_levels, (int)s->sched.level_begin.size() - 1);
  for (int L = 0; L < max_levels; ++L)
    for (size_t p = 0; p < P; ++p) {
      const Schedule & sc = b->solvers[p]->sched;
      if (L + 1 >= (int)sc.level_begin.size()) continue;
      for (int t = sc.level_begin[L]; t < sc.level_begin[L + 1]; ++t)
        tasks.push_back(BatchTask{sc.tasks[t], (int)p});
    }
  b->num_tasks = (int)tasks.size();
  drop_batch_graph(b);
  bfree(b, b->d_tasks);
  DOMA_TRY(balloc(b, &b->d_tasks, tasks.size()));
  DOMA_CUDA_TRY(cudaMemcpy(b->d_tasks, tasks.data(), tasks.size() * sizeof(BatchTask),
                           cudaMemcpyHostToDevice));
  std::vector<SweepArgs<float>> args(P);
  for (size_t p = 0; p < P; ++p) {
    args[p] = b->solvers[p]->a32;
    args[p].error = &b->d_ctl->error;
    args[p].spin_limit = 1u << 22;
    args[p].wait_bias = 0u;
  }
  DOMA_CUDA_TRY(cudaMemcpy(b->d_args, args.data(), P * sizeof(SweepArgs<float>),
                           cudaMemcpyHostToDevice));
  const int fit = sweep_batch_resident_ctas(b->dims, b->opts.scheme, b->threads, b->smem);
  if (fit <= 0) return bad("the batched sweep block does not fit on this device");
  b->grid = std::max(1, std::min(fit, b->num_tasks));
  return DOMA_OK;
}

doma_status batch_sweep(doma_batch * b)
{
  return launch_sweep_batch(b->dims, b->opts.scheme, b->grid, b->threads, b->smem, b->d_args,
                            b->d_tasks, b->num_tasks, &b->d_ctl->ticket, &b->d_ctl->exit_count,
                            &b->d_ctl->epoch, b->d_loops, b->stream);
}

doma_status batch_init_sources(doma_batch * b)
{
  for (auto * s : b->solvers)
    DOMA_TRY(launch_mgi_init(s->it, DOMA_PREC_FP32, s->d_q, s->d_sigt, b->stream));
  std::vector<BatchLoop> loops(b->solvers.size(), BatchLoop{1u, 0u, 0u, 0u, 0.0});
  DOMA_CUDA_TRY(cudaMemcpyAsync(b->d_loops, loops.data(), loops.size() * sizeof(BatchLoop),
                                cudaMemcpyHostToDevice, b->stream));
  DOMA_CUDA_TRY(cudaMemsetAsync(&b->d_ctl->error, 0, sizeof(int), b->stream));
  return DOMA_OK;
}

// One batched iteration: the all-problem sweep, every active problem's
// epilogue, the per-problem loop test.
doma_status batch_iteration(doma_batch * b, cudaStream_t st)
{
  const size_t P = b->solvers.size();
  DOMA_TRY(launch_sweep_batch(b->dims, b->opts.scheme, b->grid, b->threads, b->smem,
                              b->d_args, b->d_tasks, b->num_tasks, &b->d_ctl->ticket,
                              &b->d_ctl->exit_count, &b->d_ctl->epoch, b->d_loops, st));
  DOMA_TRY(launch_batch_epilogue(b->d_slots, b->d_block_prob, b->epi_blocks, b->d_loops,
                                 DOMA_PREC_FP32, st));
  DOMA_TRY(launch_batch_finalize(b->d_slots, b->d_loops, (int)P, b->opts.fs_tol,
                                 b->opts.fs_max_it, &b->d_ctl->still_active, st));
  return DOMA_OK;
}

// The whole batched solve as one graph: WHILE(any active) { iteration ;
// continue }.  Rebuilt whenever the schedule changes (tuning).
doma_status build_batch_graph(doma_batch * b)
{
  drop_batch_graph(b);
  cudaStream_t c0 = nullptr, c1 = nullptr;
  DOMA_CUDA_TRY(cudaStreamCreateWithFlags(&c0, cudaStreamNonBlocking));
  DOMA_CUDA_TRY(cudaStreamCreateWithFlags(&c1, cudaStreamNonBlocking));
  auto run = [&]() -> doma_status {
    DOMA_CUDA_TRY(cudaGraphCreate(&b->graph, 0));
    cudaGraphConditionalHandle h;
    DOMA_CUDA_TRY(cudaGraphConditionalHandleCreate(&h, b->graph, 1u, cudaGraphCondAssignDefault));
    DOMA_CUDA_TRY(cudaStreamBeginCaptureToGraph(c0, b->graph, nullptr, nullptr, 0,
                                                cudaStreamCaptureModeThreadLocal));
    cudaGraph_t body = nullptr;
    doma_status st = add_while(c0, h, &body);
    if (st == DOMA_OK) {
      DOMA_CUDA_TRY(cudaStreamBeginCaptureToGraph(c1, body, nullptr, nullptr, 0,
                                                  cudaStreamCaptureModeThreadLocal));
      st = batch_iteration(b, c1);
      if (st == DOMA_OK)
        st = launch_batch_continue(&b->d_ctl->still_active, &b->d_ctl->error, &b->d_ctl->iters,
                                   b->opts.fs_max_it + 1u, (unsigned long long)h, c1);
      cudaGraph_t out = nullptr;
      DOMA_CUDA_TRY(cudaStreamEndCapture(c1, &out));
    }
    cudaGraph_t out = nullptr;
    DOMA_CUDA_TRY(cudaStreamEndCapture(c0, &out));
    if (st != DOMA_OK) return st;
    DOMA_CUDA_TRY(cudaGraphInstantiate(&b->exec, b->graph, 0));
    return DOMA_OK;
  };
  const doma_status st = run();
  cudaStreamDestroy(c0);
  cudaStreamDestroy(c1);
  if (st != DOMA_OK) drop_batch_graph(b);
  return st;
}

void batch_release(doma_batch * b)
{
  if (!b) return;
  drop_batch_graph(b);
  for (auto * s : b->solvers) release(s);
  for (void * p : b->allocs) cudaFree(p);
  if (b->h_ctl) cudaFreeHost(b->h_ctl);
  if (b->own_stream) cudaStreamDestroy(b->own_stream);
  delete b;
}

}  // namespace

extern "C" {

doma_status doma_batch_create(const doma_problem * problems, size_t count, const doma_options * opts,
                              doma_batch ** out)
{
  if (!out) return bad("null output handle");
  *out = nullptr;
  if (!problems || !opts || count == 0) return bad("empty batch");
  if (opts->precision != DOMA_PREC_FP32) return bad("batched solves sweep in FP32 (DOMA_PREC_FP32)");
  doma_batch * b = new (std::nothrow) doma_batch();
  if (!b) return bad("out of host memory");
  b->opts = *opts;
  b->opts.iteration = DOMA_ITER_MULTIGROUP;
  b->dims = (int)problems[0].num_dims;
  b->tx = sweep_tile_x(opts->tile_x ? (int)opts->tile_x
                                    : (b->dims == 3 ? (opts->scheme == DOMA_SCHEME_TW_DD ? 16 : 8) : 32));
  b->opts.tile_x = (uint32_t)b->tx;
  auto fail = [&](doma_status st) {
    batch_release(b);
    return st;
  };
  for (size_t i = 0; i < count; ++i) {
    if (problems[i].num_dims != (uint32_t)b->dims) return fail(bad("all problems of a batch share num_dims"));
    doma_solver * s = nullptr;
    const doma_status st = doma_solver_create(&problems[i], &b->opts, &s);
    if (st != DOMA_OK) {
      set_error("problem " + std::to_string(i) + ": " + get_error());
      return fail(st);
    }
    b->solvers.push_back(s);
  }
  const size_t P = count;
  doma_status st = DOMA_OK;
  if ((st = balloc(b, &b->d_args, P)) != DOMA_OK) return fail(st);
  if ((st = balloc(b, &b->d_slots, P)) != DOMA_OK) return fail(st);
  if ((st = balloc(b, &b->d_loops, P)) != DOMA_OK) return fail(st);
  if ((st = balloc(b, &b->d_ctl, 1)) != DOMA_OK) return fail(st);
  if (cudaMemset(b->d_ctl, 0, sizeof(BatchCtl)) != cudaSuccess) return fail(DOMA_CUDA_ERROR);
  if (cudaMallocHost(&b->h_ctl, sizeof(BatchCtl)) != cudaSuccess) return fail(DOMA_CUDA_ERROR);
  if (cudaStreamCreateWithFlags(&b->own_stream, cudaStreamNonBlocking) != cudaSuccess)
    return fail(DOMA_CUDA_ERROR);
  b->stream = b->own_stream;
  {
    const char * env = std::getenv("DOMA_SOLVE_LOOP");
    b->use_graph = !(env && std::string(env) == "host");
  }
  // batched epilogue layout: up to 64 blocks per problem, contiguous
  std::vector<BatchSlot> slots(P);
  std::vector<int> block_prob;
  for (size_t p = 0; p < P; ++p) {
    doma_solver * s = b->solvers[p];
    slots[p].it = s->it;
    slots[p].q = s->d_q;
    slots[p].dscratch = s->d_dscratch;
    slots[p].block0 = (int)block_prob.size();
    slots[p].blocks = std::max(1, std::min(s->it.grid, 64));
    block_prob.insert(block_prob.end(), slots[p].blocks, (int)p);
  }
  b->epi_blocks = (int)block_prob.size();
  if ((st = balloc(b, &b->d_block_prob, block_prob.size())) != DOMA_OK) return fail(st);
  if (cudaMemcpy(b->d_slots, slots.data(), P * sizeof(BatchSlot), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(b->d_block_prob, block_prob.data(), block_prob.size() * sizeof(int),
                 cudaMemcpyHostToDevice) != cudaSuccess)
    return fail(DOMA_CUDA_ERROR);
  if ((st = build_batch_schedule(b)) != DOMA_OK) return fail(st);
  *out = b;
  return DOMA_OK;
}

doma_status doma_batch_set_stream(doma_batch * b, void * stream)
{
  if (!b) return bad("null batch");
  b->stream = stream ? static_cast<cudaStream_t>(stream) : b->own_stream;
  return DOMA_OK;
}

// The batch's autotuner: a block length per class of problems.  A class is
// (16-cell bucket of the longest mesh axis, ordinates per octant, groups).
// For each length in {8, 16, 32} every solver is rescheduled to it and the
// batched sweep is timed over all problems (the uniform choice) and over each
// class alone (a task list of that class's problems only); each class takes
// its fastest length.  The mixed assignment is then timed against the best
// uniform length and kept only if it is faster.  The results do not depend
// on the choice (every block length gives the same bits).
doma_status doma_batch_tune(doma_batch * b, uint32_t * tile_x)
{
  if (!b) return bad("null batch");
  const size_t P = b->solvers.size();
  std::map<std::tuple<int, int, int>, std::vector<size_t>> classes;
  for (size_t p = 0; p < P; ++p) {
    const doma_solver * s = b->solvers[p];
    const int n = (int)std::max(s->nx, std::max(s->ny, s->nz));
    classes[std::make_tuple((n + 15) / 16, s->d_oct, s->G)].push_back(p);
  }
  const int txs[3] = {8, 16, 32};
  std::vector<std::array<float, 3>> class_ms(classes.size());
  float uniform_ms[3] = {0.f, 0.f, 0.f};
  cudaEvent_t e0, e1;
  DOMA_CUDA_TRY(cudaEventCreate(&e0));
  DOMA_CUDA_TRY(cudaEventCreate(&e1));
  // one warm-up sweep, then two timed
  auto time_list = [&](const BatchTask * tasks, int count, int grid, float * ms) -> doma_status {
    auto one = [&]() {
      return launch_sweep_batch(b->dims, b->opts.scheme, grid, b->threads, b->smem, b->d_args, tasks,
                                count, &b->d_ctl->ticket, &b->d_ctl->exit_count, &b->d_ctl->epoch,
                                b->d_loops, b->stream);
    };
    DOMA_TRY(one());
    DOMA_CUDA_TRY(cudaEventRecord(e0, b->stream));
    for (int k = 0; k < 2; ++k) DOMA_TRY(one());
    DOMA_CUDA_TRY(cudaEventRecord(e1, b->stream));
    DOMA_CUDA_TRY(cudaEventSynchronize(e1));
    DOMA_CUDA_TRY(cudaEventElapsedTime(ms, e0, e1));
    return DOMA_OK;
  };
  auto apply = [&](const std::vector<int> & per_problem) -> doma_status {
    for (size_t p = 0; p < P; ++p) DOMA_TRY(reschedule(b->solvers[p], per_problem[p]));
    DOMA_TRY(build_batch_schedule(b));
    return batch_init_sources(b);
  };
  // a class's own tasks, merged level by level as build_batch_schedule merges them
  BatchTask * d_class_tasks = nullptr;
  std::vector<BatchTask> tasks;
  const int fit = sweep_batch_resident_ctas(b->dims, b->opts.scheme, b->threads, b->smem);
  if (fit <= 0) return bad("the batched sweep block does not fit on this device");
  for (int k = 0; k < 3; ++k) {
    DOMA_TRY(apply(std::vector<int>(P, txs[k])));
    DOMA_TRY(time_list(b->d_tasks, b->num_tasks, b->grid, &uniform_ms[k]));
    if (!d_class_tasks) DOMA_TRY(balloc(b, &d_class_tasks, (size_t)b->num_tasks * 4));
    size_t c = 0;
    for (auto & kv : classes) {
      tasks.clear();
      int levels = 0;
      for (size_t p : kv.second)
        levels = std::max(levels, (int)b->solvers[p]->sched.level_begin.size() - 1);
      for (int L = 0; L < levels; ++L)
        for (size_t p : kv.second) {
          const Schedule & sc = b->solvers[p]->sched;
          if (L + 1 >= (int)sc.level_begin.size()) continue;
          for (int t = sc.level_begin[L]; t < sc.level_begin[L + 1]; ++t)
            tasks.push_back(BatchTask{sc.tasks[t], (int)p});
        }
      DOMA_CUDA_TRY(cudaMemcpyAsync(d_class_tasks, tasks.data(), tasks.size() * sizeof(BatchTask),
                                    cudaMemcpyHostToDevice, b->stream));
      DOMA_TRY(time_list(d_class_tasks, (int)tasks.size(), std::min(fit, (int)tasks.size()),
                         &class_ms[c][k]));
      ++c;
    }
  }
  DOMA_CUDA_TRY(cudaStreamSynchronize(b->stream));
  bfree(b, d_class_tasks);
  int best_uniform = 0;
  for (int k = 1; k < 3; ++k)
    if (uniform_ms[k] < uniform_ms[best_uniform]) best_uniform = k;
  std::vector<int> mixed(P, txs[best_uniform]);
  {
    size_t c = 0;
    for (auto & kv : classes) {
      int bk = 0;
      for (int k = 1; k < 3; ++k)
        if (class_ms[c][k] < class_ms[c][bk]) bk = k;
      for (size_t p : kv.second) mixed[p] = txs[bk];
      ++c;
    }
  }
  DOMA_TRY(apply(mixed));
  float mixed_ms = 0.f;
  DOMA_TRY(time_list(b->d_tasks, b->num_tasks, b->grid, &mixed_ms));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (!(mixed_ms < uniform_ms[best_uniform])) {
    mixed.assign(P, txs[best_uniform]);
    DOMA_TRY(apply(mixed));
  }
  // the most common length (by problem count) stands for the batch
  int count[3] = {0, 0, 0};
  for (int tx : mixed) ++count[tx == 8 ? 0 : tx == 16 ? 1 : 2];
  int most = 0;
  for (int k = 1; k < 3; ++k)
    if (count[k] > count[most]) most = k;
  b->tx = txs[most];
  b->tune_uniform_ms[0] = uniform_ms[0];
  b->tune_uniform_ms[1] = uniform_ms[1];
  b->tune_uniform_ms[2] = uniform_ms[2];
  b->tune_mixed_ms = mixed_ms;
  b->tune_classes = (unsigned)classes.size();
  if (tile_x) *tile_x = (uint32_t)b->tx;
  return DOMA_OK;
}

doma_status doma_batch_tiles(doma_batch * b, uint32_t * tiles, size_t count)
{
  if (!b || !tiles) return bad("null batch or buffer");
  if (count < b->solvers.size()) return bad("tiles buffer shorter than the batch");
  for (size_t p = 0; p < b->solvers.size(); ++p) tiles[p] = (uint32_t)b->solvers[p]->sched.tx;
  return DOMA_OK;
}

doma_status doma_batch_tune_report(doma_batch * b, float * uniform_ms, float * mixed_ms,
                                   uint32_t * classes)
{
  if (!b) return bad("null batch");
  if (uniform_ms)
    for (int k = 0; k < 3; ++k) uniform_ms[k] = b->tune_uniform_ms[k];
  if (mixed_ms) *mixed_ms = b->tune_mixed_ms;
  if (classes) *classes = b->tune_classes;
  return DOMA_OK;
}

doma_status doma_batch_begin(doma_batch * b)
{
  if (!b) return bad("null batch");
  DOMA_TRY(batch_init_sources(b));
  DOMA_CUDA_TRY(cudaMemsetAsync(&b->d_ctl->still_active, 0, 2 * sizeof(unsigned), b->stream));
  b->iters = 0;
  b->t_begin = std::chrono::steady_clock::now();
  return DOMA_OK;
}

doma_status doma_batch_iterate(doma_batch * b, uint32_t iterations, uint32_t * active)
{
  if (!b) return bad("null batch");
  unsigned still = 1;
  for (uint32_t k = 0; k < iterations; ++k) {
    DOMA_TRY(batch_iteration(b, b->stream));
    DOMA_CUDA_TRY(cudaMemcpyAsync(b->h_ctl, b->d_ctl, sizeof(BatchCtl), cudaMemcpyDeviceToHost,
                                  b->stream));
    DOMA_CUDA_TRY(cudaStreamSynchronize(b->stream));
    ++b->iters;
    if (b->h_ctl->error) {
      set_error("a batched sweep wait for an upstream block timed out");
      return DOMA_DEVICE_WAIT_TIMEOUT;
    }
    still = b->h_ctl->still_active;
    DOMA_CUDA_TRY(cudaMemsetAsync(&b->d_ctl->still_active, 0, sizeof(unsigned), b->stream));
    if (still == 0) break;
  }
  if (active) *active = still;
  return DOMA_OK;
}

doma_status doma_batch_state(doma_batch * b, size_t index, const double ** phi,
                             const double ** increment)
{
  if (!b) return bad("null batch");
  if (index >= b->solvers.size()) return bad("problem index out of range");
  DOMA_CUDA_TRY(cudaStreamSynchronize(b->stream));
  if (phi) *phi = b->solvers[index]->d_phi;
  if (increment) *increment = b->solvers[index]->d_dscratch;
  return DOMA_OK;
}

doma_status doma_batch_set_increment(doma_batch * b, size_t index, const double * increment)
{
  if (!b) return bad("null batch");
  if (index >= b->solvers.size()) return bad("problem index out of range");
  if (!increment) return bad("null increment");
  doma_solver * s = b->solvers[index];
  DOMA_CUDA_TRY(cudaMemcpyAsync(s->d_dscratch, increment, (size_t)s->G * s->N * sizeof(double),
                                cudaMemcpyDeviceToDevice, b->stream));
  return accel_source(s->it, DOMA_PREC_FP32, s->d_dscratch, nullptr, s->d_q, b->stream);
}

doma_status doma_batch_reports(doma_batch * b, doma_report * reports, size_t count)
{
  if (!b) return bad("null batch");
  const size_t P = b->solvers.size();
  std::vector<BatchLoop> loops(P);
  DOMA_CUDA_TRY(cudaStreamSynchronize(b->stream));
  DOMA_CUDA_TRY(cudaMemcpy(loops.data(), b->d_loops, P * sizeof(BatchLoop), cudaMemcpyDeviceToHost));
  const auto t1 = std::chrono::steady_clock::now();
  const double ms = std::chrono::duration<double, std::milli>(t1 - b->t_begin).count();
  doma_status first = DOMA_OK;
  for (size_t p = 0; p < P; ++p) {
    const doma_solver * s = b->solvers[p];
    const doma_status ps = loops[p].active ? DOMA_NOT_CONVERGED : (doma_status)loops[p].status;
    if (ps != DOMA_OK && first == DOMA_OK) first = ps;
    if (reports && p < count) {
      doma_report & r = reports[p];
      r.status = ps;
      r.mg_iterations = loops[p].it;
      r.si_iterations = (uint64_t)loops[p].it * s->G;
      r.updates = (uint64_t)loops[p].it * s->G * s->N * (uint64_t)s->D;
      r.kernel_launches = (b->use_graph ? 4ull : 3ull) * b->iters;
      r.mg_residual = loops[p].res;
      r.si_residual = loops[p].res;
      r.solve_ms = ms;
      r.si_counts_len = 1;
      if (r.si_counts && r.si_counts_capacity) r.si_counts[0] = loops[p].it;
    }
  }
  if (first != DOMA_OK) set_error("a problem of the batch did not converge");
  return first;
}

doma_status doma_batch_solve(doma_batch * b, doma_report * reports, size_t count)
{
  if (!b) return bad("null batch");
  DOMA_TRY(doma_batch_begin(b));
  if (b->use_graph) {
    if (!b->exec) DOMA_TRY(build_batch_graph(b));
    DOMA_CUDA_TRY(cudaGraphLaunch(b->exec, b->stream));
    DOMA_CUDA_TRY(cudaMemcpyAsync(b->h_ctl, b->d_ctl, sizeof(BatchCtl), cudaMemcpyDeviceToHost,
                                  b->stream));
    DOMA_CUDA_TRY(cudaStreamSynchronize(b->stream));
    b->iters = b->h_ctl->iters;
    if (b->h_ctl->error) {
      set_error("a batched sweep wait for an upstream block timed out");
      return DOMA_DEVICE_WAIT_TIMEOUT;
    }
  } else {
    uint32_t active = 1;
    DOMA_TRY(doma_batch_iterate(b, b->opts.fs_max_it + 1u, &active));
  }
  return doma_batch_reports(b, reports, count);
}

doma_status doma_batch_get_scalar_flux(doma_batch * b, size_t index, double * out, size_t count)
{
  if (!b) return bad("null batch");
  if (index >= b->solvers.size()) return bad("problem index out of range");
  doma_solver * s = b->solvers[index];
  if (!out || count < (size_t)s->G * s->N) return bad("output buffer too small");
  DOMA_CUDA_TRY(cudaStreamSynchronize(b->stream));
  DOMA_CUDA_TRY(cudaMemcpy(out, s->d_phi, (size_t)s->G * s->N * sizeof(double), cudaMemcpyDeviceToHost));
  return DOMA_OK;
}

void doma_batch_destroy(doma_batch * b) { batch_release(b); }

}  // extern "C"
