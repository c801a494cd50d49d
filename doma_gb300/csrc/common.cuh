// common.cuh -- shared definitions of the GB300 sweep library.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/doma_gb300.h"

namespace doma {

constexpr double kPi = 3.14159265358979323846;  // M_PI

// Largest sweep CTA: 16 ordinates x 16 pencils.
constexpr int kMaxSweepThreads = 256;

// Error reporting (per thread, read through doma_last_error()).
void set_error(const std::string & msg);
const char * get_error();

#define DOMA_CUDA_TRY(expr)                                                                    \
  do {                                                                                         \
    cudaError_t _e = (expr);                                                                   \
    if (_e != cudaSuccess) {                                                                   \
      ::doma::set_error(std::string(#expr) + ": " + cudaGetErrorString(_e));                   \
      return DOMA_CUDA_ERROR;                                                                  \
    }                                                                                          \
  } while (0)

#define DOMA_TRY(expr)                    \
  do {                                    \
    doma_status _s = (expr);              \
    if (_s != DOMA_OK) return _s;         \
  } while (0)

// Ordinates of one octant handled by one sweep task (two per warp), at most
// kGroupMax.  The FP32 modes run groups of 8: twice the tasks per sweep, each
// half as long, which shortens the dataflow's critical path (measured on
// GB300: the DD 100^3 duct with 36 ordinates per octant 1.73 -> 1.38 ms per
// sweep; TW-DD 64^3 with 16 ordinates 258 -> 244 us once its partials were
// summed on the FP32 pipes and its body given 5 CTAs per SM).  The FP64 exact
// mode, whose tasks are bound by the SM's small FP64 pipe, runs groups of 2
// (one warp): 20^3 DD solve 37.0 -> 32.4 ms, 100^3 duct 957 -> 756 ms, against
// groups of 16; its bits do not depend on the grouping (every ordinate's w psi
// is kept and summed in DOMA's order).  Every kernel of one (precision,
// scheme) uses the same size, so single, batched and allocation-free sweeps
// give the same bits.
constexpr int kGroupMax = 16;
constexpr int kGroupExact = 2;   // the FP64 exact mode's group size
__host__ __device__ constexpr int ordinate_group(int precision, int /* scheme */)
{
  return precision == DOMA_PREC_FP32 ? 8 : kGroupExact;
}

#ifdef __CUDACC__
// FP32 mode's scalar-flux partial of one (group, octant, ordinate group) slot
// is the slot's Kahan sum kept as the unevaluated float pair hi + lo (hi =
// the sum, lo = minus its compensation).  The epilogues add a cell's slots in
// slot order in double-float arithmetic (a float pair carrying about 48
// significant bits): Knuth's TwoSum of the high parts, the low parts added,
// and Dekker's FastTwoSum to renormalise -- the "sloppy" double-float
// addition of Hida, Li and Bailey's quad-double library.  It runs on the FP32
// pipes, which GB300 issues 64 times as fast as FP64 adds, where a cell's 8
// to 40 FP64 adds made the epilogues FP64-bound.  Every kernel that reads the
// partials uses this accumulator, so they all give the same bits.
struct PartialSum {
  float h = 0.f, l = 0.f;
  __device__ __forceinline__ void add(float2 p)
  {
    const float s = __fadd_rn(h, p.x);
    const float bb = __fsub_rn(s, h);
    const float e = __fadd_rn(__fsub_rn(h, __fsub_rn(s, bb)), __fsub_rn(p.x, bb));
    const float t = __fadd_rn(e, __fadd_rn(l, p.y));
    h = __fadd_rn(s, t);
    l = __fsub_rn(t, __fsub_rn(h, s));
  }
  __device__ __forceinline__ double value() const { return __dadd_rn((double)h, (double)l); }
};
#endif

// One sweep task: energy group (multigroup mode; 0 otherwise), octant,
// ordinate group and block coordinates in the octant's sweep frame
// (i' = i for +mu, nx-1-i for -mu, likewise for y and z).
struct Task {
  int oct, og, bi, bj, bk, grp;
};

// A task of a batched sweep: the problem it belongs to and its own task.
struct BatchTask {
  Task t;
  int prob;
};

// Per-problem loop state of a batched solve (device memory).
struct BatchLoop {
  unsigned active;   // 1 while the problem iterates
  unsigned it;       // iterations done
  unsigned status;   // doma_status once finished
  unsigned pad;
  double res;        // last relative increment norm
};

// Everything a sweep launch needs.  Pointers are device pointers.
template <typename T>
struct SweepArgs {
  int nx, ny, nz;
  int d_oct;           // ordinates per octant
  int d_total;         // ordinates over all octants (exact mode row length)
  int ngroups;         // ordinate groups per octant (ceil(d_oct / ordinate_group))
  int nbx, nby, nbz;   // blocks per axis
  int tx;              // block length along x of this schedule (the batched kernel dispatches on it)
  int num_tasks;
  const Task * tasks;  // all tasks, sorted by level (a topological order)
  int task_offset;     // level-synchronous mode: first task of this launch
  const int * oct_offset;  // [8] first ordinate of each octant (octant-major tables)
  // quadrature (octant-major, |cosines|, weights)
  const double * amu;
  const double * aeta;
  const double * axi;
  const double * wgt;
  const float * amu_f;
  const float * aeta_f;
  const float * axi_f;
  // geometry in the sweep precision (physical index): widths and the
  // coefficients 2|mu|/dx [D][nx], 2|eta|/dy [D][ny], 2|xi|/dz [D][nz]
  const T * wx;
  const T * wy;
  const T * wz;
  const T * cx;
  const T * cy;
  const T * cz;
  // per-cell sweep inputs: [groups in flight][N] (one group in Gauss-Seidel mode)
  const T * q;
  const T * sigt;
  // face planes (sweep frame, per (group in flight, octant, ordinate group),
  // ordinate_group slots per face): x [G*8][ngroups][nz][ny][slots], y
  // [G*8][ngroups][nz][nx][slots], z [G*8][ngroups][ny][nx][slots]
  T * xf;
  T * yf;
  T * zf;
  double * wpsi;     // exact mode: [groups in flight][N][d_total] weighted angular flux
  float2 * octphi;   // fp32 mode: [G*8*ngroups][N] scalar-flux partials (hi, lo) per (group, octant, ordinate group)
  double theta;
  // persistent-mode scheduling state (device memory, kept between sweeps)
  unsigned * ticket;      // next task to claim (reset by the last CTA to leave)
  unsigned * exit_count;  // CTAs that have left
  unsigned * epoch;       // sweeps completed
  unsigned * done;        // [G*8][ngroups][nbz][nby][nbx] epoch in which the task finished
  int * error;            // nonzero: a bounded wait gave up (DOMA_DEVICE_WAIT_TIMEOUT)
  unsigned spin_limit;    // polls before a wait gives up
  unsigned wait_bias;     // 0; nonzero only in the wait-timeout test, where every
                          // wait targets an epoch that no block ever publishes
};

// Sweep schedule of one solver: block shape and the task list by level.
// The block is tx cells along x by a fixed 16-pencil cross-section
// (4 x 4 in (y, z) for 3D, 16 in y for 2D).
struct Schedule {
  int tx = 0, ty = 0, tz = 0;
  int ngroups = 1, gs = 1;
  int nbx = 0, nby = 0, nbz = 0;
  int threads = 0;
  size_t smem = 0;
  bool many = false;       // FP32: the body for many tasks per level (sweep_many_ctas)
  bool persistent = true;  // dataflow kernel (true) or one launch per level
  int grid = 0;            // persistent grid (CTAs)
  std::vector<Task> tasks;
  std::vector<int> level_begin;  // size levels+1
};

// Launchers (sweep.cu).
doma_status launch_sweep(int dims, int precision, int scheme, const Schedule & s,
                         const SweepArgs<double> * a64, const SweepArgs<float> * a32,
                         cudaStream_t stream, uint64_t * launches);
int sweep_tile_x(int requested);  // supported block length along x: 8, 16 or 32
// Threads of a sweep CTA for an ordinate group of gs: one per (ordinate,
// pencil), in whole warps.
int sweep_threads(int gs);
size_t sweep_smem_bytes(int dims, int precision, int scheme, int tx);
// The FP32 modes compile two bodies with the same arithmetic: DD for 8 and 12
// CTAs per SM (64 and 40 registers), TW-DD for 2 and 3 (128 and 80).  A
// schedule with three or more (ordinate group, group in flight) slots per
// octant has enough independent tasks per wavefront level for the body with
// more CTAs; fewer favour the longer-lived registers.
bool sweep_many_ctas(int precision, int ngroups, int groups_in_flight);
doma_status sweep_prepare(int dims, int precision, int scheme, int tx, size_t smem, bool many);
// CTAs of the persistent sweep kernel that fit on the device at once.
int sweep_resident_ctas(int dims, int precision, int scheme, int tx, int threads, size_t smem,
                        bool many);

// One persistent sweep over every active problem of a batch (FP32).  The
// counters are the batch's own; args[p] is problem p's sweep arguments, whose
// tx (8, 16 or 32) may differ from problem to problem.
doma_status launch_sweep_batch(int dims, int scheme, int grid, int threads, size_t smem,
                               const SweepArgs<float> * args, const BatchTask * tasks,
                               int num_tasks, unsigned * ticket, unsigned * exit_count,
                               unsigned * epoch, const BatchLoop * loops, cudaStream_t stream);
size_t sweep_batch_smem_bytes(int dims, int scheme);
int sweep_batch_resident_ctas(int dims, int scheme, int threads, size_t smem);

// Host quadrature (quadrature.cpp): np, na <= kMaxQuadPolar; allocates nothing.
constexpr unsigned kMaxQuadPolar = 512;
int gc_quadrature(unsigned np, unsigned na, unsigned dims, double * mu, double * eta,
                  double * xi, double * w, unsigned counts[8]);

}  // namespace doma
