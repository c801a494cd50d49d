// common.cuh -- shared definitions of the GB300 sweep library.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/doma_gb300.h"

namespace doma {

constexpr double kPi = 3.14159265358979323846;  // M_PI

// Largest sweep CTA (ordinates x pencils); bounds registers at 128 per thread.
constexpr int kMaxSweepThreads = 512;

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

// One sweep block task: octant and block coordinates in the octant's sweep
// frame (i' = i for +mu, nx-1-i for -mu, likewise for y and z).
struct Task {
  int oct, bi, bj, bk;
};

// Everything a sweep launch needs.  Pointers are device pointers.
template <typename T>
struct SweepArgs {
  int nx, ny, nz;
  int d_oct;           // ordinates per octant
  int d_total;         // ordinates over all octants (exact mode row length)
  int tx, ty, tz;      // block shape in cells
  const Task * tasks;  // all tasks, sorted by level
  int task_offset;     // first task of this launch
  const int * oct_offset;  // [8] first ordinate of each octant (octant-major tables)
  // quadrature (octant-major, |cosines|)
  const double * amu;
  const double * aeta;
  const double * axi;
  const double * wgt;
  const float * amu_f;
  const float * aeta_f;
  const float * axi_f;
  // geometry (physical index)
  const double * dx;
  const double * dy;
  const double * dz;
  // per-cell sweep inputs of the group being swept
  const T * q;
  const T * sigt;
  // face buffers (sweep frame, per octant): x [8][nz][ny][d_oct],
  // y [8][nz][nx][d_oct], z [8][ny][nx][d_oct]
  T * xf;
  T * yf;
  T * zf;
  double * wpsi;     // exact mode: [N][d_total] weighted angular flux
  double * octphi;   // fp32 mode: [8][N] per-octant scalar-flux partials
  double theta;
};

// Sweep schedule of one solver: block shape and the task list by level.
struct Schedule {
  int tx = 0, ty = 0, tz = 0;
  int nbx = 0, nby = 0, nbz = 0;
  int threads = 0;
  size_t smem = 0;
  std::vector<Task> tasks;
  std::vector<int> level_begin;  // size levels+1
};

// Launchers (sweep.cu).
doma_status launch_sweep(int dims, int precision, int scheme, const Schedule & s,
                         const SweepArgs<double> * a64, const SweepArgs<float> * a32,
                         cudaStream_t stream, uint64_t * launches);
size_t sweep_smem_bytes(int dims, int precision, int scheme, int tx, int ty, int tz, int d_oct);
doma_status sweep_prepare(size_t smem);

// Host quadrature (quadrature.cpp).
int gc_quadrature(unsigned np, unsigned na, unsigned dims, double * mu, double * eta,
                  double * xi, double * w, unsigned counts[8]);

}  // namespace doma
