// iteration.cuh -- per-cell iteration kernels (iteration.cu).
#pragma once

#include "common.cuh"

namespace doma {

struct IterArgs {
  size_t N = 0;               // cells
  int G = 0;                  // groups
  int D = 0;                  // ordinates (exact-mode row length of wpsi)
  int grid = 0;               // fixed grid of every per-cell kernel
  unsigned oct_mask = 0;      // octants that carry ordinates
  double src_scale = 0.25;    // 1/(4 pi) prefactor numerator: 0.25 (3D), 0.5 (2D)
  const double * vol = nullptr;       // [N]
  const uint32_t * mat = nullptr;     // [N]
  const double * total = nullptr;     // [M][G]
  const double * scatter = nullptr;   // [M][G][G] [to][from]
  const double * source = nullptr;    // [M][G] or null
  const uint8_t * fis = nullptr;      // [M] or null
  const double * chi = nullptr;       // [M][G]
  const double * nsf = nullptr;       // [M][G]
  double * phi = nullptr;             // [G][N]
  double * prev = nullptr;            // [G][N]
  const double * wpsi = nullptr;      // exact: [N][D]
  const double * octphi = nullptr;    // fp32: [8][N]
  double * partials = nullptr;        // [grid][2]
  unsigned * ticket = nullptr;        // last-block ticket (kept at 0 between launches)
};

doma_status launch_mg_source(const IterArgs & a, int g, int precision, void * q, void * sigt,
                             cudaStream_t st);
doma_status launch_si_epilogue(const IterArgs & a, int g, int precision, void * q,
                               double * norms, cudaStream_t st);
doma_status launch_mg_residual(const IterArgs & a, double * norms, cudaStream_t st);
int iteration_block();

}  // namespace doma
