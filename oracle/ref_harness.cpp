// ref_harness.cpp -- test infrastructure only.
//
// Drives DOMA's own fixed-source, eigenvalue and transient solvers (the reference, compiled from its
// unmodified sources by oracle/Makefile into oracle/_ref/libdoma_ref.so) from
// a doma_problem description, so that the CPU restatement in oracle/ and the
// GPU library can be pinned against the reference itself.  The product never
// links or loads this file.
//
// What it follows in the reference:
//   * InputParameters is filled in code instead of from XML
//     (include/InputParameters.h:50-117), because the XML reader needs pugixml,
//     which is not available: one x/y/z interval per cell, one block per cell,
//     block id = material index.
//   * BrickMesh3D/2D + {DD,TWDD}TransportSolver3D/2D are built exactly as
//     src/main.cpp:106-292 does, with omp_set_num_threads(T) equal to the T
//     handed to mesh and solver (src/main.cpp:47).
//   * The scalar flux is read through TransportSolver3D<OracleTap> /
//     TransportSolver2D<OracleTap>, explicit specialisations that the mesh and
//     cell classes befriend (include/BrickMesh3D.h:46-47,
//     include/CartesianCell3D.h:114-115).
//   * stdout of the solve (SI/MGI progress lines) is captured and returned.

#include <cstdint>
#include <cstring>
#include <iostream>
#include <sstream>
#include <string>

#include <omp.h>

#include "TransportSolver2D.h"
#include "TransportSolver3D.h"

#include "../include/doma_gb300.h"

struct OracleTap {};

template <>
class TransportSolver3D<OracleTap>
{
public:
  static std::size_t numCells(const BrickMesh3D & mesh) { return mesh._cells.size(); }
  static void readFlux(const BrickMesh3D & mesh, unsigned int G, double * out)
  {
    const std::size_t N = mesh._cells.size();
    for (std::size_t c = 0; c < N; ++c)
      for (unsigned int g = 0; g < G; ++g)
        out[g * N + c] = mesh._cells[c]._total_scalar_flux[g];
  }
  // _current_t_dnps as [D][N], zero where a cell has fewer than D groups.
  static void readDNPs(const BrickMesh3D & mesh, unsigned int D, double * out)
  {
    const std::size_t N = mesh._cells.size();
    for (std::size_t c = 0; c < N; ++c)
      for (unsigned int d = 0; d < D; ++d)
        out[d * N + c] = d < mesh._cells[c]._current_t_dnps.size() ? mesh._cells[c]._current_t_dnps[d] : 0.0;
  }
};

template <>
class TransportSolver2D<OracleTap>
{
public:
  static std::size_t numCells(const BrickMesh2D & mesh) { return mesh._cells.size(); }
  static void readFlux(const BrickMesh2D & mesh, unsigned int G, double * out)
  {
    const std::size_t N = mesh._cells.size();
    for (std::size_t c = 0; c < N; ++c)
      for (unsigned int g = 0; g < G; ++g)
        out[g * N + c] = mesh._cells[c]._total_scalar_flux[g];
  }
  // _current_t_dnps as [D][N], zero where a cell has fewer than D groups.
  static void readDNPs(const BrickMesh2D & mesh, unsigned int D, double * out)
  {
    const std::size_t N = mesh._cells.size();
    for (std::size_t c = 0; c < N; ++c)
      for (unsigned int d = 0; d < D; ++d)
        out[d * N + c] = d < mesh._cells[c]._current_t_dnps.size() ? mesh._cells[c]._current_t_dnps[d] : 0.0;
  }
};

namespace
{
InputParameters
makeParams(const doma_problem * p, const doma_options * o)
{
  InputParameters params;
  params._mode = RunMode::FixedSrc;
  params._num_e_groups = p->num_groups;
  params._t0 = 0.0;
  params._t1 = 1.0;
  params._num_steps = 1u;
  params._ic = TransientIC::Zero;
  params._src_it_tol = o->fs_tol;
  params._gs_tol = o->mg_tol;
  params._k_tol = 1e-5;
  params._dsa = false;
  params._num_src_it = o->fs_max_it;
  params._num_mg_it = o->mg_max_it;
  params._num_polar = p->num_polar;
  params._num_azimuthal = p->num_azimuthal;
  params._eq_type = o->scheme == DOMA_SCHEME_TW_DD ? EquationType::TW_DD : EquationType::DD;
  params._num_dims = p->num_dims;
  params._refinement = 0u;

  params._x_intervals.assign(p->nx, 1u);
  params._y_intervals.assign(p->ny, 1u);
  params._dx.assign(p->dx, p->dx + p->nx);
  params._dy.assign(p->dy, p->dy + p->ny);
  std::size_t N = std::size_t(p->nx) * p->ny;
  if (p->num_dims == 3)
  {
    params._z_intervals.assign(p->nz, 1u);
    params._dz.assign(p->dz, p->dz + p->nz);
    N *= p->nz;
  }
  params._blocks.assign(p->cell_material, p->cell_material + N);

  const unsigned int G = p->num_groups;
  for (unsigned int m = 0; m < p->num_materials; ++m)
  {
    MaterialProps mp;
    mp._num_d_groups = 0u;
    mp._g_total.assign(p->total + m * G, p->total + (m + 1) * G);
    mp._g_g_scatter_mat.assign(p->scatter + m * G * G, p->scatter + (m + 1) * G * G);
    if (p->source)
      mp._g_src.assign(p->source + m * G, p->source + (m + 1) * G);
    if (p->has_fission && p->has_fission[m])
    {
      mp._g_chi_p.assign(p->chi_p + m * G, p->chi_p + (m + 1) * G);
      mp._g_prod.assign(p->nu_sigma_f + m * G, p->nu_sigma_f + (m + 1) * G);
    }
    params._block_mat_info.emplace(m, mp);
  }
  return params;
}

void
copyLog(const std::string & s, char * log, std::size_t cap)
{
  if (!log || cap == 0)
    return;
  const std::size_t n = s.size() < cap - 1 ? s.size() : cap - 1;
  std::memcpy(log, s.data(), n);
  log[n] = '\0';
}
} // namespace

// A deck as DOMA's XML reader leaves it in InputParameters
// (src/InputParameters.cpp:92-524): the solver block, the quadrature, the
// mesh intervals (widths and cell counts, already scaled by refinement + 1)
// with one block id per interval triple, and the materials keyed by block id.
// The XML itself is read by the project's reader, because DOMA's needs
// pugixml; everything after that -- the mesh expansion
// (BrickMesh3D/2D constructors), the solve and the text output -- is DOMA's.
struct ref_deck
{
  uint32_t dims, num_groups, num_polar, num_azimuthal, scheme, mode;  // mode: 0 fixed, 1 eigen
  double fs_tol, mg_tol, k_tol;
  uint32_t fs_max_it, mg_max_it;
  uint32_t nxi, nyi, nzi;                 // intervals per axis (nzi = 1 in 2D)
  const double * dx;                      // interval widths
  const double * dy;
  const double * dz;
  const uint32_t * ix;                    // cells per interval
  const uint32_t * iy;
  const uint32_t * iz;
  const uint32_t * blocks;                // [nzi][nyi][nxi]
  uint32_t num_mats;
  const uint32_t * mat_ids;               // block id of each material
  const double * total;                   // [num_mats][G]
  const double * scatter;                 // [num_mats][G*G], DOMA's stored order
  const uint8_t * has_source;             // [num_mats]
  const double * source;                  // [num_mats][G]
  const uint8_t * has_fission;            // [num_mats]
  const double * chi_p;                   // [num_mats][G]
  const double * prod;                    // [num_mats][G]
};

extern "C" {

// Solve with the reference.  Returns 1 if solveFixedSource returned true, 0 if
// it returned false.  phi_out receives [G][N].  If out_base is non-empty the
// reference also writes its text output (BrickMesh3D::dumpToTextFile).
int
ref_solve(const doma_problem * p, const doma_options * o, unsigned int num_threads,
          double * phi_out, char * log, std::size_t log_cap, const char * out_base)
{
  omp_set_num_threads(static_cast<int>(num_threads));
  const InputParameters params = makeParams(p, o);
  const bool verbose = o->verbose >= 2;
  const std::string base = out_base ? std::string(out_base) : std::string();

  std::ostringstream captured;
  std::streambuf * old = std::cout.rdbuf(captured.rdbuf());
  bool ok = false;
  if (p->num_dims == 3)
  {
    std::array<BoundaryCondition, 6u> bcs;
    bcs.fill(BoundaryCondition::Vacuum);
    BrickMesh3D mesh(params, bcs, num_threads);
    mesh.validateProps();
    if (params._eq_type == EquationType::DD)
    {
      DDTransportSolver3D solver(mesh, params, verbose, num_threads);
      ok = solver.solveFixedSource(base);
    }
    else
    {
      TWDDTransportSolver3D solver(mesh, params, verbose, num_threads);
      ok = solver.solveFixedSource(base);
    }
    TransportSolver3D<OracleTap>::readFlux(mesh, p->num_groups, phi_out);
  }
  else
  {
    std::array<BoundaryCondition, 4u> bcs;
    bcs.fill(BoundaryCondition::Vacuum);
    BrickMesh2D mesh(params, bcs, num_threads);
    mesh.validateProps();
    if (params._eq_type == EquationType::DD)
    {
      DDTransportSolver2D solver(mesh, params, verbose, num_threads);
      ok = solver.solveFixedSource(base);
    }
    else
    {
      TWDDTransportSolver2D solver(mesh, params, verbose, num_threads);
      ok = solver.solveFixedSource(base);
    }
    TransportSolver2D<OracleTap>::readFlux(mesh, p->num_groups, phi_out);
  }
  std::cout.rdbuf(old);
  copyLog(captured.str(), log, log_cap);
  return ok ? 1 : 0;
}

// Eigenvalue solve with the reference (solveEigenvalue,
// src/TransportSolver3D.cpp:29-86).  precision > 0 sets std::cout's precision
// for the captured log first, so that the k and residuals it prints can be
// read back exactly; 0 keeps the stream default (the reference's own log).
int
ref_solve_eigen(const doma_problem * p, const doma_options * o, double k_tol,
                unsigned int num_threads, int precision, double * phi_out, char * log,
                std::size_t log_cap)
{
  omp_set_num_threads(static_cast<int>(num_threads));
  InputParameters params = makeParams(p, o);
  params._mode = RunMode::Eigen;
  params._k_tol = k_tol;
  const bool verbose = o->verbose >= 2;

  std::ostringstream captured;
  if (precision > 0)
    captured.precision(precision);
  std::streambuf * old = std::cout.rdbuf(captured.rdbuf());
  const std::streamsize old_precision = std::cout.precision();
  if (precision > 0)
    std::cout.precision(precision);
  bool ok = false;
  if (p->num_dims == 3)
  {
    std::array<BoundaryCondition, 6u> bcs;
    bcs.fill(BoundaryCondition::Vacuum);
    BrickMesh3D mesh(params, bcs, num_threads);
    mesh.validateProps();
    if (params._eq_type == EquationType::DD)
    {
      DDTransportSolver3D solver(mesh, params, verbose, num_threads);
      ok = solver.solveEigenvalue("");
    }
    else
    {
      TWDDTransportSolver3D solver(mesh, params, verbose, num_threads);
      ok = solver.solveEigenvalue("");
    }
    TransportSolver3D<OracleTap>::readFlux(mesh, p->num_groups, phi_out);
  }
  else
  {
    std::array<BoundaryCondition, 4u> bcs;
    bcs.fill(BoundaryCondition::Vacuum);
    BrickMesh2D mesh(params, bcs, num_threads);
    mesh.validateProps();
    if (params._eq_type == EquationType::DD)
    {
      DDTransportSolver2D solver(mesh, params, verbose, num_threads);
      ok = solver.solveEigenvalue("");
    }
    else
    {
      TWDDTransportSolver2D solver(mesh, params, verbose, num_threads);
      ok = solver.solveEigenvalue("");
    }
    TransportSolver2D<OracleTap>::readFlux(mesh, p->num_groups, phi_out);
  }
  std::cout.precision(old_precision);
  std::cout.rdbuf(old);
  copyLog(captured.str(), log, log_cap);
  return ok ? 1 : 0;
}

// Transient solve with the reference (solveTransient with TransientIC::Zero,
// src/TransportSolver3D.cpp:88-140).  The transient inputs become material
// properties and block step sources as InputParameters.cpp:286-500 would fill
// them; t0 = 0 and t1 = num_steps * dt, so that the reference's own
// dt = (t1 - t0) / num_steps is formed by the same division the caller used.
// phi_out receives the last step's flux [G][N], dnps_out ([D][N]) its
// precursors.  The reference writes its per-step text files under out_base.
int
ref_solve_transient(const doma_problem * p, const doma_options * o, const doma_transient * tr,
                    double t1, unsigned int num_threads, double * phi_out, double * dnps_out,
                    char * log, std::size_t log_cap, const char * out_base)
{
  omp_set_num_threads(static_cast<int>(num_threads));
  InputParameters params = makeParams(p, o);
  params._mode = RunMode::Transient;
  params._t0 = 0.0;
  params._t1 = t1;
  params._num_steps = tr->num_steps;
  params._ic = TransientIC::Zero;
  const unsigned int G = p->num_groups, D = tr->num_d_groups;
  for (unsigned int m = 0; m < p->num_materials; ++m)
  {
    MaterialProps & mp = params._block_mat_info.at(m);
    mp._g_inv_v.assign(tr->inv_v + m * G, tr->inv_v + (m + 1) * G);
    const unsigned int Dm = tr->d_groups ? tr->d_groups[m] : 0u;
    mp._num_d_groups = Dm;
    for (unsigned int g = 0; g < G; ++g)
      for (unsigned int d = 0; d < Dm; ++d)
      {
        mp._n_g_chi_d.push_back(tr->chi_d[(std::size_t(m) * G + g) * D + d]);
        mp._g_n_beta.push_back(tr->beta[(std::size_t(m) * G + g) * D + d]);
      }
    for (unsigned int d = 0; d < Dm; ++d)
      mp._n_lambda.push_back(tr->lambda[std::size_t(m) * D + d]);
    const unsigned int st = tr->step_type ? tr->step_type[m] : 0u;
    if (st != 0u)
    {
      SourceStep step;
      step._type = st == 1u ? StepType::Both : (st == 2u ? StepType::Insert : StepType::Remove);
      step._insert_time = tr->step_insert[m];
      step._remove_time = tr->step_remove[m];
      step._g_src.assign(tr->step_source + m * G, tr->step_source + (m + 1) * G);
      params._block_step_src.emplace(m, step);
    }
  }
  const bool verbose = o->verbose >= 2;
  const std::string base = out_base ? std::string(out_base) : std::string();

  std::ostringstream captured;
  std::streambuf * old = std::cout.rdbuf(captured.rdbuf());
  bool ok = false;
  if (p->num_dims == 3)
  {
    std::array<BoundaryCondition, 6u> bcs;
    bcs.fill(BoundaryCondition::Vacuum);
    BrickMesh3D mesh(params, bcs, num_threads);
    mesh.validateProps();
    if (params._eq_type == EquationType::DD)
    {
      DDTransportSolver3D solver(mesh, params, verbose, num_threads);
      ok = solver.solveTransient(base);
    }
    else
    {
      TWDDTransportSolver3D solver(mesh, params, verbose, num_threads);
      ok = solver.solveTransient(base);
    }
    TransportSolver3D<OracleTap>::readFlux(mesh, G, phi_out);
    if (dnps_out)
      TransportSolver3D<OracleTap>::readDNPs(mesh, D, dnps_out);
  }
  else
  {
    std::array<BoundaryCondition, 4u> bcs;
    bcs.fill(BoundaryCondition::Vacuum);
    BrickMesh2D mesh(params, bcs, num_threads);
    mesh.validateProps();
    if (params._eq_type == EquationType::DD)
    {
      DDTransportSolver2D solver(mesh, params, verbose, num_threads);
      ok = solver.solveTransient(base);
    }
    else
    {
      TWDDTransportSolver2D solver(mesh, params, verbose, num_threads);
      ok = solver.solveTransient(base);
    }
    TransportSolver2D<OracleTap>::readFlux(mesh, G, phi_out);
    if (dnps_out)
      TransportSolver2D<OracleTap>::readDNPs(mesh, D, dnps_out);
  }
  std::cout.rdbuf(old);
  copyLog(captured.str(), log, log_cap);
  return ok ? 1 : 0;
}

// The reference's quadrature, binned by octant: out arrays sized to the total
// order, octant-major; counts[8] per octant.
int
ref_quadrature(unsigned int np, unsigned int na, unsigned int dims, double * mu, double * eta,
               double * xi, double * w, unsigned int * counts)
{
  GCAngularQuadrature q(2u * na, 2u * np, dims);
  std::size_t k = 0;
  for (unsigned int o = 0; o < 8u; ++o)
  {
    const Octant oct = static_cast<Octant>(o);
    counts[o] = q.order(oct);
    for (unsigned int n = 0; n < q.order(oct); ++n, ++k)
    {
      q.direction(oct, n, mu[k], eta[k], xi[k]);
      w[k] = q.weight(oct, n);
    }
  }
  return static_cast<int>(k);
}


// Solve a deck with the reference.  Returns 1 / 0 for DOMA's true / false and
// -1 if phi_cap is too small.  phi_out receives [G][N] of the expanded mesh
// and *num_cells its N.  DOMA keeps k private: eigen decks print it in the
// captured log, with `precision` digits when precision > 0 (k_out is set to 0).
// With a non-empty out_base DOMA also writes its text output there.
int
ref_solve_deck(const ref_deck * d, unsigned int num_threads, double * phi_out, std::size_t phi_cap,
               std::size_t * num_cells, double * k_out, char * log, std::size_t log_cap,
               const char * out_base, int precision)
{
  if (k_out) *k_out = 0.0;
  omp_set_num_threads(static_cast<int>(num_threads));
  InputParameters params;
  params._mode = d->mode == 1 ? RunMode::Eigen : RunMode::FixedSrc;
  params._num_e_groups = d->num_groups;
  params._t0 = 0.0;
  params._t1 = 1.0;
  params._num_steps = 1u;
  params._ic = TransientIC::Zero;
  params._src_it_tol = d->fs_tol;
  params._gs_tol = d->mg_tol;
  params._k_tol = d->k_tol;
  params._dsa = false;
  params._num_src_it = d->fs_max_it;
  params._num_mg_it = d->mg_max_it;
  params._num_polar = d->num_polar;
  params._num_azimuthal = d->num_azimuthal;
  params._eq_type = d->scheme == DOMA_SCHEME_TW_DD ? EquationType::TW_DD : EquationType::DD;
  params._num_dims = d->dims;
  params._refinement = 0u;
  params._x_intervals.assign(d->ix, d->ix + d->nxi);
  params._y_intervals.assign(d->iy, d->iy + d->nyi);
  params._dx.assign(d->dx, d->dx + d->nxi);
  params._dy.assign(d->dy, d->dy + d->nyi);
  std::size_t nb = std::size_t(d->nxi) * d->nyi;
  if (d->dims == 3)
  {
    params._z_intervals.assign(d->iz, d->iz + d->nzi);
    params._dz.assign(d->dz, d->dz + d->nzi);
    nb *= d->nzi;
  }
  params._blocks.assign(d->blocks, d->blocks + nb);
  const unsigned int G = d->num_groups;
  for (unsigned int m = 0; m < d->num_mats; ++m)
  {
    MaterialProps mp;
    mp._num_d_groups = 0u;
    mp._g_total.assign(d->total + m * G, d->total + (m + 1) * G);
    mp._g_g_scatter_mat.assign(d->scatter + m * G * G, d->scatter + (m + 1) * G * G);
    if (d->has_source[m])
      mp._g_src.assign(d->source + m * G, d->source + (m + 1) * G);
    if (d->has_fission[m])
    {
      mp._g_chi_p.assign(d->chi_p + m * G, d->chi_p + (m + 1) * G);
      mp._g_prod.assign(d->prod + m * G, d->prod + (m + 1) * G);
    }
    params._block_mat_info.emplace(d->mat_ids[m], mp);
  }
  const std::string base = out_base ? std::string(out_base) : std::string();
  const bool eigen = d->mode == 1;

  std::ostringstream captured;
  std::streambuf * old = std::cout.rdbuf(captured.rdbuf());
  const std::streamsize old_precision = std::cout.precision();
  if (precision > 0)
    std::cout.precision(precision);
  bool ok = false;
  int rc = 0;
  auto finish = [&](auto & mesh, auto & solver, auto reader, auto counter) {
    ok = eigen ? solver.solveEigenvalue(base) : solver.solveFixedSource(base);
    const std::size_t N = counter(mesh);
    *num_cells = N;
    if (N * G > phi_cap)
    {
      rc = -1;
      return;
    }
    reader(mesh, G, phi_out);
  };
  if (d->dims == 3)
  {
    std::array<BoundaryCondition, 6u> bcs;
    bcs.fill(BoundaryCondition::Vacuum);
    BrickMesh3D mesh(params, bcs, num_threads);
    mesh.validateProps();
    if (params._eq_type == EquationType::DD)
    {
      DDTransportSolver3D solver(mesh, params, false, num_threads);
      finish(mesh, solver, TransportSolver3D<OracleTap>::readFlux, TransportSolver3D<OracleTap>::numCells);
    }
    else
    {
      TWDDTransportSolver3D solver(mesh, params, false, num_threads);
      finish(mesh, solver, TransportSolver3D<OracleTap>::readFlux, TransportSolver3D<OracleTap>::numCells);
    }
  }
  else
  {
    std::array<BoundaryCondition, 4u> bcs;
    bcs.fill(BoundaryCondition::Vacuum);
    BrickMesh2D mesh(params, bcs, num_threads);
    mesh.validateProps();
    if (params._eq_type == EquationType::DD)
    {
      DDTransportSolver2D solver(mesh, params, false, num_threads);
      finish(mesh, solver, TransportSolver2D<OracleTap>::readFlux, TransportSolver2D<OracleTap>::numCells);
    }
    else
    {
      TWDDTransportSolver2D solver(mesh, params, false, num_threads);
      finish(mesh, solver, TransportSolver2D<OracleTap>::readFlux, TransportSolver2D<OracleTap>::numCells);
    }
  }
  std::cout.precision(old_precision);
  std::cout.rdbuf(old);
  copyLog(captured.str(), log, log_cap);
  return rc < 0 ? rc : (ok ? 1 : 0);
}

} // extern "C"
