// TransportSolver.cpp -- drop-in solvers over the C ABI (see TransportSolver.h).
#include "doma/TransportSolver.h"

#include <cstdio>
#include <map>
#include <stdexcept>

#include "../../../include/doma_gb300.h"

namespace {

// Materials of a deck as the C ABI wants them: block ids renumbered 0..M-1
// in increasing id order, a source / fission entry per material (zeros and a
// false fission flag where the deck gives none, which DOMA treats alike).
struct ProblemData
{
  std::vector<uint32_t> cell_material;
  std::vector<double> total, scatter, source, chi, nsf;
  std::vector<uint8_t> fission;
  bool any_source = false, any_fission = false;
  unsigned int M = 0;
};

ProblemData gather(const InputParameters & params, const std::vector<unsigned int> & blocks)
{
  if (params._mode == RunMode::Transient)
    throw std::runtime_error("transient solves do not run on the GPU library (steady and eigen do)");
  const unsigned int G = params._num_e_groups;
  std::map<unsigned int, unsigned int> index;
  for (const auto & kv : params._block_mat_info) index.emplace(kv.first, 0u);
  ProblemData d;
  unsigned int m = 0;
  for (auto & kv : index) kv.second = m++;
  d.M = m;
  d.total.assign((size_t)m * G, 0.0);
  d.scatter.assign((size_t)m * G * G, 0.0);
  d.source.assign((size_t)m * G, 0.0);
  d.chi.assign((size_t)m * G, 0.0);
  d.nsf.assign((size_t)m * G, 0.0);
  d.fission.assign(m, 0u);
  for (const auto & kv : index) {
    const MaterialProps & p = params._block_mat_info.at(kv.first);
    const size_t o = kv.second;
    if (p._g_total.size() != G || p._g_g_scatter_mat.size() != (size_t)G * G)
      throw std::runtime_error("block " + std::to_string(kv.first) + " has incomplete cross sections");
    std::copy(p._g_total.begin(), p._g_total.end(), d.total.begin() + o * G);
    std::copy(p._g_g_scatter_mat.begin(), p._g_g_scatter_mat.end(), d.scatter.begin() + o * G * G);
    if (!p._g_src.empty()) {
      if (p._g_src.size() != G) throw std::runtime_error("bad source size");
      std::copy(p._g_src.begin(), p._g_src.end(), d.source.begin() + o * G);
      d.any_source = true;
    }
    if (!p._g_chi_p.empty()) {
      if (p._g_chi_p.size() != G || p._g_prod.size() != G)
        throw std::runtime_error("block " + std::to_string(kv.first) +
                                 " has chi_p without a matching nu_sigma_f");
      std::copy(p._g_chi_p.begin(), p._g_chi_p.end(), d.chi.begin() + o * G);
      std::copy(p._g_prod.begin(), p._g_prod.end(), d.nsf.begin() + o * G);
      d.fission[o] = 1u;
      d.any_fission = true;
    }
  }
  d.cell_material.resize(blocks.size());
  for (size_t c = 0; c < blocks.size(); ++c) {
    auto it = index.find(blocks[c]);
    if (it == index.end())
      throw std::runtime_error("Block " + std::to_string(blocks[c]) +
                               " (defined on the mesh) has no material properties!");
    d.cell_material[c] = it->second;
  }
  return d;
}

doma_options make_options(const InputParameters & params, unsigned int scheme, bool verbose)
{
  doma_options o;
  doma_default_options(&o);
  o.scheme = scheme;
  o.theta = params._theta;
  o.precision = params._precision == SweepPrecision::FP32 ? DOMA_PREC_FP32 : DOMA_PREC_FP64;
  o.fs_tol = params._src_it_tol;
  o.fs_max_it = params._num_src_it;
  o.mg_tol = params._gs_tol;
  o.mg_max_it = params._num_mg_it;
  o.verbose = verbose ? 2u : 1u;
  return o;
}

doma_solver * create(const doma_problem & p, const doma_options & o)
{
  doma_solver * s = nullptr;
  const doma_status st = doma_solver_create(&p, &o, &s);
  if (st != DOMA_OK)
    throw std::runtime_error(std::string("doma_solver_create failed: ") + doma_last_error());
  return s;
}

void fill_stats(const doma_report & r, bool converged, std::vector<uint32_t> & counts,
                SolveStats & stats);

bool run(doma_solver * s, size_t flux_values, std::vector<double> & flux, SolveStats & stats)
{
  std::vector<uint32_t> counts(1u << 16);
  doma_report r{};
  r.si_counts = counts.data();
  r.si_counts_capacity = counts.size();
  const doma_status st = doma_solver_solve_fixed_source(s, &r);
  if (st != DOMA_OK && st != DOMA_NOT_CONVERGED)
    throw std::runtime_error(std::string("fixed-source solve failed: ") + doma_last_error());
  flux.resize(flux_values);
  if (doma_solver_get_scalar_flux(s, flux.data(), flux.size()) != DOMA_OK)
    throw std::runtime_error(std::string("reading the scalar flux failed: ") + doma_last_error());
  fill_stats(r, st == DOMA_OK, counts, stats);
  return stats.converged;
}

void fill_stats(const doma_report & r, bool converged, std::vector<uint32_t> & counts,
                SolveStats & stats)
{
  stats.converged = converged;
  stats.mg_iterations = r.mg_iterations;
  stats.source_iterations = r.si_iterations;
  stats.updates = r.updates;
  stats.mg_residual = r.mg_residual;
  stats.si_residual = r.si_residual;
  stats.solve_ms = r.solve_ms;
  counts.resize(std::min(r.si_counts_len, counts.size()));
  stats.si_counts = counts;
}

// DOMA's solveEigenvalue through the C ABI; k_tol from the deck
// (InputParameters::_k_tol).
bool run_eigen(doma_solver * s, double k_tol, size_t flux_values, std::vector<double> & flux,
               SolveStats & stats, double & k)
{
  std::vector<uint32_t> counts(1u << 16);
  doma_report r{};
  r.si_counts = counts.data();
  r.si_counts_capacity = counts.size();
  const doma_status st = doma_solver_solve_eigenvalue(s, k_tol, &r, &k);
  if (st != DOMA_OK && st != DOMA_NOT_CONVERGED)
    throw std::runtime_error(std::string("eigenvalue solve failed: ") + doma_last_error());
  flux.resize(flux_values);
  if (doma_solver_get_scalar_flux(s, flux.data(), flux.size()) != DOMA_OK)
    throw std::runtime_error(std::string("reading the scalar flux failed: ") + doma_last_error());
  fill_stats(r, st == DOMA_OK, counts, stats);
  return stats.converged;
}

}  // namespace

// ---------------------------------------------------------------------------
template <typename T>
TransportSolver3D<T>::TransportSolver3D(BrickMesh3D & mesh, const InputParameters & params, bool verbose,
                                        unsigned int /*num_threads*/)
  : _mesh(mesh), _params(params), _verbose(verbose)
{
  _mesh._num_groups = params._num_e_groups;
  _mesh._flux.assign((size_t)_mesh._num_groups * _mesh.numCells(), 0.0);
}

template <typename T>
TransportSolver3D<T>::~TransportSolver3D()
{
  if (_solver) doma_solver_destroy(_solver);
}

template <typename T>
doma_solver * TransportSolver3D<T>::solver()
{
  if (!_solver) {
    const ProblemData d = gather(_params, _mesh.cellBlocks());
    doma_problem p{};
    p.num_dims = 3;
    p.nx = _mesh.numX();
    p.ny = _mesh.numY();
    p.nz = _mesh.numZ();
    p.dx = _mesh.widthsX().data();
    p.dy = _mesh.widthsY().data();
    p.dz = _mesh.widthsZ().data();
    p.num_groups = _params._num_e_groups;
    p.num_materials = d.M;
    p.cell_material = d.cell_material.data();
    p.total = d.total.data();
    p.scatter = d.scatter.data();
    p.source = d.source.data();
    p.has_fission = d.any_fission ? d.fission.data() : nullptr;
    p.chi_p = d.any_fission ? d.chi.data() : nullptr;
    p.nu_sigma_f = d.any_fission ? d.nsf.data() : nullptr;
    p.num_polar = _params._num_polar;
    p.num_azimuthal = _params._num_azimuthal;
    const doma_options o = make_options(_params, T::scheme, _verbose);
    _solver = create(p, o);
  }
  return _solver;
}

template <typename T>
bool TransportSolver3D<T>::solveFixedSource(const std::string & output_file_base, const double & /*t*/)
{
  const bool ok = run(solver(), _mesh._flux.size(), _mesh._flux, _stats);
  if (ok && output_file_base != "") _mesh.dumpToTextFile(output_file_base);
  return ok;
}

// DOMA's TransportSolver3D::solveEigenvalue (src/TransportSolver3D.cpp:29-86).
template <typename T>
bool TransportSolver3D<T>::solveEigenvalue(const std::string & output_file_base)
{
  const bool ok = run_eigen(solver(), _params._k_tol, _mesh._flux.size(), _mesh._flux, _stats, _k);
  if (ok && output_file_base != "") _mesh.dumpToTextFile(output_file_base);
  return ok;
}

// ---------------------------------------------------------------------------
template <typename T>
TransportSolver2D<T>::TransportSolver2D(BrickMesh2D & mesh, const InputParameters & params, bool verbose,
                                        unsigned int /*num_threads*/)
  : _mesh(mesh), _params(params), _verbose(verbose)
{
  _mesh._num_groups = params._num_e_groups;
  _mesh._flux.assign((size_t)_mesh._num_groups * _mesh.numCells(), 0.0);
}

template <typename T>
TransportSolver2D<T>::~TransportSolver2D()
{
  if (_solver) doma_solver_destroy(_solver);
}

template <typename T>
doma_solver * TransportSolver2D<T>::solver()
{
  if (!_solver) {
    const ProblemData d = gather(_params, _mesh.cellBlocks());
    const double one = 1.0;
    doma_problem p{};
    p.num_dims = 2;
    p.nx = _mesh.numX();
    p.ny = _mesh.numY();
    p.nz = 1;
    p.dx = _mesh.widthsX().data();
    p.dy = _mesh.widthsY().data();
    p.dz = &one;
    p.num_groups = _params._num_e_groups;
    p.num_materials = d.M;
    p.cell_material = d.cell_material.data();
    p.total = d.total.data();
    p.scatter = d.scatter.data();
    p.source = d.source.data();
    p.has_fission = d.any_fission ? d.fission.data() : nullptr;
    p.chi_p = d.any_fission ? d.chi.data() : nullptr;
    p.nu_sigma_f = d.any_fission ? d.nsf.data() : nullptr;
    p.num_polar = _params._num_polar;
    p.num_azimuthal = _params._num_azimuthal;
    const doma_options o = make_options(_params, T::scheme, _verbose);
    _solver = create(p, o);
  }
  return _solver;
}

template <typename T>
bool TransportSolver2D<T>::solveFixedSource(const std::string & output_file_base, const double & /*t*/)
{
  const bool ok = run(solver(), _mesh._flux.size(), _mesh._flux, _stats);
  if (ok && output_file_base != "") _mesh.dumpToTextFile(output_file_base);
  return ok;
}

// DOMA's TransportSolver2D::solveEigenvalue (src/TransportSolver2D.cpp:31-88).
template <typename T>
bool TransportSolver2D<T>::solveEigenvalue(const std::string & output_file_base)
{
  const bool ok = run_eigen(solver(), _params._k_tol, _mesh._flux.size(), _mesh._flux, _stats, _k);
  if (ok && output_file_base != "") _mesh.dumpToTextFile(output_file_base);
  return ok;
}

template class TransportSolver3D<DiamondDifference3D>;
template class TransportSolver3D<TWDiamondDifference3D>;
template class TransportSolver2D<DiamondDifference2D>;
template class TransportSolver2D<TWDiamondDifference2D>;
