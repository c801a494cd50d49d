// TransportSolver.cpp -- drop-in solvers over the C ABI (see TransportSolver.h).
#include "doma/TransportSolver.h"

#include <algorithm>
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
  std::vector<unsigned int> ids;          // block id of each material index
  std::vector<uint32_t> cell_material;
  std::vector<double> total, scatter, source, chi, nsf;
  std::vector<uint8_t> fission;
  bool any_source = false, any_fission = false;
  unsigned int M = 0;
};

ProblemData gather(const InputParameters & params, const std::vector<unsigned int> & blocks)
{
  const unsigned int G = params._num_e_groups;
  std::map<unsigned int, unsigned int> index;
  for (const auto & kv : params._block_mat_info) index.emplace(kv.first, 0u);
  ProblemData d;
  unsigned int m = 0;
  for (auto & kv : index) {
    kv.second = m++;
    d.ids.push_back(kv.first);
  }
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

// The transient data of a deck in the C ABI's layout: per material index
// (block ids in increasing order), delayed-group arrays padded to the most
// any block has; dt = (t1 - t0) / t_steps as DOMA forms it
// (src/TransportSolver3D.cpp:21).
struct TransientData
{
  std::vector<double> inv_v, chi_d, beta, lambda, ins, rem, src;
  std::vector<uint32_t> dg, type;
  doma_transient tr{};
};

TransientData gather_transient(const InputParameters & params, const std::vector<unsigned int> & ids)
{
  if (params._ic != TransientIC::Zero)
    throw std::runtime_error("only zero initial conditions are offered for transients (DOMA's "
                             "steady-state start reads its previous-step and precursor arrays "
                             "before it sizes them)");
  const size_t G = params._num_e_groups, M = ids.size();
  size_t D = 0;
  for (unsigned int id : ids) D = std::max<size_t>(D, params._block_mat_info.at(id)._num_d_groups);
  TransientData t;
  t.inv_v.assign(M * G, 0.0);
  t.dg.assign(M, 0u);
  t.chi_d.assign(std::max<size_t>(M * G * D, 1), 0.0);
  t.beta.assign(std::max<size_t>(M * G * D, 1), 0.0);
  t.lambda.assign(std::max<size_t>(M * D, 1), 0.0);
  t.type.assign(M, DOMA_STEP_NONE);
  t.ins.assign(M, 0.0);
  t.rem.assign(M, 0.0);
  t.src.assign(M * G, 0.0);
  for (size_t m = 0; m < M; ++m) {
    const unsigned int id = ids[m];
    const MaterialProps & p = params._block_mat_info.at(id);
    const size_t Dm = p._num_d_groups;
    if (p._g_inv_v.size() != G)
      throw std::runtime_error("block " + std::to_string(id) + " needs " + std::to_string(G) +
                               " inverse velocities for a transient");
    if (p._n_g_chi_d.size() != G * Dm || p._g_n_beta.size() != G * Dm || p._n_lambda.size() != Dm)
      throw std::runtime_error("block " + std::to_string(id) + " has incomplete delayed-neutron data");
    std::copy(p._g_inv_v.begin(), p._g_inv_v.end(), t.inv_v.begin() + m * G);
    t.dg[m] = (uint32_t)Dm;
    for (size_t g = 0; g < G; ++g)
      for (size_t d = 0; d < Dm; ++d) {
        t.chi_d[(m * G + g) * D + d] = p._n_g_chi_d[g * Dm + d];
        t.beta[(m * G + g) * D + d] = p._g_n_beta[g * Dm + d];
      }
    for (size_t d = 0; d < Dm; ++d) t.lambda[m * D + d] = p._n_lambda[d];
    auto it = params._block_step_src.find(id);
    if (it != params._block_step_src.end()) {
      const SourceStep & st = it->second;
      if (st._g_src.size() != G)
        throw std::runtime_error("the step source of block " + std::to_string(id) + " needs " +
                                 std::to_string(G) + " values");
      t.type[m] = st._type == StepType::Both ? DOMA_STEP_BOTH
                  : st._type == StepType::Insert ? DOMA_STEP_INSERT : DOMA_STEP_REMOVE;
      t.ins[m] = st._insert_time;
      t.rem[m] = st._remove_time;
      std::copy(st._g_src.begin(), st._g_src.end(), t.src.begin() + m * G);
    }
  }
  t.tr.dt = (params._t1 - params._t0) / static_cast<double>(params._num_steps);
  t.tr.num_steps = params._num_steps;
  t.tr.num_d_groups = (uint32_t)D;
  t.tr.inv_v = t.inv_v.data();
  t.tr.d_groups = t.dg.data();
  t.tr.chi_d = t.chi_d.data();
  t.tr.beta = t.beta.data();
  t.tr.lambda = t.lambda.data();
  t.tr.step_type = t.type.data();
  t.tr.step_insert = t.ins.data();
  t.tr.step_remove = t.rem.data();
  t.tr.step_source = t.src.data();
  return t;
}

void fill_stats(const doma_report & r, bool converged, std::vector<uint32_t> & counts,
                SolveStats & stats);

// DOMA's solveTransient through the C ABI (the per-step file output is the
// callback's); the mesh gets the flux the solve ended with.
bool run_transient(doma_solver * s, const doma_transient & tr, doma_step_callback cb, void * user,
                   size_t flux_values, std::vector<double> & flux, SolveStats & stats)
{
  std::vector<uint32_t> counts(1u << 20);
  doma_report r{};
  r.si_counts = counts.data();
  r.si_counts_capacity = counts.size();
  const doma_status st = doma_solver_solve_transient(s, &tr, cb, user, &r);
  if (st != DOMA_OK && st != DOMA_NOT_CONVERGED)
    throw std::runtime_error(std::string("transient solve failed: ") + doma_last_error());
  flux.resize(flux_values);
  if (doma_solver_get_scalar_flux(s, flux.data(), flux.size()) != DOMA_OK)
    throw std::runtime_error(std::string("reading the scalar flux failed: ") + doma_last_error());
  fill_stats(r, st == DOMA_OK, counts, stats);
  return stats.converged;
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

// DOMA's TransportSolver3D::solveTransient (src/TransportSolver3D.cpp:88-140 in 3D).
template <typename T>
bool TransportSolver3D<T>::solveTransient(const std::string & output_file_base)
{
  const ProblemData d = gather(_params, _mesh.cellBlocks());
  const TransientData td = gather_transient(_params, d.ids);
  doma_solver * s = solver();
  const size_t N = _mesh.numCells(), D = td.tr.num_d_groups;
  _mesh._cell_d.resize(N);
  for (size_t c = 0; c < N; ++c) _mesh._cell_d[c] = td.dg[d.cell_material[c]];
  _mesh._dnps.assign(D * N, 0.0);
  _step_base = output_file_base;
  if (output_file_base != "") {
    std::fill(_mesh._flux.begin(), _mesh._flux.end(), 0.0);
    _mesh.dumpToTextFile(output_file_base);  // the initial condition
  }
  return run_transient(s, td.tr, &TransportSolver3D<T>::stepDone, this, _mesh._flux.size(),
                       _mesh._flux, _stats);
}

template <typename T>
int TransportSolver3D<T>::stepDone(void * user, uint32_t step, double /*t*/, const double * phi,
                                     const double * dnps)
{
  auto * self = static_cast<TransportSolver3D<T> *>(user);
  BrickMesh3D & mesh = self->_mesh;
  std::copy(phi, phi + mesh._flux.size(), mesh._flux.begin());
  if (dnps) std::copy(dnps, dnps + mesh._dnps.size(), mesh._dnps.begin());
  if (self->_step_base != "") {
    const std::string name = self->_step_base + "_t" + std::to_string(step);
    mesh.dumpToTextFile(name, true);
    mesh.dumpDNPsToTextFile(name);
  }
  return 0;
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

// DOMA's TransportSolver2D::solveTransient (src/TransportSolver2D.cpp:88-140 in 3D).
template <typename T>
bool TransportSolver2D<T>::solveTransient(const std::string & output_file_base)
{
  const ProblemData d = gather(_params, _mesh.cellBlocks());
  const TransientData td = gather_transient(_params, d.ids);
  doma_solver * s = solver();
  const size_t N = _mesh.numCells(), D = td.tr.num_d_groups;
  _mesh._cell_d.resize(N);
  for (size_t c = 0; c < N; ++c) _mesh._cell_d[c] = td.dg[d.cell_material[c]];
  _mesh._dnps.assign(D * N, 0.0);
  _step_base = output_file_base;
  if (output_file_base != "") {
    std::fill(_mesh._flux.begin(), _mesh._flux.end(), 0.0);
    _mesh.dumpToTextFile(output_file_base);  // the initial condition
  }
  return run_transient(s, td.tr, &TransportSolver2D<T>::stepDone, this, _mesh._flux.size(),
                       _mesh._flux, _stats);
}

template <typename T>
int TransportSolver2D<T>::stepDone(void * user, uint32_t step, double /*t*/, const double * phi,
                                     const double * dnps)
{
  auto * self = static_cast<TransportSolver2D<T> *>(user);
  BrickMesh2D & mesh = self->_mesh;
  std::copy(phi, phi + mesh._flux.size(), mesh._flux.begin());
  if (dnps) std::copy(dnps, dnps + mesh._dnps.size(), mesh._dnps.begin());
  if (self->_step_base != "") {
    const std::string name = self->_step_base + "_t" + std::to_string(step);
    mesh.dumpToTextFile(name, true);
    mesh.dumpDNPsToTextFile(name);
  }
  return 0;
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
