// TransportSolver.h -- drop-in TransportSolver3D<T> / TransportSolver2D<T>
// running DOMA's fixed-source path on the GPU.
//
// Same constructor, solveFixedSource / solveEigenvalue signatures, return
// convention and typedef names as DOMA (DOMA include/TransportSolver3D.h:12-34,
// include/TransportSolver2D.h), so `DDTransportSolver3D s(mesh, params,
// verbose, threads); s.solveFixedSource(base);` works unchanged.  T selects
// the cell balance: DiamondDifference3D/2D or TWDiamondDifference3D/2D (the
// policy classes of DOMA's include/DiamondDifference3D.h and
// include/TWDiamondDifference3D.h; here they are tags, the arithmetic lives
// in the GPU library).  Underneath, every call goes through the C ABI of
// include/doma_gb300.h.
//
// Behaviour as in DOMA: the solves return false when an iteration cap is
// reached (the flux of the last iterate is kept in the mesh), print DOMA's
// progress lines (each SI residual too when verbose), write the text output
// when output_file_base is not empty and the solve converged.  eigenvalue()
// gives k after solveEigenvalue (DOMA keeps it private).  solveTransient
// (DOMA src/TransportSolver3D.cpp:88-140) writes the zero initial condition
// as <base>_* files, then after each step <base>_t<step>_g<g>_flux.txt and
// <base>_t<step>_d<d>_dnps.txt, and returns false as soon as a step's solve
// reaches a cap; the mesh keeps the last step's flux and precursors.
// Differences: invalid input and CUDA failures throw std::runtime_error
// instead of exiting; num_threads is accepted and unused (the device does
// the work); transients start from zero only (DOMA's steady-state start
// reads its previous-step and precursor arrays before sizing them) and
// write no files when output_file_base is empty.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "BrickMesh.h"
#include "InputParameters.h"

struct doma_solver;

struct DiamondDifference3D { static constexpr unsigned int scheme = 0u; };
struct TWDiamondDifference3D { static constexpr unsigned int scheme = 1u; };
struct DiamondDifference2D { static constexpr unsigned int scheme = 0u; };
struct TWDiamondDifference2D { static constexpr unsigned int scheme = 1u; };

// What the last solveFixedSource did.
struct SolveStats
{
  bool converged = false;
  unsigned int mg_iterations = 0;
  uint64_t source_iterations = 0;
  uint64_t updates = 0;
  double mg_residual = 0.0;
  double si_residual = 0.0;
  double solve_ms = 0.0;
  std::vector<uint32_t> si_counts;
};

template <typename T>
class TransportSolver3D;
typedef TransportSolver3D<TWDiamondDifference3D> TWDDTransportSolver3D;
typedef TransportSolver3D<DiamondDifference3D> DDTransportSolver3D;

template <typename T>
class TransportSolver3D
{
public:
  TransportSolver3D(BrickMesh3D & mesh, const InputParameters & params, bool verbose,
                    unsigned int num_threads);
  ~TransportSolver3D();
  TransportSolver3D(const TransportSolver3D &) = delete;
  TransportSolver3D & operator=(const TransportSolver3D &) = delete;

  bool solveFixedSource(const std::string & output_file_base = "", const double & t = 0.0);
  bool solveEigenvalue(const std::string & output_file_base = "");
  bool solveTransient(const std::string & output_file_base);

  const SolveStats & stats() const { return _stats; }
  double eigenvalue() const { return _k; }

private:
  doma_solver * solver();
  static int stepDone(void * user, uint32_t step, double t, const double * phi,
                      const double * dnps);

  BrickMesh3D & _mesh;
  std::string _step_base;
  const InputParameters & _params;
  const bool _verbose;
  doma_solver * _solver = nullptr;
  SolveStats _stats;
  double _k = 1.0;
};

template <typename T>
class TransportSolver2D;
typedef TransportSolver2D<TWDiamondDifference2D> TWDDTransportSolver2D;
typedef TransportSolver2D<DiamondDifference2D> DDTransportSolver2D;

template <typename T>
class TransportSolver2D
{
public:
  TransportSolver2D(BrickMesh2D & mesh, const InputParameters & params, bool verbose,
                    unsigned int num_threads);
  ~TransportSolver2D();
  TransportSolver2D(const TransportSolver2D &) = delete;
  TransportSolver2D & operator=(const TransportSolver2D &) = delete;

  bool solveFixedSource(const std::string & output_file_base = "", const double & t = 0.0);
  bool solveEigenvalue(const std::string & output_file_base = "");
  bool solveTransient(const std::string & output_file_base);

  const SolveStats & stats() const { return _stats; }
  double eigenvalue() const { return _k; }

private:
  doma_solver * solver();
  static int stepDone(void * user, uint32_t step, double t, const double * phi,
                      const double * dnps);

  BrickMesh2D & _mesh;
  std::string _step_base;
  const InputParameters & _params;
  const bool _verbose;
  doma_solver * _solver = nullptr;
  SolveStats _stats;
  double _k = 1.0;
};

extern template class TransportSolver3D<DiamondDifference3D>;
extern template class TransportSolver3D<TWDiamondDifference3D>;
extern template class TransportSolver2D<DiamondDifference2D>;
extern template class TransportSolver2D<TWDiamondDifference2D>;
