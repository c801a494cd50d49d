// doma_main.cpp -- command-line runner for <doma_inp> decks on the GPU.
//
// Same flags as DOMA's driver (src/main.cpp:20-30): -i/--input_file <deck>,
// -n/--n-threads <T> (accepted; the device does the work) and --verbose.
// 2D and 3D fixed-source, eigenvalue and transient decks are solved through
// the drop-in TransportSolver2D/3D; output goes next to the deck as
// <dir>/<stem>_* text files, and the run ends with DOMA's "Time elapsed: <s>
// (s)." line.  Like DOMA, a solve that hits an iteration cap still exits 0
// (after DOMA's failure message); --strict makes it exit 3 instead.  1D decks
// and transients with a steady-state start exit 1 with a message.
#include <chrono>
#include <cstdlib>
#include <cstring>
#include <filesystem>
#include <iostream>
#include <string>

#include "doma/BrickMesh.h"
#include "doma/InputParameters.h"
#include "doma/TransportSolver.h"

namespace {

void usage(const char * argv0)
{
  std::cerr << "Usage: " << argv0 << " -i <input_file> [-n <threads>] [--verbose] [--strict]\n"
            << "Discrete Ordinates Mini-App, fixed-source, eigenvalue and transient paths on the GPU.\n";
}

template <typename Solver, typename Mesh>
int run(Mesh & mesh, const InputParameters & params, bool verbose, unsigned threads,
        const std::string & base, bool strict,
        const std::chrono::high_resolution_clock::time_point & start)
{
  Solver solver(mesh, params, verbose, threads);
  bool ok = false;
  const char * done = "Fixed source solver finished executing.";
  if (params._mode == RunMode::Eigen) {
    ok = solver.solveEigenvalue(base);
    done = "Eigenvalue solver finished executing.";
  } else if (params._mode == RunMode::Transient) {
    ok = solver.solveTransient(base);
    done = "Transient solver finished executing.";
  } else {
    ok = solver.solveFixedSource(base);
  }
  if (ok) {
    std::cout << done << std::endl;
    const auto stop = std::chrono::high_resolution_clock::now();
    std::cout << "Time elapsed: " << std::chrono::duration_cast<std::chrono::seconds>(stop - start).count()
              << " (s)." << std::endl;
    return 0;
  }
  return strict ? 3 : 0;
}

}  // namespace

int main(int argc, char ** argv)
{
  std::string input;
  int threads = 1;
  bool verbose = false, strict = false;
  for (int a = 1; a < argc; ++a) {
    const std::string s = argv[a];
    if ((s == "-i" || s == "--input_file") && a + 1 < argc) input = argv[++a];
    else if ((s == "-n" || s == "--n-threads") && a + 1 < argc) threads = std::atoi(argv[++a]);
    else if (s == "--verbose") verbose = true;
    else if (s == "--strict") strict = true;
    else if (s == "-h" || s == "--help") { usage(argv[0]); return 0; }
    else { std::cerr << "Unknown argument: " << s << "\n"; usage(argv[0]); return 1; }
  }
  if (input.empty()) {
    std::cerr << "-i: required.\n";
    usage(argv[0]);
    return 1;
  }
  try {
    const std::filesystem::path path(input);
    const InputParameters params = parseInputParameters(path.string());
    const std::string base = (path.parent_path() / path.stem()).string();
    const auto start = std::chrono::high_resolution_clock::now();
    if (params._num_dims == 3) {
      std::array<BoundaryCondition, 6u> bcs;
      bcs.fill(BoundaryCondition::Vacuum);
      BrickMesh3D mesh(params, bcs, (unsigned)threads);
      mesh.validateProps();
      if (params._eq_type == EquationType::DD)
        return run<DDTransportSolver3D>(mesh, params, verbose, threads, base, strict, start);
      return run<TWDDTransportSolver3D>(mesh, params, verbose, threads, base, strict, start);
    }
    if (params._num_dims == 2) {
      std::array<BoundaryCondition, 4u> bcs;
      bcs.fill(BoundaryCondition::Vacuum);
      BrickMesh2D mesh(params, bcs, (unsigned)threads);
      mesh.validateProps();
      if (params._eq_type == EquationType::DD)
        return run<DDTransportSolver2D>(mesh, params, verbose, threads, base, strict, start);
      return run<TWDDTransportSolver2D>(mesh, params, verbose, threads, base, strict, start);
    }
    std::cerr << "Invalid number of dimensions: " << params._num_dims
              << " (the GPU library runs 2D and 3D decks)" << std::endl;
    return 1;
  } catch (const std::exception & e) {
    std::cerr << e.what() << std::endl;
    return 1;
  }
}
