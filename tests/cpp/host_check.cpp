// host_check.cpp -- test driver for the C++ drop-in layer (built by the tests).
//
//   host_check parse <deck>                      summary of the parsed deck (JSON)
//   host_check dump  <deck> <flux.bin> <base>    mesh from the deck, flux [G][N] from a
//                                                raw float64 file, DOMA-layout text output
//   host_check point <deck> <flux.bin> x y [z] g fluxAtPoint
//   host_check solve <deck> <flux.bin> [verbose|quiet] [base]
//                                                drop-in solver on the GPU (the deck's
//                                                mode; a fixed-source solve writes DOMA's
//                                                text output and a transient its step
//                                                files under base); writes the flux and
//                                                prints SI counts (JSON)
#include <array>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <map>
#include <string>
#include <vector>

#include "doma/BrickMesh.h"
#include "doma/InputParameters.h"
#include "doma/TransportSolver.h"

static std::vector<double> read_bin(const std::string & path)
{
  std::ifstream f(path, std::ios::binary);
  f.seekg(0, std::ios::end);
  const size_t n = (size_t)f.tellg() / sizeof(double);
  f.seekg(0);
  std::vector<double> v(n);
  f.read(reinterpret_cast<char *>(v.data()), n * sizeof(double));
  return v;
}

static void write_bin(const std::string & path, const std::vector<double> & v)
{
  std::ofstream f(path, std::ios::binary);
  f.write(reinterpret_cast<const char *>(v.data()), v.size() * sizeof(double));
}

template <typename V>
static void json_list(const V & v)
{
  std::cout << "[";
  for (size_t i = 0; i < v.size(); ++i) std::cout << (i ? ", " : "") << v[i];
  std::cout << "]";
}

int main(int argc, char ** argv)
{
  if (argc < 3) return 2;
  const std::string cmd = argv[1];
  try {
    const InputParameters p = parseInputParameters(argv[2]);
    if (cmd == "parse") {
      std::cout.precision(17);
      std::cout << "{\"mode\": " << (int)p._mode << ", \"scheme\": " << (int)p._eq_type
                << ", \"groups\": " << p._num_e_groups << ", \"fs_tol\": " << p._src_it_tol
                << ", \"fs_max_it\": " << p._num_src_it << ", \"mg_tol\": " << p._gs_tol
                << ", \"mg_max_it\": " << p._num_mg_it << ", \"np\": " << p._num_polar
                << ", \"na\": " << p._num_azimuthal << ", \"dims\": " << p._num_dims
                << ", \"refinement\": " << p._refinement << ", \"theta\": " << p._theta
                << ", \"precision\": " << (int)p._precision << ", \"dx\": ";
      json_list(p._dx);
      std::cout << ", \"dy\": ";
      json_list(p._dy);
      std::cout << ", \"dz\": ";
      json_list(p._dz);
      std::cout << ", \"ix\": ";
      json_list(p._x_intervals);
      std::cout << ", \"iy\": ";
      json_list(p._y_intervals);
      std::cout << ", \"iz\": ";
      json_list(p._z_intervals);
      std::cout << ", \"k_tol\": " << p._k_tol;
      std::cout << ", \"blocks\": ";
      json_list(p._blocks);
      std::cout << ", \"materials\": {";
      std::map<unsigned, const MaterialProps *> sorted;
      for (const auto & kv : p._block_mat_info) sorted[kv.first] = &kv.second;
      bool first = true;
      for (const auto & kv : sorted) {
        std::cout << (first ? "" : ", ") << "\"" << kv.first << "\": {\"total\": ";
        json_list(kv.second->_g_total);
        std::cout << ", \"scatter\": ";
        json_list(kv.second->_g_g_scatter_mat);
        std::cout << ", \"source\": ";
        json_list(kv.second->_g_src);
        std::cout << ", \"chi_p\": ";
        json_list(kv.second->_g_chi_p);
        std::cout << ", \"prod\": ";
        json_list(kv.second->_g_prod);
        std::cout << ", \"delayed_groups\": " << kv.second->_num_d_groups << ", \"inv_v\": ";
        json_list(kv.second->_g_inv_v);
        std::cout << ", \"chi_d\": ";
        json_list(kv.second->_n_g_chi_d);
        std::cout << ", \"beta\": ";
        json_list(kv.second->_g_n_beta);
        std::cout << ", \"lambda\": ";
        json_list(kv.second->_n_lambda);
        std::cout << "}";
        first = false;
      }
      std::cout << "}, \"t0\": " << p._t0 << ", \"t1\": " << p._t1 << ", \"t_steps\": "
                << p._num_steps << ", \"ic\": " << (int)p._ic << ", \"steps\": {";
      std::map<unsigned, const SourceStep *> steps;
      for (const auto & kv : p._block_step_src) steps[kv.first] = &kv.second;
      first = true;
      for (const auto & kv : steps) {
        std::cout << (first ? "" : ", ") << "\"" << kv.first << "\": {\"type\": "
                  << (int)kv.second->_type << ", \"insert\": " << kv.second->_insert_time
                  << ", \"remove\": " << kv.second->_remove_time << ", \"source\": ";
        json_list(kv.second->_g_src);
        std::cout << "}";
        first = false;
      }
      std::cout << "}}" << std::endl;
      return 0;
    }
    if (p._num_dims == 3) {
      std::array<BoundaryCondition, 6u> bcs;
      bcs.fill(BoundaryCondition::Vacuum);
      BrickMesh3D mesh(p, bcs, 1);
      mesh.validateProps();
      if (cmd == "dump") {
        mesh.setScalarFlux(read_bin(argv[3]));
        mesh.dumpToTextFile(argv[4]);
        return 0;
      }
      if (cmd == "point") {
        mesh.setScalarFlux(read_bin(argv[3]));
        double v = 0;
        const bool ok = mesh.fluxAtPoint(atof(argv[4]), atof(argv[5]), atof(argv[6]), atoi(argv[7]), v);
        std::printf("{\"found\": %s, \"flux\": %.17g}\n", ok ? "true" : "false", v);
        return 0;
      }
      if (cmd == "solve") {
        const bool verbose = argc > 4 && std::string(argv[4]) == "verbose";
        bool ok;
        SolveStats st;
        const bool eigen = p._mode == RunMode::Eigen;
        const bool transient = p._mode == RunMode::Transient;
        const std::string base = argc > 5 ? argv[5] : "";
        double k = 0.0;
        if (p._eq_type == EquationType::DD) {
          DDTransportSolver3D s(mesh, p, verbose, 1);
          ok = transient ? s.solveTransient(base) : eigen ? s.solveEigenvalue() : s.solveFixedSource(base);
          st = s.stats();
          k = s.eigenvalue();
        } else {
          TWDDTransportSolver3D s(mesh, p, verbose, 1);
          ok = transient ? s.solveTransient(base) : eigen ? s.solveEigenvalue() : s.solveFixedSource(base);
          st = s.stats();
          k = s.eigenvalue();
        }
        write_bin(argv[3], mesh.scalarFlux());
        char kbuf[64];
        std::snprintf(kbuf, sizeof kbuf, "%.17g", k);
        std::cout << "{\"converged\": " << (ok ? "true" : "false") << ", \"mg\": " << st.mg_iterations
                  << ", \"k\": " << kbuf << ", \"si_counts\": ";
        json_list(st.si_counts);
        std::cout << "}" << std::endl;
        return 0;
      }
    } else {
      std::array<BoundaryCondition, 4u> bcs;
      bcs.fill(BoundaryCondition::Vacuum);
      BrickMesh2D mesh(p, bcs, 1);
      mesh.validateProps();
      if (cmd == "dump") {
        mesh.setScalarFlux(read_bin(argv[3]));
        mesh.dumpToTextFile(argv[4]);
        return 0;
      }
      if (cmd == "point") {
        mesh.setScalarFlux(read_bin(argv[3]));
        double v = 0;
        const bool ok = mesh.fluxAtPoint(atof(argv[4]), atof(argv[5]), atoi(argv[6]), v);
        std::printf("{\"found\": %s, \"flux\": %.17g}\n", ok ? "true" : "false", v);
        return 0;
      }
      if (cmd == "solve") {
        const bool verbose = argc > 4 && std::string(argv[4]) == "verbose";
        bool ok;
        SolveStats st;
        const bool eigen = p._mode == RunMode::Eigen;
        const bool transient = p._mode == RunMode::Transient;
        const std::string base = argc > 5 ? argv[5] : "";
        double k = 0.0;
        if (p._eq_type == EquationType::DD) {
          DDTransportSolver2D s(mesh, p, verbose, 1);
          ok = transient ? s.solveTransient(base) : eigen ? s.solveEigenvalue() : s.solveFixedSource(base);
          st = s.stats();
          k = s.eigenvalue();
        } else {
          TWDDTransportSolver2D s(mesh, p, verbose, 1);
          ok = transient ? s.solveTransient(base) : eigen ? s.solveEigenvalue() : s.solveFixedSource(base);
          st = s.stats();
          k = s.eigenvalue();
        }
        write_bin(argv[3], mesh.scalarFlux());
        char kbuf[64];
        std::snprintf(kbuf, sizeof kbuf, "%.17g", k);
        std::cout << "{\"converged\": " << (ok ? "true" : "false") << ", \"mg\": " << st.mg_iterations
                  << ", \"k\": " << kbuf << ", \"si_counts\": ";
        json_list(st.si_counts);
        std::cout << "}" << std::endl;
        return 0;
      }
    }
  } catch (const std::exception & e) {
    std::cerr << e.what() << std::endl;
    return 1;
  }
  return 2;
}
