// BrickMesh.cpp -- mesh construction and text output (see BrickMesh.h).
//
// Construction follows DOMA's BrickMesh3D constructor
// (src/BrickMesh3D.cpp:8-102; 2D: src/BrickMesh2D.cpp:8-80): interval i of an
// axis holds n_i cells of width dx_i / n_i; the block id of each interval
// brick is expanded to its cells; cell centres start at half the first width
// and advance by each cell's own width (DOMA's accumulation, kept so that
// the written centres and fluxAtPoint agree with DOMA on graded meshes too).
// Output follows BrickMesh3D::dumpToTextFile (src/BrickMesh3D.cpp:217-271):
// "num_x: ..." lines in _dims.txt, one value per line elsewhere, six
// significant digits for coordinates and fluxes.
#include "doma/BrickMesh.h"

#include <algorithm>
#include <fstream>
#include <iomanip>
#include <stdexcept>

namespace {

void expand(const std::vector<unsigned int> & counts, const std::vector<double> & lengths,
            std::vector<double> & widths, std::vector<double> & centres)
{
  widths.clear();
  for (size_t i = 0; i < counts.size(); ++i) {
    const double w = lengths[i] / static_cast<double>(counts[i]);
    for (unsigned int j = 0; j < counts[i]; ++j) widths.push_back(w);
  }
  centres.resize(widths.size());
  if (widths.empty()) return;
  double c = 0.5 * widths[0];
  for (size_t i = 0; i < widths.size(); ++i) {
    centres[i] = c;
    c += widths[i];
  }
}

unsigned int total(const std::vector<unsigned int> & v)
{
  unsigned int t = 0;
  for (auto x : v) t += x;
  return t;
}

void check_axis(const std::vector<unsigned int> & counts, const std::vector<double> & lengths, const char * axis)
{
  if (counts.size() != lengths.size())
    throw std::runtime_error(std::string("Error: the ") + axis +
                             " interval counts and lengths differ in size!");
  for (auto c : counts)
    if (c == 0) throw std::runtime_error(std::string("Error: an ") + axis + " interval has no cells!");
}

// Shared by both meshes: DOMA's dumpDNPsToTextFile.
void dump_dnps(const std::string & file_name, const std::vector<double> & dnps,
               const std::vector<unsigned int> & cell_d, size_t N)
{
  unsigned int D = 0;
  for (unsigned int d : cell_d) D = std::max(D, d);
  for (unsigned int d = 0; d < D; ++d) {
    std::ofstream out(file_name + "_d" + std::to_string(d) + "_dnps.txt", std::ofstream::out);
    out << std::setprecision(6);
    for (size_t c = 0; c < N; ++c) {
      if (cell_d[c] == D && (size_t)d * N + c < dnps.size())
        out << dnps[(size_t)d * N + c] << std::endl;
      else
        out << 0.0 << std::endl;
    }
  }
}

}  // namespace

// ---------------------------------------------------------------------------
BrickMesh3D::BrickMesh3D(const InputParameters & params, const std::array<BoundaryCondition, 6u> & bcs,
                         unsigned int num_threads)
  : _bcs(bcs), _params(params), _num_threads(num_threads)
{
  const auto & nx = params._x_intervals;
  const auto & ny = params._y_intervals;
  const auto & nz = params._z_intervals;
  if (nx.size() * ny.size() * nz.size() != params._blocks.size())
    throw std::runtime_error("Error: The blocks vector is not equal to the number of subdivisions!");
  check_axis(nx, params._dx, "x");
  check_axis(ny, params._dy, "y");
  check_axis(nz, params._dz, "z");
  _tot_num_x = total(nx);
  _tot_num_y = total(ny);
  _tot_num_z = total(nz);
  expand(nx, params._dx, _wx, _cx);
  expand(ny, params._dy, _wy, _cy);
  expand(nz, params._dz, _wz, _cz);
  _block_of_cell.reserve((size_t)_tot_num_x * _tot_num_y * _tot_num_z);
  for (size_t k = 0; k < nz.size(); ++k)
    for (unsigned int kk = 0; kk < nz[k]; ++kk)
      for (size_t j = 0; j < ny.size(); ++j)
        for (unsigned int jj = 0; jj < ny[j]; ++jj)
          for (size_t i = 0; i < nx.size(); ++i)
            for (unsigned int ii = 0; ii < nx[i]; ++ii)
              _block_of_cell.push_back(params._blocks[(k * ny.size() + j) * nx.size() + i]);
  _num_groups = params._num_e_groups;
  _flux.assign((size_t)_num_groups * _block_of_cell.size(), 0.0);
}

void BrickMesh3D::validateProps()
{
  for (auto b : _block_of_cell)
    if (_params._block_mat_info.count(b) == 0)
      throw std::runtime_error("Block " + std::to_string(b) +
                               " (defined on the mesh) has no material properties!");
}

bool BrickMesh3D::fluxAtPoint(const double & x, const double & y, const double & z, unsigned int g,
                              double & returned_flux) const
{
  // Same containment test and scan order as DOMA (CartesianCell3D::pointInCell).
  const size_t N = numCells();
  for (unsigned int k = 0; k < _tot_num_z; ++k)
    for (unsigned int j = 0; j < _tot_num_y; ++j)
      for (unsigned int i = 0; i < _tot_num_x; ++i) {
        const bool in_x = (_cx[i] - 0.5 * _wx[i]) <= x && (_cx[i] + 0.5 * _wx[i]) >= x;
        const bool in_y = (_cy[j] - 0.5 * _wy[j]) <= y && (_cy[j] + 0.5 * _wy[j]) >= y;
        const bool in_z = (_cz[k] - 0.5 * _wz[k]) <= z && (_cz[k] + 0.5 * _wz[k]) >= z;
        if (in_x && in_y && in_z) {
          returned_flux = _flux[(size_t)g * N + ((size_t)k * _tot_num_y + j) * _tot_num_x + i];
          return true;
        }
      }
  return false;
}

void BrickMesh3D::dumpToTextFile(const std::string & file_name, bool only_flux)
{
  const size_t N = numCells();
  if (!only_flux) {
    std::ofstream dims(file_name + "_dims.txt", std::ofstream::out);
    dims << "num_x: " << _tot_num_x << std::endl;
    dims << "num_y: " << _tot_num_y << std::endl;
    dims << "num_z: " << _tot_num_z << std::endl;
    dims << "num_g: " << _num_groups << std::endl;
    std::ofstream blocks(file_name + "_blocks.txt", std::ofstream::out);
    std::ofstream x(file_name + "_meshx.txt", std::ofstream::out);
    std::ofstream y(file_name + "_meshy.txt", std::ofstream::out);
    std::ofstream z(file_name + "_meshz.txt", std::ofstream::out);
    x << std::setprecision(6);
    y << std::setprecision(6);
    z << std::setprecision(6);
    if (_num_groups > 0)
      for (unsigned int k = 0; k < _tot_num_z; ++k)
        for (unsigned int j = 0; j < _tot_num_y; ++j)
          for (unsigned int i = 0; i < _tot_num_x; ++i) {
            x << _cx[i] << std::endl;
            y << _cy[j] << std::endl;
            z << _cz[k] << std::endl;
            blocks << _block_of_cell[((size_t)k * _tot_num_y + j) * _tot_num_x + i] << std::endl;
          }
  }
  for (unsigned int g = 0; g < _num_groups; ++g) {
    std::ofstream flux(file_name + "_g" + std::to_string(g) + "_flux.txt", std::ofstream::out);
    flux << std::setprecision(6);
    for (size_t c = 0; c < N; ++c) flux << _flux[(size_t)g * N + c] << std::endl;
  }
}

void BrickMesh3D::setScalarFlux(const std::vector<double> & flux)
{
  if (flux.size() != _flux.size()) throw std::runtime_error("scalar flux size mismatch");
  _flux = flux;
}

// ---------------------------------------------------------------------------
BrickMesh2D::BrickMesh2D(const InputParameters & params, const std::array<BoundaryCondition, 4u> & bcs,
                         unsigned int num_threads)
  : _bcs(bcs), _params(params), _num_threads(num_threads)
{
  const auto & nx = params._x_intervals;
  const auto & ny = params._y_intervals;
  if (nx.size() * ny.size() != params._blocks.size())
    throw std::runtime_error("Error: The blocks vector is not equal to the number of subdivisions!");
  check_axis(nx, params._dx, "x");
  check_axis(ny, params._dy, "y");
  _tot_num_x = total(nx);
  _tot_num_y = total(ny);
  expand(nx, params._dx, _wx, _cx);
  expand(ny, params._dy, _wy, _cy);
  _block_of_cell.reserve((size_t)_tot_num_x * _tot_num_y);
  for (size_t j = 0; j < ny.size(); ++j)
    for (unsigned int jj = 0; jj < ny[j]; ++jj)
      for (size_t i = 0; i < nx.size(); ++i)
        for (unsigned int ii = 0; ii < nx[i]; ++ii)
          _block_of_cell.push_back(params._blocks[j * nx.size() + i]);
  _num_groups = params._num_e_groups;
  _flux.assign((size_t)_num_groups * _block_of_cell.size(), 0.0);
}

void BrickMesh2D::validateProps()
{
  for (auto b : _block_of_cell)
    if (_params._block_mat_info.count(b) == 0)
      throw std::runtime_error("Block " + std::to_string(b) +
                               " (defined on the mesh) has no material properties!");
}

bool BrickMesh2D::fluxAtPoint(const double & x, const double & y, unsigned int g, double & returned_flux) const
{
  const size_t N = numCells();
  for (unsigned int j = 0; j < _tot_num_y; ++j)
    for (unsigned int i = 0; i < _tot_num_x; ++i) {
      const bool in_x = (_cx[i] - 0.5 * _wx[i]) <= x && (_cx[i] + 0.5 * _wx[i]) >= x;
      const bool in_y = (_cy[j] - 0.5 * _wy[j]) <= y && (_cy[j] + 0.5 * _wy[j]) >= y;
      if (in_x && in_y) {
        returned_flux = _flux[(size_t)g * N + (size_t)j * _tot_num_x + i];
        return true;
      }
    }
  return false;
}

void BrickMesh2D::dumpToTextFile(const std::string & file_name, bool only_flux)
{
  const size_t N = numCells();
  if (!only_flux) {
    std::ofstream dims(file_name + "_dims.txt", std::ofstream::out);
    dims << "num_x: " << _tot_num_x << std::endl;
    dims << "num_y: " << _tot_num_y << std::endl;
    dims << "num_g: " << _num_groups << std::endl;
    std::ofstream blocks(file_name + "_blocks.txt", std::ofstream::out);
    std::ofstream x(file_name + "_meshx.txt", std::ofstream::out);
    std::ofstream y(file_name + "_meshy.txt", std::ofstream::out);
    x << std::setprecision(6);
    y << std::setprecision(6);
    if (_num_groups > 0)
      for (unsigned int j = 0; j < _tot_num_y; ++j)
        for (unsigned int i = 0; i < _tot_num_x; ++i) {
          x << _cx[i] << std::endl;
          y << _cy[j] << std::endl;
          blocks << _block_of_cell[(size_t)j * _tot_num_x + i] << std::endl;
        }
  }
  for (unsigned int g = 0; g < _num_groups; ++g) {
    std::ofstream flux(file_name + "_g" + std::to_string(g) + "_flux.txt", std::ofstream::out);
    flux << std::setprecision(6);
    for (size_t c = 0; c < N; ++c) flux << _flux[(size_t)g * N + c] << std::endl;
  }
}

void BrickMesh2D::setScalarFlux(const std::vector<double> & flux)
{
  if (flux.size() != _flux.size()) throw std::runtime_error("scalar flux size mismatch");
  _flux = flux;
}

void BrickMesh3D::dumpDNPsToTextFile(const std::string & file_name)
{
  dump_dnps(file_name, _dnps, _cell_d, numCells());
}

void BrickMesh2D::dumpDNPsToTextFile(const std::string & file_name)
{
  dump_dnps(file_name, _dnps, _cell_d, numCells());
}
