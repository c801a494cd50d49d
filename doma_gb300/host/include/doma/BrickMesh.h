// BrickMesh.h -- tensor-product Cartesian meshes with DOMA's public interface.
//
// BrickMesh3D / BrickMesh2D keep DOMA's constructor, validateProps,
// fluxAtPoint and dumpToTextFile (DOMA include/BrickMesh3D.h:17-30,
// include/BrickMesh2D.h), the cell numbering (x fastest) and the text output
// layout, so post-processing scripts that read DOMA's files keep working.
// Storage is this library's: per-axis cell widths, a block id per cell and
// the scalar flux as one [G][N] array (structure of arrays) that the GPU
// solver fills in a single copy.
#pragma once

#include <array>
#include <string>
#include <vector>

#include "InputParameters.h"

template <typename T>
class TransportSolver3D;
template <typename T>
class TransportSolver2D;

class BrickMesh3D
{
public:
  BrickMesh3D(const InputParameters & params, const std::array<BoundaryCondition, 6u> & bcs,
              unsigned int num_threads);

  // Every block id on the mesh has material properties (throws otherwise).
  void validateProps();

  // Scalar flux of group g in the cell containing (x, y, z); false if the
  // point is not on the mesh.
  bool fluxAtPoint(const double & x, const double & y, const double & z, unsigned int g,
                   double & returned_flux) const;

  // <base>_dims.txt, _blocks.txt, _meshx/y/z.txt and _g<g>_flux.txt.
  void dumpToTextFile(const std::string & file_name, bool only_flux = false);
  // <base>_d<d>_dnps.txt for each delayed group d below the most that any
  // cell's material has; a cell whose material has fewer prints 0
  // (DOMA src/BrickMesh3D.cpp:273-295).
  void dumpDNPsToTextFile(const std::string & file_name);

  unsigned int numX() const { return _tot_num_x; }
  unsigned int numY() const { return _tot_num_y; }
  unsigned int numZ() const { return _tot_num_z; }
  size_t numCells() const { return _block_of_cell.size(); }
  unsigned int numGroups() const { return _num_groups; }
  const std::vector<double> & widthsX() const { return _wx; }
  const std::vector<double> & widthsY() const { return _wy; }
  const std::vector<double> & widthsZ() const { return _wz; }
  const std::vector<unsigned int> & cellBlocks() const { return _block_of_cell; }
  // [g * numCells() + cell]
  const std::vector<double> & scalarFlux() const { return _flux; }
  // [d * numCells() + cell] precursors after the last transient step
  const std::vector<double> & precursors() const { return _dnps; }
  // Replace the scalar flux ([G][N]; throws on a size mismatch).
  void setScalarFlux(const std::vector<double> & flux);

private:
  template <typename T>
  friend class TransportSolver3D;

  unsigned int _tot_num_x = 0, _tot_num_y = 0, _tot_num_z = 0;
  unsigned int _num_groups = 0;
  std::vector<double> _wx, _wy, _wz;      // cell widths per axis
  std::vector<double> _cx, _cy, _cz;      // cell centres per axis, as DOMA accumulates them
  std::vector<unsigned int> _block_of_cell;
  std::array<BoundaryCondition, 6u> _bcs;
  const InputParameters & _params;
  unsigned int _num_threads;
  std::vector<double> _flux;
  std::vector<double> _dnps;             // [D][N] precursor concentrations (transients)
  std::vector<unsigned int> _cell_d;     // [N] delayed groups of each cell's material
};

class BrickMesh2D
{
public:
  BrickMesh2D(const InputParameters & params, const std::array<BoundaryCondition, 4u> & bcs,
              unsigned int num_threads);

  void validateProps();
  bool fluxAtPoint(const double & x, const double & y, unsigned int g, double & returned_flux) const;
  void dumpToTextFile(const std::string & file_name, bool only_flux = false);
  void dumpDNPsToTextFile(const std::string & file_name);

  unsigned int numX() const { return _tot_num_x; }
  unsigned int numY() const { return _tot_num_y; }
  size_t numCells() const { return _block_of_cell.size(); }
  unsigned int numGroups() const { return _num_groups; }
  const std::vector<double> & widthsX() const { return _wx; }
  const std::vector<double> & widthsY() const { return _wy; }
  const std::vector<unsigned int> & cellBlocks() const { return _block_of_cell; }
  const std::vector<double> & scalarFlux() const { return _flux; }
  const std::vector<double> & precursors() const { return _dnps; }
  void setScalarFlux(const std::vector<double> & flux);

private:
  template <typename T>
  friend class TransportSolver2D;

  unsigned int _tot_num_x = 0, _tot_num_y = 0;
  unsigned int _num_groups = 0;
  std::vector<double> _wx, _wy;
  std::vector<double> _cx, _cy;
  std::vector<unsigned int> _block_of_cell;
  std::array<BoundaryCondition, 4u> _bcs;
  const InputParameters & _params;
  unsigned int _num_threads;
  std::vector<double> _flux;
  std::vector<double> _dnps;             // [D][N] precursor concentrations (transients)
  std::vector<unsigned int> _cell_d;     // [N] delayed groups of each cell's material
};
