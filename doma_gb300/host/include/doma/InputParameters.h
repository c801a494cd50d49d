// InputParameters.h -- the parsed <doma_inp> deck.
//
// Field names, meanings and containers match DOMA's InputParameters and
// MaterialProps (DOMA include/InputParameters.h:10-119), so a caller that
// fills the struct in code, or reads a deck with parseInputParameters, can
// switch libraries without changes.  Two optional <solver> attributes that
// DOMA ignores are added: theta="..." (TW-DD theta, DOMA's constant 0.9 by
// default) and precision="fp64|fp32".  Errors throw std::runtime_error with
// DOMA's message instead of exiting the process.
#pragma once

#include <string>
#include <unordered_map>
#include <vector>

#include "TransportBase.h"

struct SourceStep
{
  StepType _type = StepType::Both;
  double _insert_time = 0.0;
  double _remove_time = 0.0;
  std::vector<double> _g_src;
};

struct MaterialProps
{
  std::vector<double> _g_total;
  std::vector<double> _g_prod;
  std::vector<double> _g_chi_p;
  std::vector<double> _g_inv_v;
  std::vector<double> _g_g_scatter_mat;  // [to * G + from]
  std::vector<double> _g_src;
  unsigned int _num_d_groups = 0u;
  std::vector<double> _n_g_chi_d;
  std::vector<double> _g_n_beta;
  std::vector<double> _n_lambda;
};

struct InputParameters
{
  RunMode _mode = RunMode::FixedSrc;
  unsigned int _num_e_groups = 0u;
  double _t0 = 0.0;
  double _t1 = 0.0;
  unsigned int _num_steps = 1u;
  TransientIC _ic = TransientIC::Zero;
  double _src_it_tol = 1e-8;
  double _gs_tol = 1e-8;
  double _k_tol = 1e-5;
  bool _dsa = false;
  unsigned int _num_src_it = 1000u;
  unsigned int _num_mg_it = 100u;
  unsigned int _num_polar = 1u;
  unsigned int _num_azimuthal = 1u;
  EquationType _eq_type = EquationType::DD;
  unsigned int _num_dims = 3u;
  unsigned int _refinement = 0u;
  std::vector<unsigned int> _x_intervals;
  std::vector<unsigned int> _y_intervals;
  std::vector<unsigned int> _z_intervals;
  std::vector<double> _dx;
  std::vector<double> _dy;
  std::vector<double> _dz;
  std::vector<unsigned int> _blocks;
  std::unordered_map<CertesianFaceSide, BoundaryCondition> _bcs;
  std::unordered_map<unsigned int, MaterialProps> _block_mat_info;
  std::unordered_map<unsigned int, SourceStep> _block_step_src;

  // GPU additions (optional in decks).
  double _theta = 0.9;
  SweepPrecision _precision = SweepPrecision::FP64;
};

// Read a <doma_inp> deck (DOMA src/InputParameters.cpp:92-524).
InputParameters parseInputParameters(const std::string & file_path);
// Same, from the XML text itself.
InputParameters parseInputParametersFromString(const std::string & xml_text);

// DOMA's comma-separated list readers (src/InputParameters.cpp:9-49).
void parseVecFromString(const std::string & str, std::vector<double> & res);
void parseVecFromString(const std::string & str, std::vector<unsigned int> & res);
