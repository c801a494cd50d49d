// InputParameters.cpp -- reader of DOMA's <doma_inp> decks.
//
// Follows DOMA's reader (src/InputParameters.cpp:92-524) element by element:
// <solver> (solve_type, scheme, num_groups, fs_tol, fs_max_it, mg_tol,
// mg_max_it, k_tol for eigen, t0/t1/t_steps/ics for transients, dsa),
// <angular_quad> (np, na), <mesh> (dims, refinement, dx/dy/dz, ix/iy/iz
// scaled by refinement + 1, blocks), <materials>/<mat block=...> with
// <reaction type=... mgxs=...> (scatter honours transpose="true"), and
// <transients>/<source_step>.  Numeric attributes are read the way pugixml's
// as_double / as_uint read them (strtod / strtoul, the default when absent),
// and the same validity checks produce the same messages, thrown as
// std::runtime_error.
#include "doma/InputParameters.h"

#include <algorithm>
#include <climits>
#include <cstdlib>
#include <stdexcept>

#include "xml.h"

using doma_host::XmlNode;

namespace {

[[noreturn]] void fail(const std::string & msg) { throw std::runtime_error(msg); }

double as_double(const XmlNode & n, const std::string & a, double dflt)
{
  bool found = false;
  const std::string v = n.attr(a, &found);
  if (!found) return dflt;
  return std::strtod(v.c_str(), nullptr);
}

unsigned int as_uint(const XmlNode & n, const std::string & a, unsigned int dflt)
{
  bool found = false;
  const std::string v = n.attr(a, &found);
  if (!found) return dflt;
  return static_cast<unsigned int>(std::strtoul(v.c_str(), nullptr, 10));
}

bool as_bool(const XmlNode & n, const std::string & a, bool dflt)
{
  bool found = false;
  const std::string v = n.attr(a, &found);
  if (!found || v.empty()) return dflt;
  // pugixml: true iff the first character is one of 1 t T y Y
  const char c = v[0];
  return c == '1' || c == 't' || c == 'T' || c == 'y' || c == 'Y';
}

double parseDoubleParam(const XmlNode & n, const std::string & name)
{
  const double v = as_double(n, name, -1.0);
  if (v >= 0.0) return v;
  fail("You must provide a valid param in " + name + "!");
}

unsigned int parseUintParam(const XmlNode & n, const std::string & name)
{
  if (as_uint(n, name, UINT_MAX) != UINT_MAX) return as_uint(n, name, 0u);
  fail("You must provide a valid param in " + name + "!");
}

std::string parseStringParam(const XmlNode & n, const std::string & name)
{
  const std::string v = n.attr(name);
  if (!v.empty()) return v;
  fail("You must provide a valid param in " + name + "!");
}

template <typename T, typename Conv>
void split_list(const std::string & str, std::vector<T> & res, Conv conv)
{
  std::string s = str;
  s.erase(std::remove(s.begin(), s.end(), ' '), s.end());
  s.erase(std::remove(s.begin(), s.end(), '\n'), s.end());
  size_t start = 0;
  for (;;) {
    const size_t comma = s.find(',', start);
    const std::string piece = s.substr(start, comma == std::string::npos ? std::string::npos : comma - start);
    try {
      res.emplace_back(conv(piece));
    } catch (const std::exception &) {
      fail("Invalid number '" + piece + "' in list \"" + str + "\"");
    }
    if (comma == std::string::npos) break;
    start = comma + 1;
  }
}

void check_count(const std::vector<double> & v, size_t want, bool allow_empty, const std::string & what,
                 const std::string & tag)
{
  if (v.size() == want || (allow_empty && v.empty())) return;
  fail("Not enough " + what + " have been provided! The simulation requires " + std::to_string(want) +
       " " + what + "; '" + tag + "' only provides " + std::to_string(v.size()) + ".");
}

InputParameters parse_document(const XmlNode & doc)
{
  const XmlNode * p = doc.child("doma_inp");
  if (!p) fail("A solver block has not been provided!");
  InputParameters params;

  // <solver>
  const XmlNode * s = p->child("solver");
  if (!s) fail("A solver block has not been provided!");
  params._dsa = s->attr("dsa") == "true";
  const std::string st = s->attr("solve_type");
  if (st == "steady") params._mode = RunMode::FixedSrc;
  else if (st == "eigen") params._mode = RunMode::Eigen;
  else if (st == "transient") params._mode = RunMode::Transient;
  else fail("Unknown run_mode " + st);
  const std::string sch = s->attr("scheme");
  if (sch == "dd") params._eq_type = EquationType::DD;
  else if (sch == "tw_dd") params._eq_type = EquationType::TW_DD;
  else fail("Unknown scheme " + sch);
  params._num_e_groups = parseUintParam(*s, "num_groups");
  params._src_it_tol = parseDoubleParam(*s, "fs_tol");
  params._num_src_it = parseUintParam(*s, "fs_max_it");
  params._gs_tol = parseDoubleParam(*s, "mg_tol");
  params._num_mg_it = parseUintParam(*s, "mg_max_it");
  if (params._mode == RunMode::Eigen) params._k_tol = parseDoubleParam(*s, "k_tol");
  if (params._mode == RunMode::Transient) {
    params._t0 = parseDoubleParam(*s, "t0");
    params._t1 = parseDoubleParam(*s, "t1");
    params._num_steps = parseUintParam(*s, "t_steps");
    const std::string ic = s->attr("ics");
    if (ic == "zero") params._ic = TransientIC::Zero;
    else if (ic == "steady") params._ic = TransientIC::SteadyState;
    else fail("Unknown initial condition " + ic);
  }
  if (s->has_attr("theta")) {
    params._theta = as_double(*s, "theta", 0.9);
    if (!(params._theta >= 0.0 && params._theta <= 1.0)) fail("theta must lie in [0, 1]");
  }
  if (s->has_attr("precision")) {
    const std::string pr = s->attr("precision");
    if (pr == "fp64") params._precision = SweepPrecision::FP64;
    else if (pr == "fp32") params._precision = SweepPrecision::FP32;
    else fail("Unknown precision " + pr);
  }

  // <angular_quad>
  const XmlNode * aq = p->child("angular_quad");
  if (!aq) fail("An angular quadrature block has not been provided!");
  params._num_polar = parseUintParam(*aq, "np");
  params._num_azimuthal = parseUintParam(*aq, "na");

  // <mesh>
  const XmlNode * m = p->child("mesh");
  if (!m) fail("A mesh block has not been provided!");
  params._num_dims = parseUintParam(*m, "dims");
  params._refinement = parseUintParam(*m, "refinement");
  auto axis = [&](const char * d, const char * i, const char * what_d, const char * what_i,
                  std::vector<double> & widths, std::vector<unsigned int> & counts) {
    const XmlNode * dn = m->child(d);
    if (!dn) fail(std::string("Mesh ") + what_d + " dimensions have not been provided!");
    parseVecFromString(parseStringParam(*dn, "vals"), widths);
    const XmlNode * in = m->child(i);
    if (!in) fail(std::string("Mesh ") + what_i + " divisions have not been provided!");
    parseVecFromString(parseStringParam(*in, "vals"), counts);
    for (auto & c : counts) c *= (params._refinement + 1);
  };
  axis("dx", "ix", "x", "x", params._dx, params._x_intervals);
  if (params._num_dims > 1) axis("dy", "iy", "y", "y", params._dy, params._y_intervals);
  if (params._num_dims > 2) axis("dz", "iz", "z", "z", params._dz, params._z_intervals);
  const XmlNode * b = m->child("blocks");
  if (!b) fail("Mesh blocks have not been provided!");
  parseVecFromString(parseStringParam(*b, "vals"), params._blocks);

  // <materials>
  const XmlNode * mats = p->child("materials");
  if (!mats) fail("A materials block has not been provided!");
  const unsigned int G = params._num_e_groups;
  for (const auto & mn : mats->children) {
    const unsigned int blk = parseUintParam(*mn, "block");
    if (params._block_mat_info.count(blk) != 0u)
      fail("A block can only contain one set of material properties, you have provided multiple "
           "material properties for block " + std::to_string(blk) + "!");
    MaterialProps & mp = params._block_mat_info[blk];
    mp._num_d_groups = params._mode == RunMode::Transient ? parseUintParam(*mn, "delayed_groups") : 0u;
    for (const auto & rx : mn->children) {
      const std::string type = rx->attr("type");
      if (type == "total") parseVecFromString(parseStringParam(*rx, "mgxs"), mp._g_total);
      else if (type == "scatter") {
        parseVecFromString(parseStringParam(*rx, "mgxs"), mp._g_g_scatter_mat);
        check_count(mp._g_g_scatter_mat, (size_t)G * G, false, "cross sections", "scatter");
        if (as_bool(*rx, "transpose", false)) {
          const auto tr = mp._g_g_scatter_mat;
          for (unsigned int r = 0; r < G; ++r)
            for (unsigned int c = 0; c < G; ++c) mp._g_g_scatter_mat[r * G + c] = tr[c * G + r];
        }
      }
      else if (type == "source") parseVecFromString(parseStringParam(*rx, "mgxs"), mp._g_src);
      else if (type == "chi_p") parseVecFromString(parseStringParam(*rx, "mgxs"), mp._g_chi_p);
      else if (type == "nu_sigma_f") parseVecFromString(parseStringParam(*rx, "mgxs"), mp._g_prod);
      else if (type == "inv_vel") parseVecFromString(parseStringParam(*rx, "mgxs"), mp._g_inv_v);
      else if (type == "chi_d") parseVecFromString(parseStringParam(*rx, "mgxs"), mp._n_g_chi_d);
      else if (type == "beta") parseVecFromString(parseStringParam(*rx, "mgxs"), mp._g_n_beta);
      else if (type == "lambda_d") parseVecFromString(parseStringParam(*rx, "mgxs"), mp._n_lambda);
      else fail("Unsupported reaction type " + type);
    }
    check_count(mp._g_total, G, false, "cross sections", "total");
    check_count(mp._g_g_scatter_mat, (size_t)G * G, false, "cross sections", "scatter");
    check_count(mp._g_src, G, true, "external sources", "source");
    check_count(mp._g_chi_p, G, true, "prompt fission spectra values", "chi");
    check_count(mp._g_prod, G, true, "fission production cross sections", "nu_sigma_f");
    if (params._mode == RunMode::Transient) {
      check_count(mp._g_inv_v, G, false, "inverse velocities", "inv_vel");
      check_count(mp._n_g_chi_d, (size_t)G * mp._num_d_groups, false, "delayed fission spectra values", "chi_d");
      check_count(mp._g_n_beta, (size_t)G * mp._num_d_groups, false, "delayed fractions", "beta");
      check_count(mp._n_lambda, mp._num_d_groups, false, "delayed decay constants", "lambda_d");
    }
    if (params._dsa)
      for (double t : mp._g_total)
        if (t < 1e-6)
          fail("Void region detected! You cannot use synthetic acceleration when cross sections are "
               "close to zero.");
  }

  // <transients> (read for completeness; transient solves are not run here)
  const XmlNode * tr = p->child("transients");
  if (tr && params._mode == RunMode::Transient) {
    for (const auto & tn : tr->children) {
      if (tn->name != "source_step") continue;
      const unsigned int blk = parseUintParam(*tn, "block");
      if (params._block_step_src.count(blk) != 0u)
        fail("A block can only contain one step source, you have provided multiple step sources for block " +
             std::to_string(blk) + "!");
      SourceStep & step = params._block_step_src[blk];
      const bool ins = !tn->attr("insert_at").empty(), rem = !tn->attr("remove_at").empty();
      if (ins && rem) {
        step._type = StepType::Both;
        step._insert_time = parseDoubleParam(*tn, "insert_at");
        step._remove_time = parseDoubleParam(*tn, "remove_at");
        if (step._remove_time < step._insert_time)
          fail("The step source for block " + std::to_string(blk) + " is removed before it is inserted!");
      } else if (ins) {
        step._type = StepType::Insert;
        step._insert_time = parseDoubleParam(*tn, "insert_at");
      } else if (rem) {
        step._type = StepType::Remove;
        step._remove_time = parseDoubleParam(*tn, "remove_at");
      } else {
        fail("A step source for block " + std::to_string(blk) + " needs insert_at or remove_at!");
      }
      parseVecFromString(parseStringParam(*tn, "mgxs"), step._g_src);
    }
  }
  return params;
}

}  // namespace

void parseVecFromString(const std::string & str, std::vector<double> & res)
{
  split_list(str, res, [](const std::string & s) { return std::stod(s); });
}

void parseVecFromString(const std::string & str, std::vector<unsigned int> & res)
{
  split_list(str, res, [](const std::string & s) { return static_cast<unsigned int>(std::stoul(s)); });
}

InputParameters parseInputParametersFromString(const std::string & xml_text)
{
  auto doc = doma_host::parse_xml(xml_text);
  return parse_document(*doc);
}

InputParameters parseInputParameters(const std::string & file_path)
{
  auto doc = doma_host::parse_xml_file(file_path);
  return parse_document(*doc);
}
