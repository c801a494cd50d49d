// quadrature.cpp -- Gauss-Legendre x Chebyshev product quadrature, binned by
// octant, computed on the host and uploaded once per solver.
//
// Restates GCAngularQuadrature (src/GCAngularQuadrature.cpp:9-100) with
// LegendrePolynomial / ChebyshevPolynomial (src/AngularPolynomials.cpp:8-110):
// the polar cosine mu (along x) is a Gauss-Legendre root on [-1, 1] found by
// Newton iteration from cos(pi (i - 1/4) / (n + 1/2)) until |step| <= 2e-16,
// the azimuth is the Chebyshev angle (2j - 1) pi / (2 n_c) on (0, pi),
// eta = sqrt(1 - mu^2) cos(omega), xi = sqrt(1 - mu^2) sin(omega), weights
// w_L * pi / n_c, and in 3D the negated direction is added after each one.
// Directions are binned into octants PPP..MMM in generation order.  The
// arithmetic keeps the reference's association so the tables are bit-equal
// to DOMA's (checked against tests/golden/quadrature.npz); this file is built
// with -ffp-contract=off for that reason.
#include <cmath>

#include "common.cuh"

namespace doma {
namespace {

double legendre_value(unsigned deg, double x)
{
  if (deg == 0u) return 1.0;
  if (deg == 1u) return x;
  double v = 1.0, v1 = x, v2 = 1.0;
  for (unsigned i = 2; i <= deg; ++i) {
    v = ((2.0 * static_cast<double>(i) - 1.0) * x * v1 - (static_cast<double>(i) - 1.0) * v2) /
        static_cast<double>(i);
    v2 = v1;
    v1 = v;
  }
  return v;
}

double legendre_slope(unsigned deg, double x)
{
  if (deg == 0u) return 0.0;
  if (deg == 1u) return 1.0;
  double v = 1.0, d = 0.0, v1 = x, v2 = 1.0;
  const double f = 1.0 / (x * x - 1.0);
  for (unsigned i = 2; i <= deg; ++i) {
    v = ((2.0 * static_cast<double>(i) - 1.0) * x * v1 - (static_cast<double>(i) - 1.0) * v2) /
        static_cast<double>(i);
    d = static_cast<double>(i) * f * (x * v - v1);
    v2 = v1;
    v1 = v;
  }
  return d;
}

int octant_of(double mu, double eta, double xi)
{
  if (!(mu != 0.0 && eta != 0.0 && xi != 0.0)) return -1;  // also rejects NaN
  return (mu < 0.0 ? 4 : 0) + (eta < 0.0 ? 2 : 0) + (xi < 0.0 ? 1 : 0);
}

}  // namespace

int gc_quadrature(unsigned np, unsigned na, unsigned dims, double * mu, double * eta,
                  double * xi, double * w, unsigned counts[8])
{
  // No heap use: the no-allocation sweep entry point calls this too.  The
  // Legendre roots and weights live on the stack (n_l <= 2 * kMaxQuadPolar),
  // and the directions are generated once per octant in generation order,
  // which bins them exactly as generating all and filtering would.
  if (np == 0 || na == 0 || (dims != 2 && dims != 3) || np > kMaxQuadPolar || na > kMaxQuadPolar)
    return -1;
  const unsigned n_l = 2u * np, n_c = 2u * na;
  double root[2 * kMaxQuadPolar], lw[2 * kMaxQuadPolar];
  for (unsigned i = 1; i <= n_l; ++i) {
    double dr;
    double x = std::cos(kPi * (static_cast<double>(i) - 0.25) / (static_cast<double>(n_l) + 0.5));
    double v = legendre_value(n_l, x);
    double d = legendre_slope(n_l, x);
    int guard = 0;
    do {
      dr = v / d;
      x -= dr;
      v = legendre_value(n_l, x);
      d = legendre_slope(n_l, x);
    } while (std::abs(dr) > 2e-16 && ++guard < 1000);
    root[i - 1] = x;
    lw[i - 1] = 2.0 / ((1.0 - x * x) * d * d);
  }
  const double cheb_w = kPi / static_cast<double>(n_c);
  unsigned k = 0;
  for (int o = -1; o < 8; ++o) {  // o = -1: validity pass only
    if (o >= 0) counts[o] = 0;
    for (unsigned i = 1; i <= n_l; ++i) {
      for (unsigned j = 1; j <= n_c; ++j) {
        const double weight = lw[i - 1] * cheb_w;
        const double m = root[i - 1];
        const double omega = (2 * static_cast<double>(j) - 1.0) / (2.0 * static_cast<double>(n_c)) * kPi;
        for (unsigned copy = 0; copy < (dims > 2 ? 2u : 1u); ++copy) {
          double dm, de, dx;
          if (copy == 0) {
            dm = m;
            de = std::sqrt(1.0 - (m * m)) * std::cos(omega);
            dx = std::sqrt(1.0 - (m * m)) * std::sin(omega);
          } else {
            dm = -1.0 * m;
            de = -1.0 * std::sqrt(1.0 - (m * m)) * std::cos(omega);
            dx = -1.0 * std::sqrt(1.0 - (m * m)) * std::sin(omega);
          }
          const int oc = octant_of(dm, de, dx);
          if (o < 0) {
            if (oc < 0) return -1;
            continue;
          }
          if (oc != o) continue;
          mu[k] = dm; eta[k] = de; xi[k] = dx; w[k] = weight;
          ++k;
          ++counts[o];
        }
      }
    }
  }
  return static_cast<int>(k);
}

}  // namespace doma
