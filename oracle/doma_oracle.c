/*
 * doma_oracle.c -- TEST INFRASTRUCTURE ONLY: CPU restatement of DOMA's 2D/3D
 * fixed-source path, the checker for the GPU library.  Never shipped in or
 * called by the product.
 *
 * Every floating-point expression keeps the association and operation order
 * of the DOMA source it restates (cited per function), and the file is built
 * with -ffp-contract=off, so with one thread the scalar flux it produces is
 * bit-for-bit DOMA's (pinned by tests/golden/).  Storage is this file's own:
 * per-thread face planes instead of DOMA's per-cell face arrays, per-group
 * cross-section arrays instead of a hash-map lookup per cell solve.  The
 * values a cell solve sees are the same, because every cell reads only faces
 * that its upwind neighbours wrote for the same ordinate.
 *
 * Parallelism mirrors DOMA's: an OpenMP loop over the ordinates of one octant
 * with per-thread swept-flux accumulators, reduced in thread order
 * (src/TransportSolver3D.cpp:565-653).
 */
#include "doma_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <omp.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* ------------------------------------------------------------------------ */
/* Quadrature: src/AngularPolynomials.cpp:8-110, src/GCAngularQuadrature.cpp:9-100 */

static double legendre_value(unsigned deg, double x)
{
  /* LegendrePolynomial::evaluate (src/AngularPolynomials.cpp:43-63) */
  if (deg == 0u) return 1.0;
  if (deg == 1u) return x;
  double v = 1.0, v1 = x, v2 = 1.0;
  for (unsigned i = 2; i <= deg; ++i) {
    v = ((2.0 * (double)i - 1.0) * x * v1 - ((double)i - 1.0) * v2) / (double)i;
    v2 = v1;
    v1 = v;
  }
  return v;
}

static double legendre_derivative(unsigned deg, double x)
{
  /* LegendrePolynomial::evaluateDerivative (src/AngularPolynomials.cpp:67-94) */
  if (deg == 0u) return 0.0;
  if (deg == 1u) return 1.0;
  double v = 1.0, d = 0.0, v1 = x, v2 = 1.0;
  const double f = 1.0 / (x * x - 1.0);
  for (unsigned i = 2; i <= deg; ++i) {
    v = ((2.0 * (double)i - 1.0) * x * v1 - ((double)i - 1.0) * v2) / (double)i;
    d = (double)i * f * (x * v - v1);
    v2 = v1;
    v1 = v;
  }
  return d;
}

static void legendre_rule(unsigned deg, double *roots, double *weights)
{
  /* Newton iteration from the cosine guess, stop at |dr| <= 2e-16
   * (src/AngularPolynomials.cpp:8-38). */
  for (unsigned i = 1; i <= deg; ++i) {
    double dr;
    double x = cos(M_PI * ((double)i - 0.25) / ((double)deg + 0.5));
    double v = legendre_value(deg, x);
    double d = legendre_derivative(deg, x);
    do {
      dr = v / d;
      x -= dr;
      v = legendre_value(deg, x);
      d = legendre_derivative(deg, x);
    } while (fabs(dr) > 2e-16);
    roots[i - 1] = x;
    weights[i - 1] = 2.0 / ((1.0 - x * x) * d * d);
  }
}

static int classify(double mu, double eta, double xi)
{
  /* GCAngularQuadrature::classifyDirection (src/GCAngularQuadrature.cpp:78-100):
   * octant index = 4*(mu<0) + 2*(eta<0) + (xi<0); zero components are rejected. */
  if (mu == 0.0 || eta == 0.0 || xi == 0.0 || mu != mu || eta != eta || xi != xi) return -1;
  return (mu < 0.0 ? 4 : 0) + (eta < 0.0 ? 2 : 0) + (xi < 0.0 ? 1 : 0);
}

int oracle_quadrature(uint32_t np, uint32_t na, uint32_t dims, double *mu, double *eta,
                      double *xi, double *w, uint32_t counts[8])
{
  if (np == 0 || na == 0 || (dims != 2 && dims != 3)) return -1;
  const unsigned n_l = 2u * np, n_c = 2u * na;
  const unsigned total = (dims == 3 ? 2u : 1u) * n_l * n_c;
  double *lr = malloc(sizeof(double) * n_l), *lw = malloc(sizeof(double) * n_l);
  double *um = malloc(sizeof(double) * total), *ue = malloc(sizeof(double) * total);
  double *ux = malloc(sizeof(double) * total), *uw = malloc(sizeof(double) * total);
  int *oc = malloc(sizeof(int) * total);
  int rc = (int)total;
  legendre_rule(n_l, lr, lw);
  const double cw = M_PI / (double)n_c; /* ChebyshevPolynomial weights (:99-110) */
  unsigned k = 0;
  for (unsigned i = 1; i <= n_l; ++i) {
    for (unsigned j = 1; j <= n_c; ++j) {
      const double weight = lw[i - 1] * cw;
      const double m = lr[i - 1];
      const double omega = (2 * (double)j - 1.0) / (2.0 * (double)n_c) * M_PI;
      um[k] = m;
      ue[k] = sqrt(1.0 - (m * m)) * cos(omega);
      ux[k] = sqrt(1.0 - (m * m)) * sin(omega);
      uw[k] = weight;
      ++k;
      if (dims > 2) {
        um[k] = -1.0 * m;
        ue[k] = -1.0 * sqrt(1.0 - (m * m)) * cos(omega);
        ux[k] = -1.0 * sqrt(1.0 - (m * m)) * sin(omega);
        uw[k] = weight;
        ++k;
      }
    }
  }
  for (unsigned n = 0; n < total; ++n) {
    oc[n] = classify(um[n], ue[n], ux[n]);
    if (oc[n] < 0) rc = -1;
  }
  if (rc > 0) {
    /* stable binning: octant-major, then generation order */
    unsigned out = 0;
    for (int o = 0; o < 8; ++o) {
      counts[o] = 0;
      for (unsigned n = 0; n < total; ++n) {
        if (oc[n] != o) continue;
        mu[out] = um[n]; eta[out] = ue[n]; xi[out] = ux[n]; w[out] = uw[n];
        ++out;
        ++counts[o];
      }
    }
  }
  free(lr); free(lw); free(um); free(ue); free(ux); free(uw); free(oc);
  return rc;
}

/* ------------------------------------------------------------------------ */
/* Solver state */

typedef struct {
  const doma_problem *p;
  const doma_options *o;
  unsigned dims, nx, ny, nz, G, T;
  size_t N;
  double src_scale;   /* 0.25 in 3D, 0.5 in 2D (src/TransportSolver2D.cpp:351) */
  /* quadrature, octant-major */
  double *amu, *aeta, *axi, *w;
  uint32_t counts[8];
  uint32_t offs[8];
  /* per cell */
  double *vol;        /* lx*ly*lz (src/CartesianCell3D.cpp:140) or lx*ly (2D) */
  double *phi;        /* [G][N] total scalar flux */
  double *prev;       /* [G][N] previous MG iterate */
  double *q;          /* [N] current iteration source */
  double *cur;        /* [N] current (increment) scalar flux */
  double *sigt;       /* [N] total xs of the group being solved */
  double **swept;     /* [T][N] per-thread swept flux */
  double *octpsi;     /* single-thread-order mode with T > 1: [ordinates of an octant][N] w*psi */
  double **zf;        /* [T][nx*ny] per-thread z-face plane (3D) */
  double **yf;        /* [T][nx] per-thread y-face line */
} oracle_state;

/* Single-thread-order mode (oracle_set_single_thread_order): with T > 1
 * threads the ordinates of an octant are still swept in parallel, but each
 * writes w*psi to its own row, the rows are added to every cell's running sum
 * in ordinate order, and the residual norms are summed sequentially.  The
 * result is then bit-equal to a one-thread run (DOMA's T = 1 order), at
 * multi-thread speed.  Off, the threads accumulate privately and the partial
 * sums are added in thread order, as DOMA does with T threads
 * (src/TransportSolver3D.cpp:610-621). */
static int g_single_thread_order = 0;

void oracle_set_single_thread_order(int on) { g_single_thread_order = on != 0; }

static int validate(const doma_problem *p, const doma_options *o)
{
  if (!p || !o) return -1;
  if (p->num_dims != 2 && p->num_dims != 3) return -1;
  if (p->nx == 0 || p->ny == 0 || p->nz == 0) return -1;
  if (p->num_dims == 2 && p->nz != 1) return -1;
  if (!p->dx || !p->dy || (p->num_dims == 3 && !p->dz)) return -1;
  if (p->num_groups == 0 || p->num_materials == 0) return -1;
  if (!p->cell_material || !p->total || !p->scatter) return -1;
  if (p->has_fission && (!p->chi_p || !p->nu_sigma_f)) return -1;
  if (p->num_polar == 0 || p->num_azimuthal == 0) return -1;
  const size_t N = (size_t)p->nx * p->ny * p->nz;
  for (size_t c = 0; c < N; ++c)
    if (p->cell_material[c] >= p->num_materials) return -1;
  if (o->scheme != DOMA_SCHEME_DD && o->scheme != DOMA_SCHEME_TW_DD) return -1;
  return 0;
}

static int state_init(oracle_state *s, const doma_problem *p, const doma_options *o, unsigned T)
{
  memset(s, 0, sizeof(*s));
  if (validate(p, o)) return -1;
  s->p = p; s->o = o;
  s->dims = p->num_dims; s->nx = p->nx; s->ny = p->ny; s->nz = p->nz;
  s->G = p->num_groups; s->T = T ? T : 1;
  s->N = (size_t)p->nx * p->ny * p->nz;
  s->src_scale = s->dims == 3 ? 0.25 : 0.5;
  const unsigned D = (s->dims == 3 ? 8u : 4u) * p->num_polar * p->num_azimuthal;
  double *mu = malloc(sizeof(double) * D), *eta = malloc(sizeof(double) * D);
  double *xi = malloc(sizeof(double) * D);
  s->w = malloc(sizeof(double) * D);
  if (oracle_quadrature(p->num_polar, p->num_azimuthal, s->dims, mu, eta, xi, s->w, s->counts) < 0) {
    free(mu); free(eta); free(xi); free(s->w);
    return -1;
  }
  s->amu = malloc(sizeof(double) * D); s->aeta = malloc(sizeof(double) * D);
  s->axi = malloc(sizeof(double) * D);
  for (unsigned n = 0; n < D; ++n) {
    s->amu[n] = fabs(mu[n]); s->aeta[n] = fabs(eta[n]); s->axi[n] = fabs(xi[n]);
  }
  free(mu); free(eta); free(xi);
  unsigned off = 0;
  for (int oc = 0; oc < 8; ++oc) { s->offs[oc] = off; off += s->counts[oc]; }

  const size_t N = s->N;
  s->vol = malloc(sizeof(double) * N);
  for (unsigned k = 0; k < s->nz; ++k)
    for (unsigned j = 0; j < s->ny; ++j)
      for (unsigned i = 0; i < s->nx; ++i) {
        const size_t c = ((size_t)k * s->ny + j) * s->nx + i;
        s->vol[c] = s->dims == 3 ? p->dx[i] * p->dy[j] * p->dz[k] : p->dx[i] * p->dy[j];
      }
  s->phi = calloc(N * s->G, sizeof(double));
  s->prev = calloc(N * s->G, sizeof(double));
  s->q = calloc(N, sizeof(double));
  s->cur = calloc(N, sizeof(double));
  s->sigt = calloc(N, sizeof(double));
  s->swept = malloc(sizeof(double *) * s->T);
  s->zf = malloc(sizeof(double *) * s->T);
  s->yf = malloc(sizeof(double *) * s->T);
  for (unsigned t = 0; t < s->T; ++t) {
    s->swept[t] = calloc(N, sizeof(double));
    s->zf[t] = calloc((size_t)s->nx * s->ny, sizeof(double));
    s->yf[t] = calloc(s->nx, sizeof(double));
  }
  if (g_single_thread_order && s->T > 1) {
    uint32_t most = 0;
    for (int oc = 0; oc < 8; ++oc) most = s->counts[oc] > most ? s->counts[oc] : most;
    s->octpsi = malloc(sizeof(double) * N * most);
    if (!s->octpsi) return -1;
  }
  return 0;
}

static void state_free(oracle_state *s)
{
  free(s->amu); free(s->aeta); free(s->axi); free(s->w);
  free(s->vol); free(s->phi); free(s->prev); free(s->q); free(s->cur); free(s->sigt);
  if (s->swept)
    for (unsigned t = 0; t < s->T; ++t) { free(s->swept[t]); free(s->zf[t]); free(s->yf[t]); }
  free(s->swept); free(s->zf); free(s->yf); free(s->octpsi);
}

/* ------------------------------------------------------------------------ */
/* Multigroup source: TransportSolver3D::updateMultigroupSource, fixed-source
 * terms only (src/TransportSolver3D.cpp:339-402; 2D: src/TransportSolver2D.cpp:341-402). */
static void mg_source(oracle_state *s, unsigned g)
{
  const doma_problem *p = s->p;
  const unsigned G = s->G;
  const double a = s->src_scale;
  #pragma omp parallel for schedule(static)
  for (size_t c = 0; c < s->N; ++c) {
    const unsigned m = p->cell_material[c];
    s->cur[c] = 0.0;
    double q = p->source ? a * p->source[(size_t)m * G + g] / M_PI : 0.0;
    const int fis = p->has_fission && p->has_fission[m];
    for (unsigned gp = 0; gp < G; ++gp) {
      if (gp != g)
        q += a * p->scatter[((size_t)m * G + g) * G + gp] * s->phi[(size_t)gp * s->N + c] / M_PI;
      if (fis)
        q += a * p->chi_p[(size_t)m * G + g] * p->nu_sigma_f[(size_t)m * G + gp] *
             s->phi[(size_t)gp * s->N + c] / M_PI;
    }
    s->q[c] = q;
    s->prev[(size_t)g * s->N + c] = s->phi[(size_t)g * s->N + c];
    s->phi[(size_t)g * s->N + c] = 0.0;
    s->sigt[c] = p->total[(size_t)m * G + g];
  }
}

/* ------------------------------------------------------------------------ */
/* Cell solves.  Expressions keep DOMA's association exactly. */

/* DiamondDifference3D::solve (include/DiamondDifference3D.h:28-48) */
static inline double dd3(double q, double st, double amu, double aeta, double axi,
                         double lx, double ly, double lz, double *x, double *y, double *z)
{
  double c = q + (2.0 * *x * amu / lx) + (2.0 * *y * aeta / ly) + (2.0 * *z * axi / lz);
  c /= (2.0 * amu / lx) + (2.0 * aeta / ly) + (2.0 * axi / lz) + st;
  *x = 2.0 * c - *x;
  *y = 2.0 * c - *y;
  *z = 2.0 * c - *z;
  return c;
}

/* TWDiamondDifference3D::solve (include/TWDiamondDifference3D.h:29-91), with
 * DOMA's constexpr theta = theta_s = 0.9 turned into the parameter th. */
static inline double twdd3(double q, double st, double amu, double aeta, double axi,
                           double lx, double ly, double lz, double V, double th,
                           double *x, double *y, double *z)
{
  const double A = ly * lz, B = lx * lz, C = lx * ly;
  const double xu = *x, yu = *y, zu = *z;
  double a = 0.5;
  if (xu > 1e-8) {
    a = q * V * th + (aeta * B * yu + axi * C * zu) * th + amu * A * xu;
    a /= (st * V + 2.0 * aeta * B + 2.0 * axi * C) * xu;
    a = -1.0 * (a - 1.0);
  }
  double b = 0.5;
  if (yu > 1e-8) {
    b = q * V * th + (amu * A * xu + axi * C * zu) * th + aeta * B * yu;
    b /= (st * V + 2.0 * amu * A + 2.0 * axi * C) * yu;
    b = -1.0 * (b - 1.0);
  }
  double cc = 0.5;
  if (zu > 1e-8) {
    cc = q * V * th + (amu * A * xu + aeta * B * yu) * th + axi * C * zu;
    cc /= (st * V + 2.0 * amu * A + 2.0 * aeta * B) * zu;
    cc = -1.0 * (cc - 1.0);
  }
  a = a < 0.5 ? 0.5 : a;   a = a > 1.0 ? 1.0 : a;
  b = b < 0.5 ? 0.5 : b;   b = b > 1.0 ? 1.0 : b;
  cc = cc < 0.5 ? 0.5 : cc; cc = cc > 1.0 ? 1.0 : cc;
  double c = q * V + (amu * A / a * xu) + (aeta * B / b * yu) + (axi * C / cc * zu);
  c /= st * V + (amu * A / a) + (aeta * B / b) + (axi * C / cc);
  *x = (c / a) - (((1.0 - a) / a) * xu);
  *y = (c / b) - (((1.0 - b) / b) * yu);
  *z = (c / cc) - (((1.0 - cc) / cc) * zu);
  return c;
}

/* DiamondDifference2D::solve (include/DiamondDifference2D.h:28-44) */
static inline double dd2(double q, double st, double amu, double aeta,
                         double lx, double ly, double *x, double *y)
{
  double c = q + (2.0 * *x * amu / lx) + (2.0 * *y * aeta / ly);
  c /= (2.0 * amu / lx) + (2.0 * aeta / ly) + st;
  *x = 2.0 * c - *x;
  *y = 2.0 * c - *y;
  return c;
}

/* TWDiamondDifference2D::solve (include/TWDiamondDifference2D.h:32-75),
 * including the bare abs_xi term of the b weight (:51). */
static inline double twdd2(double q, double st, double amu, double aeta, double axi,
                           double lx, double ly, double V, double th, double *x, double *y)
{
  const double A = ly, B = lx;
  const double xu = *x, yu = *y;
  double a = 0.5;
  if (xu > 1e-8) {
    a = q * V * th + (aeta * B * yu) * th + amu * A * xu;
    a /= (st * V + 2.0 * aeta * B) * xu;
    a = -1.0 * (a - 1.0);
  }
  double b = 0.5;
  if (yu > 1e-8) {
    b = q * V * th + (amu * A * xu + axi) * th + aeta * B * yu;
    b /= (st * V + 2.0 * amu * A) * yu;
    b = -1.0 * (b - 1.0);
  }
  a = a < 0.5 ? 0.5 : a;  a = a > 1.0 ? 1.0 : a;
  b = b < 0.5 ? 0.5 : b;  b = b > 1.0 ? 1.0 : b;
  double c = q * V + (amu * A / a * xu) + (aeta * B / b * yu);
  c /= st * V + (amu * A / a) + (aeta * B / b);
  *x = (c / a) - (((1.0 - a) / a) * xu);
  *y = (c / b) - (((1.0 - b) / b) * yu);
  return c;
}

/* ------------------------------------------------------------------------ */
/* One ordinate over the whole mesh, in DOMA's lexicographic order for its
 * octant (src/TransportSolver3D.cpp:655-874; 2D: src/TransportSolver2D.cpp:637-725). */
static void sweep_ordinate(oracle_state *s, int oct, unsigned n, unsigned tid)
{
  const doma_problem *p = s->p;
  const unsigned nx = s->nx, ny = s->ny, nz = s->nz;
  const int rx = (oct & 4) != 0, ry = (oct & 2) != 0, rz = (oct & 1) != 0;
  const double amu = s->amu[n], aeta = s->aeta[n], axi = s->axi[n], wt = s->w[n];
  const int tw = s->o->scheme == DOMA_SCHEME_TW_DD;
  const double th = s->o->theta;
  double *sw = s->swept[tid], *zf = s->zf[tid], *yf = s->yf[tid];
  /* single-thread-order mode: this ordinate's own row, summed in order later */
  const int own_row = s->octpsi != NULL;
  if (own_row) sw = s->octpsi + (size_t)(n - s->offs[oct]) * s->N;

  if (s->dims == 3) {
    memset(zf, 0, sizeof(double) * nx * ny);
    for (unsigned kk = 0; kk < nz; ++kk) {
      const unsigned k = rz ? nz - 1 - kk : kk;
      memset(yf, 0, sizeof(double) * nx);
      for (unsigned jj = 0; jj < ny; ++jj) {
        const unsigned j = ry ? ny - 1 - jj : jj;
        double xface = 0.0;
        for (unsigned ii = 0; ii < nx; ++ii) {
          const unsigned i = rx ? nx - 1 - ii : ii;
          const size_t c = ((size_t)k * ny + j) * nx + i;
          double *zc = &zf[(size_t)j * nx + i];
          double psi;
          if (tw)
            psi = twdd3(s->q[c], s->sigt[c], amu, aeta, axi, p->dx[i], p->dy[j], p->dz[k],
                        s->vol[c], th, &xface, &yf[i], zc);
          else
            psi = dd3(s->q[c], s->sigt[c], amu, aeta, axi, p->dx[i], p->dy[j], p->dz[k],
                      &xface, &yf[i], zc);
          if (own_row) sw[c] = wt * psi;
          else sw[c] += wt * psi;
        }
      }
    }
  } else {
    memset(yf, 0, sizeof(double) * nx);
    for (unsigned jj = 0; jj < ny; ++jj) {
      const unsigned j = ry ? ny - 1 - jj : jj;
      double xface = 0.0;
      for (unsigned ii = 0; ii < nx; ++ii) {
        const unsigned i = rx ? nx - 1 - ii : ii;
        const size_t c = (size_t)j * nx + i;
        double psi;
        if (tw)
          psi = twdd2(s->q[c], s->sigt[c], amu, aeta, axi, p->dx[i], p->dy[j], s->vol[c], th,
                      &xface, &yf[i]);
        else
          psi = dd2(s->q[c], s->sigt[c], amu, aeta, p->dx[i], p->dy[j], &xface, &yf[i]);
        if (own_row) sw[c] = wt * psi;
        else sw[c] += wt * psi;
      }
    }
  }
}

/* TransportSolver3D::sweep + parallelSweepOctant (src/TransportSolver3D.cpp:565-653) */
static void sweep(oracle_state *s)
{
  for (int oct = 0; oct < 8; ++oct) {
    const int cnt = (int)s->counts[oct];
    const unsigned off = s->offs[oct];
    if (cnt == 0) continue;   /* 2D: only PPP, PMP, MPP, MMP carry ordinates */
    #pragma omp parallel for schedule(static)
    for (int n = 0; n < cnt; ++n)
      sweep_ordinate(s, oct, off + (unsigned)n, (unsigned)omp_get_thread_num());
    if (s->octpsi) {
      /* the one-thread order: ordinates of this octant, in order, onto the running sum */
      double *sw = s->swept[0];
      #pragma omp parallel for schedule(static)
      for (size_t c = 0; c < s->N; ++c)
        for (int n = 0; n < cnt; ++n) sw[c] += s->octpsi[(size_t)n * s->N + c];
    }
  }
  #pragma omp parallel for schedule(static)
  for (size_t c = 0; c < s->N; ++c) {
    for (unsigned t = 0; t < s->T; ++t) {
      s->cur[c] += s->swept[t][c];
      s->swept[t][c] = 0.0;
    }
  }
}

/* computeScatteringResidual (src/TransportSolver3D.cpp:547-563) */
static double si_residual(oracle_state *s, unsigned g)
{
  double diff = 0.0, tot = 0.0;
  const double *phi = s->phi + (size_t)g * s->N;
  #pragma omp parallel for reduction(+:diff, tot) schedule(static) if(!g_single_thread_order)
  for (size_t c = 0; c < s->N; ++c) {
    const double d = s->cur[c];
    const double t = phi[c] + s->cur[c];
    diff = diff + (d * d) * s->vol[c];
    tot = tot + (t * t) * s->vol[c];
  }
  return tot > 1e-8 ? sqrt(diff) / sqrt(tot) : 0.0;
}

/* updateScatteringSource (src/TransportSolver3D.cpp:531-545) */
static void si_update(oracle_state *s, unsigned g)
{
  const doma_problem *p = s->p;
  const unsigned G = s->G;
  double *phi = s->phi + (size_t)g * s->N;
  #pragma omp parallel for schedule(static)
  for (size_t c = 0; c < s->N; ++c) {
    const unsigned m = p->cell_material[c];
    phi[c] += s->cur[c];
    s->q[c] = s->src_scale * p->scatter[((size_t)m * G + g) * G + g] * s->cur[c] / M_PI;
    s->cur[c] = 0.0;
  }
}

/* computeMGFluxResidual (src/TransportSolver3D.cpp:318-337) */
static double mg_residual(oracle_state *s)
{
  double diff = 0.0, tot = 0.0;
  #pragma omp parallel for reduction(+:diff, tot) schedule(static) if(!g_single_thread_order)
  for (size_t c = 0; c < s->N; ++c) {
    for (unsigned g = 0; g < s->G; ++g) {
      const double a = s->phi[(size_t)g * s->N + c];
      const double d = a - s->prev[(size_t)g * s->N + c];
      diff = diff + (d * d) * s->vol[c];
      tot = tot + (a * a) * s->vol[c];
    }
  }
  return tot > 1e-8 ? sqrt(diff) / sqrt(tot) : 0.0;
}

/* ------------------------------------------------------------------------ */

int oracle_solve(const doma_problem *p, const doma_options *o, uint32_t num_threads,
                 double *phi_out, uint32_t *si_counts, size_t si_cap, size_t *si_len,
                 uint32_t *mg_iterations, double *mg_res_out)
{
  oracle_state s;
  const unsigned T = num_threads ? num_threads : 1;
  omp_set_num_threads((int)T);
  if (state_init(&s, p, o, T)) { state_free(&s); return -1; }
  size_t nsi = 0;
  int ok = 1;
  unsigned mg = 0;
  double mres = 0.0;
  /* solveFixedSource (src/TransportSolver3D.cpp:262-316) */
  do {
    for (unsigned g = 0; g < s.G && ok; ++g) {
      mg_source(&s, g);
      /* sourceIteration (src/TransportSolver3D.cpp:458-497) */
      unsigned it = 0;
      double res = 0.0;
      do {
        sweep(&s);
        res = si_residual(&s, g);
        si_update(&s, g);
        ++it;
      } while (it < o->fs_max_it && o->fs_tol < res);
      if (si_counts && nsi < si_cap) si_counts[nsi] = it;
      ++nsi;
      if (!(it < o->fs_max_it)) ok = 0;
    }
    if (!ok) break;
    mres = mg_residual(&s);
    ++mg;
  } while (mg < o->mg_max_it && o->mg_tol < mres && s.G > 1u);
  if (ok && !(mg < o->mg_max_it)) ok = 0;
  memcpy(phi_out, s.phi, sizeof(double) * s.N * s.G);
  if (si_len) *si_len = nsi;
  if (mg_iterations) *mg_iterations = mg;
  if (mg_res_out) *mg_res_out = mres;
  state_free(&s);
  return ok;
}

/* ------------------------------------------------------------------------ */
/* k-eigenvalue power iteration: TransportSolver3D::solveEigenvalue
 * (src/TransportSolver3D.cpp:29-86; 2D: src/TransportSolver2D.cpp:31-88).
 * The flux starts at 1 in every group (initializeSolve, :512-515).  The
 * group source (updateMultigroupSourceEigen, :404-430) is *added* to the
 * current iteration source, which still holds the previous group's last
 * scattering-increment source -- the reference never resets it there. */
static void mg_source_eigen(oracle_state *s, unsigned g, double k)
{
  const doma_problem *p = s->p;
  const unsigned G = s->G;
  const double a = s->src_scale;
  #pragma omp parallel for schedule(static)
  for (size_t c = 0; c < s->N; ++c) {
    const unsigned m = p->cell_material[c];
    s->cur[c] = 0.0;
    double q = s->q[c];
    const int fis = p->has_fission && p->has_fission[m];
    for (unsigned gp = 0; gp < G; ++gp) {
      if (gp != g)
        q += a * p->scatter[((size_t)m * G + g) * G + gp] * s->phi[(size_t)gp * s->N + c] / M_PI;
      if (fis)
        q += a * p->chi_p[(size_t)m * G + g] * p->nu_sigma_f[(size_t)m * G + gp] *
             s->phi[(size_t)gp * s->N + c] / M_PI / k;
    }
    s->q[c] = q;
    s->prev[(size_t)g * s->N + c] = s->phi[(size_t)g * s->N + c];
    s->phi[(size_t)g * s->N + c] = 0.0;
    s->sigt[c] = p->total[(size_t)m * G + g];
  }
}

/* updateEigenvalue (src/TransportSolver3D.cpp:432-456): cells in order,
 * groups inner, cells without a production cross section skipped. */
static double k_update(oracle_state *s, double k)
{
  const doma_problem *p = s->p;
  const unsigned G = s->G;
  double num = 0.0, den = 0.0;
  for (size_t c = 0; c < s->N; ++c) {
    const unsigned m = p->cell_material[c];
    if (!(p->has_fission && p->has_fission[m])) continue;
    for (unsigned g = 0; g < G; ++g) {
      num = num + s->vol[c] * p->nu_sigma_f[(size_t)m * G + g] * s->phi[(size_t)g * s->N + c];
      den = den + s->vol[c] * p->nu_sigma_f[(size_t)m * G + g] * s->prev[(size_t)g * s->N + c] / k;
    }
  }
  return num / den;
}

int oracle_solve_eigen(const doma_problem *p, const doma_options *o, double k_tol,
                       uint32_t num_threads, double *phi_out, double *k_out,
                       uint32_t *si_counts, size_t si_cap, size_t *si_len,
                       uint32_t *pi_iterations, double *shape_res_out, double *k_res_out)
{
  oracle_state s;
  const unsigned T = num_threads ? num_threads : 1;
  omp_set_num_threads((int)T);
  if (state_init(&s, p, o, T)) { state_free(&s); return -1; }
  for (size_t i = 0; i < s.N * s.G; ++i) s.phi[i] = 1.0;
  size_t nsi = 0;
  int ok = 1;
  unsigned mg = 0;
  double k = 1.0, k_prev = 0.0, shape = 0.0, kdiff = 0.0;
  do {
    for (unsigned g = 0; g < s.G && ok; ++g) {
      mg_source_eigen(&s, g, k);
      unsigned it = 0;
      double res = 0.0;
      do {
        sweep(&s);
        res = si_residual(&s, g);
        si_update(&s, g);
        ++it;
      } while (it < o->fs_max_it && o->fs_tol < res);
      if (si_counts && nsi < si_cap) si_counts[nsi] = it;
      ++nsi;
      if (!(it < o->fs_max_it)) ok = 0;
    }
    if (!ok) break;   /* solveEigenvalue returns false at once */
    k_prev = k;
    k = k_update(&s, k);
    shape = mg_residual(&s);
    kdiff = fabs(k - k_prev);
    ++mg;
  } while (mg < o->mg_max_it && (o->mg_tol < shape || k_tol < kdiff));
  if (ok && !(mg < o->mg_max_it)) ok = 0;
  memcpy(phi_out, s.phi, sizeof(double) * s.N * s.G);
  if (k_out) *k_out = k;
  if (si_len) *si_len = nsi;
  if (pi_iterations) *pi_iterations = mg;
  if (shape_res_out) *shape_res_out = shape;
  if (k_res_out) *k_res_out = kdiff;
  state_free(&s);
  return ok;
}

/* ------------------------------------------------------------------------ */
/* Transient fixed source from a zero initial condition:
 * TransportSolver3D::solveTransient (src/TransportSolver3D.cpp:88-140) with
 * initZeroIC, updateStepFluxes and stepDNPs (:142-260), and the transient
 * terms of updateMultigroupSource (:339-402; 2D: TransportSolver2D.cpp).
 * Kept as DOMA has them: the delayed-neutron and time terms sit inside the
 * loop over source groups g', so each is added G times; the 3D cell solve
 * does not see the 1/(v dt) term (the sweep is not handed the mode), the 2D
 * one does (tot = sigma_t + inv_v / dt). */
typedef struct {
  const doma_transient *tr;
  unsigned D;
  double *phi_last;   /* [G][N] */
  double *dnps;       /* [N][D]: DOMA's _current_t_dnps (== _last_t_dnps between steps) */
} transient_state;

static unsigned mat_d(const transient_state *ts, unsigned m)
{
  return ts->tr->d_groups ? ts->tr->d_groups[m] : 0u;
}

static void mg_source_transient(oracle_state *s, const transient_state *ts, unsigned g, double t)
{
  const doma_problem *p = s->p;
  const doma_transient *tr = ts->tr;
  const unsigned G = s->G, D = ts->D;
  const double a = s->src_scale, dt = tr->dt;
  #pragma omp parallel for schedule(static)
  for (size_t c = 0; c < s->N; ++c) {
    const unsigned m = p->cell_material[c];
    const unsigned Dm = mat_d(ts, m);
    s->cur[c] = 0.0;
    double q = p->source ? a * p->source[(size_t)m * G + g] / M_PI : 0.0;
    const unsigned st = tr->step_type ? tr->step_type[m] : 0u;
    if (st != 0u) {
      const double ins = tr->step_insert[m], rem = tr->step_remove[m];
      const double v = a * tr->step_source[(size_t)m * G + g] / M_PI;
      if (st == 1u) q += ins <= t && t <= rem ? v : 0.0;
      else if (st == 2u) q += ins <= t ? v : 0.0;
      else q += t <= rem ? v : 0.0;
    }
    const int fis = p->has_fission && p->has_fission[m];
    for (unsigned gp = 0; gp < G; ++gp) {
      const double pg = s->phi[(size_t)gp * s->N + c];
      if (gp != g)
        q += a * p->scatter[((size_t)m * G + g) * G + gp] * pg / M_PI;
      if (fis && Dm == 0u)
        q += a * p->chi_p[(size_t)m * G + g] * p->nu_sigma_f[(size_t)m * G + gp] * pg / M_PI;
      else if (fis && Dm > 0u) {
        double g_beta = 0.0;
        for (unsigned d = 0; d < Dm; ++d) g_beta += tr->beta[((size_t)m * G + gp) * D + d];
        q += a * (1.0 - g_beta) * p->chi_p[(size_t)m * G + g] * p->nu_sigma_f[(size_t)m * G + gp] *
             pg / M_PI;
      }
      for (unsigned d = 0; d < Dm; ++d)
        q += a * tr->chi_d[((size_t)m * G + g) * D + d] * ts->dnps[c * D + d] *
             tr->lambda[(size_t)m * D + d] / M_PI;
      q += a * ts->phi_last[(size_t)g * s->N + c] * tr->inv_v[(size_t)m * G + g] / dt / M_PI;
    }
    s->q[c] = q;
    s->prev[(size_t)g * s->N + c] = s->phi[(size_t)g * s->N + c];
    s->phi[(size_t)g * s->N + c] = 0.0;
    s->sigt[c] = p->total[(size_t)m * G + g];
    if (s->dims == 2) s->sigt[c] += tr->inv_v[(size_t)m * G + g] / dt;
  }
}

/* stepDNPs (src/TransportSolver3D.cpp:236-260) */
static void step_dnps(oracle_state *s, transient_state *ts)
{
  const doma_problem *p = s->p;
  const doma_transient *tr = ts->tr;
  const unsigned G = s->G, D = ts->D;
  for (size_t c = 0; c < s->N; ++c) {
    const unsigned m = p->cell_material[c];
    const unsigned Dm = mat_d(ts, m);
    for (unsigned d = 0; d < Dm; ++d) {
      double c_src = 0.0;
      for (unsigned g = 0; g < G; ++g)
        c_src += p->nu_sigma_f[(size_t)m * G + g] * s->phi[(size_t)g * s->N + c] *
                 tr->beta[((size_t)m * G + g) * D + d];
      const double lam = tr->lambda[(size_t)m * D + d];
      const double decay = exp(-lam * tr->dt);
      ts->dnps[c * D + d] = (c_src / lam) * (1.0 - decay) + ts->dnps[c * D + d] * decay;
    }
  }
}

int oracle_solve_transient(const doma_problem *p, const doma_options *o, const doma_transient *tr,
                           uint32_t num_threads, double *phi_steps, double *dnps_out,
                           uint32_t *steps_done, uint32_t *si_counts, size_t si_cap,
                           size_t *si_len)
{
  oracle_state s;
  const unsigned T = num_threads ? num_threads : 1;
  omp_set_num_threads((int)T);
  if (!tr || !(tr->dt > 0.0) || !tr->inv_v) return -1;
  if (tr->num_d_groups && (!tr->d_groups || !tr->chi_d || !tr->beta || !tr->lambda)) return -1;
  if (tr->step_type && (!tr->step_insert || !tr->step_remove || !tr->step_source)) return -1;
  if (state_init(&s, p, o, T)) { state_free(&s); return -1; }
  transient_state ts;
  ts.tr = tr;
  ts.D = tr->num_d_groups;
  ts.phi_last = calloc(s.N * s.G, sizeof(double));
  ts.dnps = calloc(s.N * (ts.D ? ts.D : 1), sizeof(double));
  size_t nsi = 0;
  int ok = 1;
  unsigned step = 0;
  double t = 0.0;
  for (; step < tr->num_steps; ++step) {
    /* solveFixedSource("", t) in transient mode: no re-initialisation */
    unsigned mg = 0;
    double mres = 0.0;
    do {
      for (unsigned g = 0; g < s.G && ok; ++g) {
        mg_source_transient(&s, &ts, g, t);
        unsigned it = 0;
        double res = 0.0;
        do {
          sweep(&s);
          res = si_residual(&s, g);
          si_update(&s, g);
          ++it;
        } while (it < o->fs_max_it && o->fs_tol < res);
        if (si_counts && nsi < si_cap) si_counts[nsi] = it;
        ++nsi;
        if (!(it < o->fs_max_it)) ok = 0;
      }
      if (!ok) break;
      mres = mg_residual(&s);
      ++mg;
    } while (mg < o->mg_max_it && o->mg_tol < mres && s.G > 1u);
    if (ok && !(mg < o->mg_max_it)) ok = 0;
    if (!ok) {
      /* the reference returns with the failing step's partial flux in place */
      if (phi_steps)
        memcpy(phi_steps + (size_t)step * s.N * s.G, s.phi, sizeof(double) * s.N * s.G);
      break;
    }
    step_dnps(&s, &ts);
    if (phi_steps) memcpy(phi_steps + (size_t)step * s.N * s.G, s.phi, sizeof(double) * s.N * s.G);
    if (step != tr->num_steps - 1u) {
      /* updateStepFluxes */
      memcpy(ts.phi_last, s.phi, sizeof(double) * s.N * s.G);
      memset(s.phi, 0, sizeof(double) * s.N * s.G);
      memset(s.q, 0, sizeof(double) * s.N);
    }
    t += tr->dt;
  }
  if (dnps_out && ts.D)
    for (size_t c = 0; c < s.N; ++c)
      for (unsigned d = 0; d < ts.D; ++d) dnps_out[(size_t)d * s.N + c] = ts.dnps[c * ts.D + d];
  if (steps_done) *steps_done = step;
  if (si_len) *si_len = nsi;
  free(ts.phi_last);
  free(ts.dnps);
  state_free(&s);
  return ok;
}

int oracle_source_iterations(const doma_problem *p, const doma_options *o,
                             uint32_t num_threads, uint32_t group, uint32_t count,
                             double *phi_out, double *residuals)
{
  oracle_state s;
  const unsigned T = num_threads ? num_threads : 1;
  omp_set_num_threads((int)T);
  if (!p || group >= p->num_groups) return -1;
  if (state_init(&s, p, o, T)) { state_free(&s); return -1; }
  mg_source(&s, group);
  for (unsigned it = 0; it < count; ++it) {
    sweep(&s);
    const double r = si_residual(&s, group);
    if (residuals) residuals[it] = r;
    si_update(&s, group);
  }
  if (phi_out) memcpy(phi_out, s.phi, sizeof(double) * s.N * s.G);
  state_free(&s);
  return 0;
}

int oracle_multigroup_solve(const doma_problem *p, const doma_options *o, uint32_t num_threads,
                            double *phi_out, uint32_t *iterations, double *residual)
{
  oracle_state s;
  const unsigned T = num_threads ? num_threads : 1;
  omp_set_num_threads((int)T);
  if (state_init(&s, p, o, T)) { state_free(&s); return -1; }
  const size_t N = s.N;
  const unsigned G = s.G;
  const double a = s.src_scale;
  double *qall = calloc(N * G, sizeof(double)), *dall = calloc(N * G, sizeof(double));
  double *q_own = s.q;
  for (size_t c = 0; c < N; ++c) {
    const unsigned m = p->cell_material[c];
    for (unsigned g = 0; g < G; ++g)
      qall[(size_t)g * N + c] = p->source ? a * p->source[(size_t)m * G + g] / M_PI : 0.0;
  }
  unsigned it = 0;
  double res = 0.0;
  do {
    for (unsigned g = 0; g < G; ++g) {
      s.q = qall + (size_t)g * N;
      for (size_t c = 0; c < N; ++c) {
        s.sigt[c] = p->total[(size_t)p->cell_material[c] * G + g];
        s.cur[c] = 0.0;
      }
      sweep(&s);
      memcpy(dall + (size_t)g * N, s.cur, sizeof(double) * N);
    }
    double diff = 0.0, tot = 0.0;
    for (size_t c = 0; c < N; ++c) {
      const unsigned m = p->cell_material[c];
      for (unsigned g = 0; g < G; ++g) {
        const double d = dall[(size_t)g * N + c];
        const double t = s.phi[(size_t)g * N + c] + d;
        diff = diff + (d * d) * s.vol[c];
        tot = tot + (t * t) * s.vol[c];
        s.phi[(size_t)g * N + c] = t;
      }
      const int fis = p->has_fission && p->has_fission[m];
      for (unsigned h = 0; h < G; ++h) {
        double acc = 0.0;
        for (unsigned g = 0; g < G; ++g) {
          double k = p->scatter[((size_t)m * G + h) * G + g];
          if (fis) k = k + p->chi_p[(size_t)m * G + h] * p->nu_sigma_f[(size_t)m * G + g];
          acc = acc + k * dall[(size_t)g * N + c];
        }
        qall[(size_t)h * N + c] = a * acc / M_PI;
      }
    }
    res = tot > 1e-8 ? sqrt(diff) / sqrt(tot) : 0.0;
    ++it;
  } while (it < o->fs_max_it && o->fs_tol < res && isfinite(res));
  s.q = q_own;
  memcpy(phi_out, s.phi, sizeof(double) * N * G);
  if (iterations) *iterations = it;
  if (residual) *residual = res;
  free(qall);
  free(dall);
  state_free(&s);
  return it < o->fs_max_it ? 1 : 0;
}
