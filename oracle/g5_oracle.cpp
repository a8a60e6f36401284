/*
 * g5_oracle.cpp — CPU restatement (FP64) of godunov_five_eq's per-block
 * timestep, GodunovImplemV0::do_time_step (scheme/GodunovImplemV0.cpp:85-151).
 *
 * TEST INFRASTRUCTURE ONLY: the parity checker and the timed CPU baseline.
 * The product never links this file.
 *
 * The staging follows the reference literally: a ghosted primitive array Q
 * (ghost width 2), ghosted slope arrays (ghost width 1), one flux array and
 * one u* array per direction, then the per-direction read-back update and the
 * volume-fraction renormalisation.  Every arithmetic expression keeps the
 * reference's operation order; build with -ffp-contract=off so that no
 * multiply-add is fused (results are then identical on x86-64 and aarch64).
 *
 * Pinned to the reference's own code compiled from its tree (oracle/refpin,
 * golden vectors in tests/golden/, tests/test_golden.py): riemann_hllc and
 * computePrimitives per state, and one whole do_time_step of periodic tiles
 * of same-level blocks through the reference's scheme functors (limited
 * slopes, MUSCL-Hancock and THINC reconstruction, flux store, read-back
 * update with both volume-fraction source terms, renormalisation, CFL
 * reduction), 2D and 3D, bit for bit; the refinement flags of the
 * reference's ComputeRefineFlags over threshold sweeps; the boundary fill of
 * the reference's FillOutsideCellFunctor (ZERO_GRADIENT and WALL faces).
 *
 * Unpinned restatements (external kalypsso core, absent):
 *   - stiffened-gas mixture EOS (Allaire, Clerc & Kokh 2002);
 *   - Youngs normal (3x3(x3) weighted central differences, unit cell);
 *   - stencil semantics: restriction = mean of the 2^dim fine cells,
 *     prolongation = SIMPLE_COPY of the coarse cell containing the ghost
 *     cell centre, or the minmod extrapolation / conservative order-2 and
 *     order-4 interpolation of prolong_ghost, coarse/fine face sums over the
 *     2^(dim-1) fine faces;
 *   - tanh evaluated by g5o_tanh (Cody-Waite reduced Taylor expm1).
 */
#include "g5_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#ifdef _OPENMP
#  include <omp.h>
#endif

namespace
{

// variable ids, models/FiveEq.h:35-50
template <int DIM>
struct Ids
{
  static constexpr int ID = 0, IP = 1, IE = 1, IU = 2, IV = 3;
  static constexpr int IW = (DIM == 2) ? 3 : 4;
  static constexpr int HC = IW + 1;
  static constexpr int IA0 = HC, IAD0 = HC + 1, IA1 = HC + 2, IAD1 = HC + 3;
  static constexpr int NV = HC + 4;
};

struct Settings
{
  double smallr, smallc, smallp, slope_type;
  double gamma[2], pinf[2], xi[2], gpx[2];
  int    kind[2], mg_any;
  double mg[2][8], mg_rho0[2];
};

static Settings
make_settings(const G5OParams * p)
{
  Settings s;
  // models/HydroSettings.cpp:18-29: smallp = smallc^2
  s.smallr = p->smallr;
  s.smallc = p->smallc;
  s.smallp = p->smallc * p->smallc;
  s.slope_type = p->slope_type;
  for (int k = 0; k < 2; ++k)
  {
    s.gamma[k] = p->gamma[k];
    s.pinf[k] = p->pinf[k];
    s.xi[k] = 1.0 / (p->gamma[k] - 1.0);
    s.gpx[k] = p->gamma[k] * p->pinf[k] * s.xi[k];
    s.kind[k] = p->eos[k];
    for (int j = 0; j < 8; ++j)
      s.mg[k][j] = p->mg[k][j];
    s.mg_rho0[k] = p->eos[k] != 0 ? p->mg[k][0] : 1.0;
  }
  s.mg_any = p->eos[0] != 0 || p->eos[1] != 0;
  return s;
}

/* ---------------------------------------------------------------------------
 * Stiffened-gas mixture EOS (restated; the reference aliases the external
 * core::eos::MieGruneisenMixture, eos/eos_utils.h:27-28).
 *   xi_k = 1/(gamma_k-1),  S = a0 xi0 + a1 xi1,  PI = a0 g0 pinf0 xi0 + a1 g1 pinf1 xi1
 *   p    = (rho e - PI) / S
 *   e    = (p S + PI) / rho
 *   c^2  = (p (S + 1) + PI) / (rho S)          (c clamped at 0 from below)
 * ------------------------------------------------------------------------- */
static inline double
eos_S(const Settings & s, double a0, double a1)
{
  return a0 * s.xi[0] + a1 * s.xi[1];
}
static inline double
eos_PI(const Settings & s, double a0, double a1)
{
  return a0 * s.gpx[0] + a1 * s.gpx[1];
}
/* Mie-Grueneisen material laws (restated from their published forms; the
 * reference's core::eos::MieGruneisenMixture is external), each written
 * p = G(rho) rho e + f(rho), giving G, dG/drho, f, df/drho:
 *   stiffened gas: G = gamma - 1, f = -gamma pinf
 *   JWL (Lee, Hornig & Kury 1968), mg = {rho0, Gamma0, A1, A2, R1, R2, e0},
 *     x_i = R_i rho0/rho: G = Gamma0, f = sum_i A_i (1 - Gamma0/x_i) exp(-x_i) - Gamma0 rho e0
 *   SHOCKWAVE (Grueneisen form, cubic Us-up Hugoniot fit, Steinberg),
 *     mg = {rho0, Gamma0, c0, s1, s2, s3, b, e0}, mu = rho/rho0 - 1:
 *     G rho = (Gamma0 + b mu) rho0, f = pc - (Gamma0 + b mu) rho0 e0,
 *     pc = rho0 c0^2 mu N/D^2 (mu > 0) else rho0 c0^2 mu,
 *     N = 1 + (1 - Gamma0/2) mu - b mu^2/2, D = 1 - (s1-1) mu - s2 mu^2/(mu+1) - s3 mu^3/(mu+1)^2
 *   SHOCKWAVE2 (linear Us-up Hugoniot reference), mg = {rho0, Gamma0, c0, s, alpha, e0, p0},
 *     eta = 1 - rho0/rho: pH = p0 + rho0 c0^2 eta/(1 - s eta)^2,
 *     eH = e0 + (pH + p0) eta/(2 rho0), G = Gamma0 (rho0/rho)^alpha, f = pH - G rho eH
 * Mixture under pressure equilibrium (Allaire, Clerc & Kokh 2002), material
 * densities rho_k = (alpha rho)_k/alpha_k (rho0_k when alpha_k = 0), xi_k = 1/G_k:
 *   S = sum a_k xi_k, PI = -sum a_k xi_k f_k: p = (rho e - PI)/S
 *   rho c^2 S = p C1 + C0, C1 = sum a_k (h_k + 1), C0 = sum a_k (xi_k rho_k f'_k - h_k f_k),
 *   h_k = xi_k (1 + rho_k G'_k xi_k); bulk modulus rho_k c_k^2 = (1 + rho_k G'_k/G_k)(p - f_k) + rho_k f'_k + G_k p.
 * exp/log use only IEEE +,-,*,/ and exact frexp/ldexp (exp: Cody-Waite + the
 * Taylor expm1 below; log: 2 atanh((m-1)/(m+1)) series), so the values are the
 * same bits on any IEEE machine. */
static inline double expm1_small(double r);

static inline double
g5_exp(double x)
{
  if (x != x)
    return x;
  if (x < -745.5)
    return 0.0;
  if (x > 709.7)
    return HUGE_VAL;
  const double k = floor(x * 1.4426950408889634 + 0.5);
  const double r = (x - k * 0.6931471824645996) - k * -1.904654299957768e-09;
  return ldexp(expm1_small(r) + 1.0, (int)k);
}

static inline double
g5_log(double x)
{
  int    e;
  double m = frexp(x, &e);
  if (m < 0.7071067811865476)
  {
    m = m * 2.0;
    e = e - 1;
  }
  const double t = (m - 1.0) / (m + 1.0);
  const double t2 = t * t;
  static const double c[13] = { 1.0 / 1.0,  1.0 / 3.0,  1.0 / 5.0,  1.0 / 7.0,  1.0 / 9.0,  1.0 / 11.0, 1.0 / 13.0,
                                1.0 / 15.0, 1.0 / 17.0, 1.0 / 19.0, 1.0 / 21.0, 1.0 / 23.0, 1.0 / 25.0 };
  double              sr = c[12];
  for (int j = 11; j >= 0; --j)
    sr = sr * t2 + c[j];
  const double de = (double)e;
  return (2.0 * t * sr + de * 0.6931471824645996) + de * -1.904654299957768e-09;
}

static inline void
mg_law(const Settings & s, int k, double rho, double & G, double & dG, double & f, double & df)
{
  const double * c = s.mg[k];
  if (s.kind[k] == 1)
  {
    const double rho0 = c[0], w = c[1], A1 = c[2], A2 = c[3], R1 = c[4], R2 = c[5], e0 = c[6];
    const double x1 = R1 * rho0 / rho, x2 = R2 * rho0 / rho;
    const double E1 = g5_exp(-x1), E2 = g5_exp(-x2);
    G = w;
    dG = 0.0;
    f = A1 * (1.0 - w / x1) * E1 + A2 * (1.0 - w / x2) * E2 - w * rho * e0;
    df = (A1 * E1 * (x1 - w - w / x1) + A2 * E2 * (x2 - w - w / x2)) / rho - w * e0;
  }
  else if (s.kind[k] == 2)
  {
    const double rho0 = c[0], g0 = c[1], c0 = c[2], s1 = c[3], s2 = c[4], s3 = c[5], b = c[6], e0 = c[7];
    const double mu = rho / rho0 - 1.0;
    const double K = rho0 * c0 * c0;
    double       pc, dpc;
    if (mu > 0.0)
    {
      const double m1 = mu + 1.0;
      const double N = 1.0 + (1.0 - 0.5 * g0) * mu - 0.5 * b * mu * mu;
      const double Np = (1.0 - 0.5 * g0) - b * mu;
      const double D = 1.0 - (s1 - 1.0) * mu - s2 * mu * mu / m1 - s3 * mu * mu * mu / (m1 * m1);
      const double Dp = -(s1 - 1.0) - s2 * (mu * mu + 2.0 * mu) / (m1 * m1) - s3 * (mu * mu * mu + 3.0 * mu * mu) / (m1 * m1 * m1);
      pc = K * mu * N / (D * D);
      dpc = K * ((N + mu * Np) / (D * D) - 2.0 * mu * N * Dp / (D * D * D));
    }
    else
    {
      pc = K * mu;
      dpc = K;
    }
    const double gr = (g0 + b * mu) * rho0;
    G = gr / rho;
    dG = b / rho - G / rho;
    f = pc - gr * e0;
    df = dpc / rho0 - b * e0;
  }
  else if (s.kind[k] == 3)
  {
    const double rho0 = c[0], g0 = c[1], c0 = c[2], sl = c[3], al = c[4], e0 = c[5], p0 = c[6];
    const double eta = 1.0 - rho0 / rho;
    const double w = 1.0 - sl * eta;
    const double K = rho0 * c0 * c0;
    const double pH = p0 + K * eta / (w * w);
    const double eH = e0 + (pH + p0) * eta / (2.0 * rho0);
    const double v = rho0 / rho;
    double       gp;
    if (al == 1.0)
      gp = v;
    else if (al == 0.0)
      gp = 1.0;
    else
      gp = g5_exp(al * g5_log(v));
    G = g0 * gp;
    dG = -al * G / rho;
    const double dpH = K * (1.0 + sl * eta) / (w * w * w);
    const double deH = (dpH * eta + pH + p0) / (2.0 * rho0);
    const double deta = rho0 / (rho * rho);
    f = pH - G * rho * eH;
    df = dpH * deta - (dG * rho + G) * eH - G * rho * deH * deta;
  }
  else
  {
    G = s.gamma[k] - 1.0;
    dG = 0.0;
    f = -s.gamma[k] * s.pinf[k];
    df = 0.0;
  }
}

static inline double
mg_material_density(const Settings & s, int k, double a, double ar)
{
  return a > 0.0 ? fmax(ar / a, s.smallr) : s.mg_rho0[k];
}

static inline void
mg_mixture(const Settings & s, double a0, double a1, double ar0, double ar1, double & S, double & PI, double & C1, double & C0)
{
  S = 0.0;
  PI = 0.0;
  C1 = 0.0;
  C0 = 0.0;
  for (int k = 0; k < 2; ++k)
  {
    const double a = k == 0 ? a0 : a1;
    const double rho = mg_material_density(s, k, a, k == 0 ? ar0 : ar1);
    double       G, dG, f, df;
    mg_law(s, k, rho, G, dG, f, df);
    const double xi = 1.0 / G;
    const double h = xi * (1.0 + rho * dG * xi);
    S = S + a * xi;
    PI = PI - a * xi * f;
    C1 = C1 + a * (h + 1.0);
    C0 = C0 + a * (xi * rho * df - h * f);
  }
}

/* mixture EOS entry points: (a0, a1) volume fractions, (ar0, ar1) partial
 * densities (read by the Mie-Grueneisen laws only) */
static inline double
mixture_pressure(const Settings & s, double rho, double eint, double a0, double a1, double ar0, double ar1)
{
  if (!s.mg_any)
    return (rho * eint - eos_PI(s, a0, a1)) / eos_S(s, a0, a1);
  double S, PI, C1, C0;
  mg_mixture(s, a0, a1, ar0, ar1, S, PI, C1, C0);
  return (rho * eint - PI) / S;
}
static inline double
mixture_specific_eint(const Settings & s, double rho, double p, double a0, double a1, double ar0, double ar1)
{
  if (!s.mg_any)
    return (p * eos_S(s, a0, a1) + eos_PI(s, a0, a1)) / rho;
  double S, PI, C1, C0;
  mg_mixture(s, a0, a1, ar0, ar1, S, PI, C1, C0);
  return (p * S + PI) / rho;
}
static inline double
mixture_sound_speed(const Settings & s, double rho, double p, double a0, double a1, double ar0, double ar1)
{
  if (!s.mg_any)
  {
    const double S = eos_S(s, a0, a1);
    const double c2 = (p * (S + 1.0) + eos_PI(s, a0, a1)) / (rho * S);
    return sqrt(fmax(c2, 0.0));
  }
  double S, PI, C1, C0;
  mg_mixture(s, a0, a1, ar0, ar1, S, PI, C1, C0);
  const double c2 = (p * C1 + C0) / (rho * S);
  return sqrt(fmax(c2, 0.0));
}

/* Miller-Puckett factor pieces: K_k = rho_k c_k^2 (stiffened gas:
 * gamma_k (p + pinf_k)), 1/Kbar = a0/K0 + a1/K1 */
static inline double
material_bulk_modulus(const Settings & s, int k, double p, double a, double ar)
{
  if (!s.mg_any)
    return s.gamma[k] * (p + s.pinf[k]);
  const double rho = mg_material_density(s, k, a, ar);
  double       G, dG, f, df;
  mg_law(s, k, rho, G, dG, f, df);
  return (1.0 + rho * dG / G) * (p - f) + rho * df + G * p;
}
static inline double
mixture_bulk_modulus(const Settings & s, double p, double a0, double a1, double ar0, double ar1)
{
  return 1.0 / (a0 / material_bulk_modulus(s, 0, p, a0, ar0) + a1 / material_bulk_modulus(s, 1, p, a1, ar1));
}

/* ---------------------------------------------------------------------------
 * tanh without libm: tanh(x) = expm1(2x) / (expm1(2x) + 2), x >= 0.
 * expm1 by Cody-Waite range reduction y = k ln2 + r, |r| <= ln2/2, and a
 * degree-16 Taylor polynomial of expm1(r).  Only IEEE +,-,*,/ and ldexp are
 * used, so the value is reproducible bit for bit on any IEEE machine.
 * ------------------------------------------------------------------------- */
static const double kInvFact[17] = { 1.0,
                                     1.0,
                                     0.5,
                                     0.16666666666666666,
                                     0.041666666666666664,
                                     0.008333333333333333,
                                     0.001388888888888889,
                                     0.0001984126984126984,
                                     2.48015873015873e-05,
                                     2.7557319223985893e-06,
                                     2.755731922398589e-07,
                                     2.505210838544172e-08,
                                     2.08767569878681e-09,
                                     1.6059043836821613e-10,
                                     1.1470745597729725e-11,
                                     7.647163731819816e-13,
                                     4.779477332387385e-14 };

static inline double
expm1_small(double r)
{
  double p = kInvFact[16];
  for (int k = 15; k >= 1; --k)
    p = p * r + kInvFact[k];
  return p * r;
}

static inline double
g5_expm1(double y)
{
  if (fabs(y) < 0.34657359027997264)
    return expm1_small(y);
  const double ln2_hi = 0.6931471824645996;     // ln 2 rounded to 24 significant bits
  const double ln2_lo = -1.904654299957768e-09; // ln 2 - ln2_hi
  const double k = floor(y * 1.4426950408889634 + 0.5);
  const double r = (y - k * ln2_hi) - k * ln2_lo;
  return ldexp(expm1_small(r) + 1.0, (int)k) - 1.0;
}

static inline double
g5_tanh(double x)
{
  if (x != x)
    return x;
  const double ax = fabs(x);
  double       t;
  if (ax > 22.0)
    t = 1.0;
  else
  {
    const double em = g5_expm1(2.0 * ax);
    t = em / (em + 2.0);
  }
  return x < 0.0 ? -t : t;
}

/* ---------------------------------------------------------------------------
 * models/utils.h
 * ------------------------------------------------------------------------- */
template <int DIM>
static inline void
hydro_sanitizer(double * q) // models/utils.h:36-73
{
  using H = Ids<DIM>;
  const double eps = 1e-12;
  if (q[H::IAD0] < eps)
    q[H::IAD0] = 0.0;
  if (q[H::IAD1] < eps)
    q[H::IAD1] = 0.0;
  if (q[H::IA0] < eps)
    q[H::IA0] = 0.0;
  if (q[H::IA0] > 1.0 - eps)
    q[H::IA0] = 1.0;
  if (q[H::IA1] < eps)
    q[H::IA1] = 0.0;
  if (q[H::IA1] > 1.0 - eps)
    q[H::IA1] = 1.0;
}

template <int DIM>
static inline double
compute_mixture_ekin(const double * u, const Settings & s) // models/utils.h:124-151
{
  using H = Ids<DIM>;
  const double d = fmax(u[H::ID], s.smallr);
  const double ux = u[H::IU] / d;
  const double uy = u[H::IV] / d;
  if (DIM == 2)
    return 0.5 * (ux * ux + uy * uy);
  const double uz = u[H::IW] / d;
  return 0.5 * (ux * ux + uy * uy + uz * uz);
}

template <int DIM>
static inline double
compute_mixture_pressure(const double * u, const Settings & s) // models/utils.h:160-185
{
  using H = Ids<DIM>;
  const double d = fmax(u[H::IAD0] + u[H::IAD1], s.smallr);
  const double ekin = compute_mixture_ekin<DIM>(u, s);
  const double eint = u[H::IE] / d - ekin;
  return mixture_pressure(s, d, eint, u[H::IA0], 1 - u[H::IA0], u[H::IAD0], u[H::IAD1]);
}

template <int DIM>
static inline double
computePrimitives(const double * u, double * q, const Settings & s) // models/utils.h:200-250
{
  using H = Ids<DIM>;
  const double d = fmax(u[H::ID], s.smallr);
  const double ux = u[H::IU] / d;
  const double uy = u[H::IV] / d;
  const double ekin = compute_mixture_ekin<DIM>(u, s);
  const double eint = u[H::IE] / d - ekin;
  const double p = mixture_pressure(s, d, eint, u[H::IA0], 1.0 - u[H::IA0], u[H::IAD0], u[H::IAD1]);
  q[H::ID] = d;
  q[H::IP] = p;
  q[H::IU] = ux;
  q[H::IV] = uy;
  if (DIM == 3)
    q[H::IW] = u[H::IW] / d;
  q[H::IA0] = fmax(0.0, fmin(1.0, u[H::IA0])); // sanitize_alpha, models/utils.h:82-87
  q[H::IAD0] = u[H::IAD0];
  q[H::IA1] = 1.0 - q[H::IA0];
  q[H::IAD1] = u[H::IAD1];
  hydro_sanitizer<DIM>(q);
  return mixture_sound_speed(s, d, p, q[H::IA0], 1.0 - q[H::IA0], q[H::IAD0], q[H::IAD1]);
}

/* ---------------------------------------------------------------------------
 * models/RiemannSolvers.h:57-262 (riemann_hllc); out = flux[NV], ustar,
 * phistar0, phistar1.
 * ------------------------------------------------------------------------- */
template <int DIM>
static inline void
riemann_hllc(const double * ql, const double * qr, const Settings & s, double * flux, double & ustar, double & phistar0, double & phistar1)
{
  using H = Ids<DIM>;
  const double smallr = s.smallr, smallp = s.smallp, smallc = s.smallc;

  const double rl = fmax(ql[H::IAD0] + ql[H::IAD1], smallr);
  double       pl = fmax(ql[H::IP], rl * smallp);
  const double ul = ql[H::IU];
  const double eintl = mixture_specific_eint(s, rl, pl, ql[H::IA0], 1 - ql[H::IA0], ql[H::IAD0], ql[H::IAD1]);
  pl = mixture_pressure(s, rl, eintl, ql[H::IA0], 1 - ql[H::IA0], ql[H::IAD0], ql[H::IAD1]);
  double ecinl = 0.5 * rl * ul * ul;
  ecinl += 0.5 * rl * ql[H::IV] * ql[H::IV];
  if (DIM == 3)
    ecinl += 0.5 * rl * ql[H::IW] * ql[H::IW];
  const double cl = mixture_sound_speed(s, rl, pl, ql[H::IA0], 1 - ql[H::IA0], ql[H::IAD0], ql[H::IAD1]);
  const double etotl = rl * eintl + ecinl;
  const double ptotl = pl;

  const double rr = fmax(qr[H::IAD0] + qr[H::IAD1], smallr);
  double       pr = fmax(qr[H::IP], rr * smallp);
  const double ur = qr[H::IU];
  const double eintr = mixture_specific_eint(s, rr, pr, qr[H::IA0], 1 - qr[H::IA0], qr[H::IAD0], qr[H::IAD1]);
  pr = mixture_pressure(s, rr, eintr, qr[H::IA0], 1 - qr[H::IA0], qr[H::IAD0], qr[H::IAD1]);
  double ecinr = 0.5 * rr * ur * ur;
  ecinr += 0.5 * rr * qr[H::IV] * qr[H::IV];
  if (DIM == 3)
    ecinr += 0.5 * rr * qr[H::IW] * qr[H::IW];
  const double cr = mixture_sound_speed(s, rr, pr, qr[H::IA0], 1 - qr[H::IA0], qr[H::IAD0], qr[H::IAD1]);
  const double etotr = rr * eintr + ecinr;
  const double ptotr = pr;

  const double cfastl = sqrt(fmax(cl * cl, smallc * smallc));
  const double cfastr = sqrt(fmax(cr * cr, smallc * smallc));
  const double SL = fmin(ul, ur) - fmax(cfastl, cfastr);
  const double SR = fmax(ul, ur) + fmax(cfastl, cfastr);

  const double rcl = rl * (ul - SL);
  const double rcr = rr * (SR - ur);

  const double us = (rcr * ur + rcl * ul + (ptotl - ptotr)) / (rcr + rcl);
  const double ptotstar = (rcr * ptotl + rcl * ptotr + rcl * rcr * (ul - ur)) / (rcr + rcl);

  const double factorL = (SL - ul) / (SL - us);
  const double etotstarl = ((SL - ul) * etotl - ptotl * ul + ptotstar * us) / (SL - us);
  const double factorR = (SR - ur) / (SR - us);
  const double etotstarr = ((SR - ur) * etotr - ptotr * ur + ptotstar * us) / (SR - us);

  double ro, ro_0, ro_1, uo, ptoto, etoto;
  if (SL > 0.0)
  {
    ro_0 = ql[H::IAD0];
    ro_1 = ql[H::IAD1];
    ro = rl;
    uo = ul;
    ptoto = ptotl;
    etoto = etotl;
  }
  else if (us > 0.0)
  {
    ro_0 = ql[H::IAD0] * factorL;
    ro_1 = ql[H::IAD1] * factorL;
    ro = rl * factorL;
    uo = us;
    ptoto = ptotstar;
    etoto = etotstarl;
  }
  else if (SR > 0.0)
  {
    ro_0 = qr[H::IAD0] * factorR;
    ro_1 = qr[H::IAD1] * factorR;
    ro = rr * factorR;
    uo = us;
    ptoto = ptotstar;
    etoto = etotstarr;
  }
  else
  {
    ro_0 = qr[H::IAD0];
    ro_1 = qr[H::IAD1];
    ro = rr;
    uo = ur;
    ptoto = ptotr;
    etoto = etotr;
  }

  for (int v = 0; v < H::NV; ++v)
    flux[v] = 0.0;
  flux[H::IAD0] = ro_0 * uo;
  flux[H::IAD1] = ro_1 * uo;
  flux[H::ID] = (ro_0 + ro_1) * uo;
  flux[H::IU] = ro * uo * uo + ptoto;
  flux[H::IP] = (etoto + ptoto) * uo;
  flux[H::IV] = (flux[H::ID] > 0.0) ? flux[H::ID] * ql[H::IV] : flux[H::ID] * qr[H::IV];
  if (DIM == 3)
    flux[H::IW] = (flux[H::ID] > 0.0) ? flux[H::ID] * ql[H::IW] : flux[H::ID] * qr[H::IW];
  if (flux[H::ID] > 0.0)
  {
    phistar0 = ql[H::IA0];
    phistar1 = 1.0 - ql[H::IA0];
  }
  else
  {
    phistar0 = qr[H::IA0];
    phistar1 = 1.0 - qr[H::IA0];
  }
  ustar = uo;
}

/* scheme/ComputeLimitedSlopesFunctor.cpp:116-137 */
static inline double
slope_unsplit_scalar(double q, double qPlus, double qMinus, double slope_type)
{
  double dq = 0;
  if (slope_type == 1 || slope_type == 2)
  {
    const double dlft = slope_type * (q - qMinus);
    const double drgt = slope_type * (qPlus - q);
    const double dcen = 0.5 * (qPlus - qMinus);
    const double dsgn = (dcen >= 0.0) ? 1.0 : -1.0;
    const double slop = fmin(fabs(dlft), fabs(drgt));
    const double dlim = (dlft * drgt) <= 0.0 ? 0.0 : slop;
    dq = dsgn * fmin(dlim, fabs(dcen));
  }
  return dq;
}

/* ---------------------------------------------------------------------------
 * the solver context
 * ------------------------------------------------------------------------- */
struct Ctx
{
  G5OParams            prm;
  Settings             s;
  int                  dim, b, nv, ns, nc, nthreads;
  int                  n_owned, n_outside, n_total, n_inst;
  std::vector<int32_t> level, coord, nbr, out_src, inst;
  std::vector<int8_t>  nbr_rel, out_normal, out_border;
  // work arrays (sized for the owned blocks)
  std::vector<double> Q, slopes[3], flux, ustar;
};

/* index helpers ------------------------------------------------------------ */
template <int DIM>
struct Geo
{
  int b, G, S;
  explicit Geo(int b_) : b(b_), G(b_ + 4), S(b_ + 2) {}
  int ncell() const { return DIM == 2 ? b * b : b * b * b; }
  int nghost() const { return DIM == 2 ? G * G : G * G * G; }
  int nslope() const { return DIM == 2 ? S * S : S * S * S; }
  int cell(int i, int j, int k) const { return i + b * (j + b * k); }
  int ghost(int i, int j, int k) const { return (i + 2) + G * ((j + 2) + G * (DIM == 3 ? (k + 2) : 0)); }
  int slope(int i, int j, int k) const { return (i + 1) + S * ((j + 1) + S * (DIM == 3 ? (k + 1) : 0)); }
  // flux array of direction d: extent b+1 along d, b otherwise
  int fext(int d, int e) const { return b + (d == e ? 1 : 0); }
  int nflux(int d) const { return DIM == 2 ? fext(d, 0) * fext(d, 1) : fext(d, 0) * fext(d, 1) * fext(d, 2); }
  int flux(int d, int i, int j, int k) const { return i + fext(d, 0) * (j + fext(d, 1) * k); }
};

static inline int
slot_index(int dim, const int * d)
{
  return dim == 2 ? (d[0] + 1) + 3 * (d[1] + 1) : (d[0] + 1) + 3 * (d[1] + 1) + 9 * (d[2] + 1);
}

/* read all conservative variables of cell c of block n */
template <int DIM>
static inline void
load_u(const Ctx & x, const double * U, int n, int c, double * u)
{
  const int nc = Geo<DIM>(x.b).ncell();
  for (int v = 0; v < Ids<DIM>::NV; ++v)
    u[v] = U[((size_t)n * Ids<DIM>::NV + v) * nc + c];
}

/* ---------------------------------------------------------------------------
 * Prolongation of a ghost cell that lies in a coarser neighbour
 * (ConvertToPrimitivesVariablesFunctor.cpp:893-917).  The stencil helpers the
 * reference calls (getNeighLoc, compute_minmod_slopes,
 * compute_linear_combination, the ConservativeInterpolation coefficient
 * tables) live in the external kalypsso core; restated here:
 *
 *  - a stencil point is a level-(l-1) cell q of the coarse grid around owned
 *    block n (l = the block's level; q in coarse cells relative to the block,
 *    whose footprint is [0, b/2)^dim).  Its value is the cell of the
 *    coarser neighbour that holds it, the mean of the 2^dim level-l cells
 *    that cover it (the block itself or a same-level neighbour), or, in a
 *    finer neighbour, the mean of those 2^dim means of 2^dim level-(l+1)
 *    cells (sums x fastest, then divided by 2^dim, as the restriction);
 *  - EXTRAPOLATE_LINEAR_MINMOD (:278-300, :544-620): the coarse value plus
 *    0.25 * (+-1) * the minmod slope (ComputeLimitedSlopesFunctor's slope with
 *    slope_type 1) per direction, +1 for the upper half of the coarse cell;
 *  - CONSERVATIVE_INTERPOLATION_ORDER_2/4 (:341-488): the half-cell averages
 *    of the quadratic (quartic) polynomial whose cell averages match 3 (5)
 *    coarse cells, applied along x, then y (then z):
 *    lower half (1/8, 1, -1/8), (-3/128, 22/128, 1, -22/128, 3/128), upper
 *    half the same reversed; sums left to right.
 * ID = IAD0 + IAD1 and IA1 = 1 - IA0 are recomputed as the reference does.
 * ------------------------------------------------------------------------- */
template <int DIM>
static double
coarse_cell_value(const Ctx & x, const double * U, int n, const int * q, int var)
{
  using H = Ids<DIM>;
  const Geo<DIM> geo(x.b);
  const int      b = x.b, h = b / 2;
  int            s[3] = { 0, 0, 0 }, f[3] = { 0, 0, 0 };
  bool           own = true;
  for (int e = 0; e < DIM; ++e)
  {
    s[e] = q[e] < 0 ? -1 : (q[e] >= h ? 1 : 0);
    f[e] = 2 * q[e] - s[e] * b; // first level-l cell of q in the slot's same-level block
    if (s[e] != 0)
      own = false;
  }
  auto cellv = [&](int blk, int i, int j, int k) { return U[((size_t)blk * H::NV + var) * geo.ncell() + geo.cell(i, j, k)]; };
  auto mean = [&](int blk, int i0, int j0, int k0) {
    double sum = 0.0;
    for (int oz = 0; oz < (DIM == 3 ? 2 : 1); ++oz)
      for (int oy = 0; oy < 2; ++oy)
        for (int ox = 0; ox < 2; ++ox)
          sum += cellv(blk, i0 + ox, j0 + oy, k0 + oz);
    return sum / (double)(1 << DIM);
  };
  if (own)
    return mean(n, f[0], f[1], f[2]);
  const int       slot = slot_index(DIM, s);
  const int       rel = x.nbr_rel[(size_t)n * x.ns + slot];
  const int32_t * nb = &x.nbr[((size_t)n * x.ns + slot) * x.nc];
  if (rel == 0)
    return mean(nb[0], f[0], f[1], f[2]);
  if (rel < 0)
  {
    int cc[3] = { 0, 0, 0 };
    for (int e = 0; e < DIM; ++e)
      cc[e] = ((x.coord[(size_t)n * 3 + e] + s[e]) & 1) * h + (f[e] >> 1);
    return cellv(nb[0], cc[0], cc[1], cc[2]);
  }
  int ch[3] = { 0, 0, 0 }, l[3] = { 0, 0, 0 };
  for (int e = 0; e < DIM; ++e)
  {
    ch[e] = f[e] >= h ? 1 : 0;
    l[e] = 2 * (f[e] - ch[e] * h);
  }
  int F = nb[DIM == 2 ? ch[0] + 2 * ch[1] : ch[0] + 2 * ch[1] + 4 * ch[2]];
  if (F < 0)
  {
    // a child of the finer neighbour that does not touch the block (order-4
    // stencils of 8-cell blocks reach it): the same-level neighbour of the
    // touching sibling, when that sibling is owned and the child is a leaf
    int ct[3] = { 0, 0, 0 }, dl[3] = { 0, 0, 0 };
    for (int e = 0; e < DIM; ++e)
    {
      ct[e] = s[e] == 0 ? ch[e] : (s[e] < 0 ? 1 : 0);
      dl[e] = ch[e] - ct[e];
    }
    const int T = nb[DIM == 2 ? ct[0] + 2 * ct[1] : ct[0] + 2 * ct[1] + 4 * ct[2]];
    const int st = slot_index(DIM, dl);
    if (T < 0 || T >= x.n_owned || x.nbr_rel[(size_t)T * x.ns + st] != 0)
      return NAN; // unresolvable here: the GPU raises its mesh status
    F = x.nbr[((size_t)T * x.ns + st) * x.nc];
  }
  double sum = 0.0;
  for (int oz = 0; oz < (DIM == 3 ? 2 : 1); ++oz)
    for (int oy = 0; oy < 2; ++oy)
      for (int ox = 0; ox < 2; ++ox)
        sum += mean(F, l[0] + 2 * ox, l[1] + 2 * oy, l[2] + 2 * oz);
  return sum / (double)(1 << DIM);
}

static const double kConsO2[2][3] = { { 0.125, 1.0, -0.125 }, { -0.125, 1.0, 0.125 } };
static const double kConsO4[2][5] = { { -3.0 / 128.0, 22.0 / 128.0, 1.0, -22.0 / 128.0, 3.0 / 128.0 },
                                      { 3.0 / 128.0, -22.0 / 128.0, 1.0, 22.0 / 128.0, -3.0 / 128.0 } };

static inline double
lin_comb(const double * c, const double * v, int np)
{
  double r = c[0] * v[0];
  for (int i = 1; i < np; ++i)
    r = r + c[i] * v[i];
  return r;
}

template <int DIM>
static void ghost_state(const Ctx & x, const double * U, int n, const int * g, double * u, int prolongation);

/* prolonged conservative state of the fine cell at position pos (0 lower,
 * 1 upper half per direction) of the coarse cell q, whose stencil values
 * V(q', var) come from the caller */
template <int DIM, typename Val>
static void
prolong_point(int mode, Val V, const int * q, const int * pos, double * u)
{
  using H = Ids<DIM>;
  const int vars[7] = { H::IAD0, H::IAD1, H::IA0, H::IE, H::IU, H::IV, H::IW };
  const int nvars = DIM == 2 ? 6 : 7;
  for (int t = 0; t < nvars; ++t)
  {
    const int var = vars[t];
    double    r;
    if (mode == 1)
    {
      const double u0 = V(q, var);
      double       sl[3] = { 0.0, 0.0, 0.0 };
      for (int e = 0; e < DIM; ++e)
      {
        int qp[3] = { q[0], q[1], q[2] }, qm[3] = { q[0], q[1], q[2] };
        qp[e] += 1;
        qm[e] -= 1;
        sl[e] = slope_unsplit_scalar(u0, V(qp, var), V(qm, var), 1.0);
      }
      r = u0;
      for (int e = 0; e < DIM; ++e)
        r = r + 0.25 * (double)(pos[e] ? 1 : -1) * sl[e];
    }
    else
    {
      const int      rr = mode == 2 ? 1 : 2, np = 2 * rr + 1;
      const double * cx = mode == 2 ? kConsO2[pos[0]] : kConsO4[pos[0]];
      const double * cy = mode == 2 ? kConsO2[pos[1]] : kConsO4[pos[1]];
      const double * cz = mode == 2 ? kConsO2[DIM == 3 ? pos[2] : 0] : kConsO4[DIM == 3 ? pos[2] : 0];
      double         valy[5];
      for (int k = (DIM == 3 ? -rr : 0); k <= (DIM == 3 ? rr : 0); ++k)
      {
        double valx[5];
        for (int j = -rr; j <= rr; ++j)
        {
          double pts[5];
          for (int i = -rr; i <= rr; ++i)
          {
            const int qq[3] = { q[0] + i, q[1] + j, q[2] + k };
            pts[i + rr] = V(qq, var);
          }
          valx[j + rr] = lin_comb(cx, pts, np);
        }
        valy[DIM == 3 ? k + rr : 0] = lin_comb(cy, valx, np);
      }
      r = DIM == 3 ? lin_comb(cz, valy, np) : valy[0];
    }
    u[var] = r;
  }
  u[H::ID] = u[H::IAD0] + u[H::IAD1];
  u[H::IA1] = 1.0 - u[H::IA0];
}

/* conservative state of ghost cell g (block coords, in a coarser slot) */
template <int DIM>
static void
prolong_ghost(const Ctx & x, const double * U, int n, const int * g, double * u)
{
  int q[3] = { 0, 0, 0 }, pos[3] = { 0, 0, 0 };
  for (int e = 0; e < DIM; ++e)
  {
    q[e] = (g[e] + 2) / 2 - 1; // coarse cell holding the ghost cell
    pos[e] = (g[e] + 2) & 1;   // 0 lower, 1 upper half
  }
  prolong_point<DIM>(
    x.prm.prolongation, [&](const int * qq, int var) { return coarse_cell_value<DIM>(x, U, n, qq, var); }, q, pos, u);
}

/* value of variable var at cell q of the grid of owned block n's own level
 * around the block (q in [-2, b+2)): the block's cell, a same-level
 * neighbour's cell, the coarser neighbour's cell holding it or the mean of the
 * 2^dim cells of a finer neighbour covering it (the ghost fill's values) */
template <int DIM>
static double
level_cell_value(const Ctx & x, const double * U, int n, const int * q, int var)
{
  int  g[3] = { q[0], q[1], DIM == 3 ? q[2] : 0 };
  bool inner = true;
  for (int e = 0; e < DIM; ++e)
    inner = inner && q[e] >= 0 && q[e] < x.b;
  double u[Ids<DIM>::NV];
  if (inner)
  {
    const Geo<DIM> geo(x.b);
    return U[((size_t)n * Ids<DIM>::NV + var) * geo.ncell() + geo.cell(q[0], q[1], DIM == 3 ? q[2] : 0)];
  }
  // outside the block: the SIMPLE_COPY / restriction ghost fill of that cell
  ghost_state<DIM>(x, U, n, g, u, 0);
  return u[var];
}
/* ---------------------------------------------------------------------------
 * ConvertToPrimitivesVariablesFunctor::fill_ghosts
 * (scheme/ConvertToPrimitivesVariablesFunctor.cpp:833-926): one ghosted cell
 * (g = cell coords relative to the block, in [-2, b+2)) of owned block n.
 * ------------------------------------------------------------------------- */
template <int DIM>
static void
ghost_state(const Ctx & x, const double * U, int n, const int * g, double * u, int prolongation)
{
  using H = Ids<DIM>;
  const Geo<DIM> geo(x.b);
  const int      b = x.b;
  int            d[3] = { 0, 0, 0 }, v[3] = { 0, 0, 0 };
  bool           inner = true;
  for (int e = 0; e < DIM; ++e)
  {
    d[e] = g[e] < 0 ? -1 : (g[e] >= b ? 1 : 0);
    v[e] = g[e] - d[e] * b;
    if (d[e] != 0)
      inner = false;
  }
  if (inner)
  {
    // fill_inner, :494-510
    load_u<DIM>(x, U, n, geo.cell(v[0], v[1], v[2]), u);
  }
  else
  {
    const int s = slot_index(DIM, d);
    const int rel = x.nbr_rel[(size_t)n * x.ns + s];
    const int32_t * nb = &x.nbr[((size_t)n * x.ns + s) * x.nc];
    if (rel == 0)
    {
      // same level: plain copy (fill_ghost_copy without restriction, :516-537)
      load_u<DIM>(x, U, nb[0], geo.cell(v[0], v[1], v[2]), u);
    }
    else if (rel < 0 && prolongation != 0)
    {
      // coarser neighbour, EXTRAPOLATE_LINEAR_MINMOD or conservative
      // interpolation (:898-912)
      prolong_ghost<DIM>(x, U, n, g, u);
    }
    else if (rel < 0)
    {
      // coarser neighbour: SIMPLE_COPY prolongation (:893-897) of the coarse
      // cell containing the ghost cell centre
      int cc[3] = { 0, 0, 0 };
      for (int e = 0; e < DIM; ++e)
      {
        const int vc = x.coord[(size_t)n * 3 + e] + d[e]; // virtual same-level neighbour
        const int ch = vc & 1;                             // its child position in the coarse block
        cc[e] = ch * (b / 2) + (v[e] >> 1);
      }
      load_u<DIM>(x, U, nb[0], geo.cell(cc[0], cc[1], cc[2]), u);
    }
    else
    {
      // finer neighbour: restriction = mean of the 2^dim fine cells
      // (get_conservative_vars_restriction, :208-246)
      int f0[3] = { 0, 0, 0 }, ch[3] = { 0, 0, 0 };
      for (int e = 0; e < DIM; ++e)
      {
        const int f = 2 * v[e];
        ch[e] = f / b;
        f0[e] = f - ch[e] * b;
      }
      const int child = DIM == 2 ? ch[0] + 2 * ch[1] : ch[0] + 2 * ch[1] + 4 * ch[2];
      const int F = nb[child];
      const int vars[7] = { H::IE, H::IU, H::IV, H::IW, H::IAD0, H::IAD1, H::IA0 };
      const int nvars = DIM == 2 ? 7 : 7;
      for (int t = 0; t < nvars; ++t)
      {
        const int var = vars[t];
        if (DIM == 2 && t == 3)
          continue; // IW == IV in 2D
        double sum = 0.0;
        for (int oz = 0; oz < (DIM == 3 ? 2 : 1); ++oz)
          for (int oy = 0; oy < 2; ++oy)
            for (int ox = 0; ox < 2; ++ox)
            {
              const int c = geo.cell(f0[0] + ox, f0[1] + oy, DIM == 3 ? f0[2] + oz : 0);
              sum += U[((size_t)F * H::NV + var) * geo.ncell() + c];
            }
        u[var] = sum / (double)(1 << DIM);
      }
      u[H::IA1] = 1.0 - u[H::IA0];
      u[H::ID] = u[H::IAD0] + u[H::IAD1];
    }
  }
}

template <int DIM>
static void
fill_ghost_cell(const Ctx & x, const double * U, int n, const int * g, double * q)
{
  using H = Ids<DIM>;
  double u[H::NV];
  ghost_state<DIM>(x, U, n, g, u, x.prm.prolongation);
  double qq[H::NV];
  computePrimitives<DIM>(u, qq, x.s);
  // set_primitive_vars, :252-270
  q[H::ID] = qq[H::ID];
  q[H::IAD0] = qq[H::IAD0];
  q[H::IAD1] = qq[H::IAD1];
  q[H::IA0] = qq[H::IA0];
  q[H::IA1] = 1.0 - qq[H::IA0];
  q[H::IP] = qq[H::IP];
  q[H::IU] = qq[H::IU];
  q[H::IV] = qq[H::IV];
  if (DIM == 3)
    q[H::IW] = qq[H::IW];
}

/* ---------------------------------------------------------------------------
 * Youngs normal on the alpha field of the ghosted array (unit cell size),
 * restated: central differences weighted (1,2,1) (2D) / (1,2,1)x(1,2,1) (3D),
 * n = -grad / |grad| (zero vector when the gradient vanishes).
 * ------------------------------------------------------------------------- */
template <int DIM>
static void
youngs_normal(const double * Qa, const Geo<DIM> & geo, int i, int j, int k, double * n)
{
  auto A = [&](int a, int bb, int c) { return Qa[geo.ghost(i + a, j + bb, k + c)]; };
  double g[3] = { 0, 0, 0 };
  if (DIM == 2)
  {
    g[0] = (A(1, -1, 0) + 2.0 * A(1, 0, 0) + A(1, 1, 0)) - (A(-1, -1, 0) + 2.0 * A(-1, 0, 0) + A(-1, 1, 0));
    g[1] = (A(-1, 1, 0) + 2.0 * A(0, 1, 0) + A(1, 1, 0)) - (A(-1, -1, 0) + 2.0 * A(0, -1, 0) + A(1, -1, 0));
  }
  else
  {
    const double w[3] = { 1.0, 2.0, 1.0 };
    for (int c = -1; c <= 1; ++c)
      for (int bb = -1; bb <= 1; ++bb)
      {
        const double ww = w[bb + 1] * w[c + 1];
        g[0] += ww * (A(1, bb, c) - A(-1, bb, c));
        g[1] += ww * (A(bb, 1, c) - A(bb, -1, c));
        g[2] += ww * (A(bb, c, 1) - A(bb, c, -1));
      }
  }
  double nrm = g[0] * g[0] + g[1] * g[1];
  if (DIM == 3)
    nrm += g[2] * g[2];
  nrm = sqrt(nrm);
  for (int e = 0; e < 3; ++e)
    n[e] = (nrm > 0.0) ? -g[e] / nrm : 0.0;
}

/* ---------------------------------------------------------------------------
 * reconstruct_state (MUSCL + Hancock),
 * scheme/ComputeFluxesAndStoreFunctor.cpp:126-213 (2D), :220-327 (3D).
 * ------------------------------------------------------------------------- */
template <int DIM>
static void
reconstruct_muscl(const Ctx & x, const double * q, const double * const * sl, const double * off, double dtdx, double * qr)
{
  using H = Ids<DIM>;
  const double r0 = q[H::IAD0], r1 = q[H::IAD1];
  const double r = r0 + r1;
  const double p = q[H::IP], u = q[H::IU], v = q[H::IV];
  const double w = DIM == 3 ? q[H::IW] : 0.0;
  const double c = mixture_sound_speed(x.s, r, p, q[H::IA0], 1 - q[H::IA0], r0, r1);
  // sl[d][var]
  const double drx0 = sl[0][H::IAD0], drx1 = sl[0][H::IAD1], dpx = sl[0][H::IP], dux = sl[0][H::IU], dvx = sl[0][H::IV];
  const double dry0 = sl[1][H::IAD0], dry1 = sl[1][H::IAD1], dpy = sl[1][H::IP], duy = sl[1][H::IU], dvy = sl[1][H::IV];
  if (DIM == 2)
  {
    qr[H::IAD0] = r0 + off[0] * drx0 + off[1] * dry0;
    qr[H::IAD1] = r1 + off[0] * drx1 + off[1] * dry1;
    qr[H::IP] = p + off[0] * dpx + off[1] * dpy;
    qr[H::IU] = u + off[0] * dux + off[1] * duy;
    qr[H::IV] = v + off[0] * dvx + off[1] * dvy;
    if (x.prm.integrator == 0)
    {
      const double dtdy = dtdx;
      const double sr0 = (-u * (drx0 + drx1) - dux * r) * dtdx + (-v * (dry0 + dry1) - dvy * r) * dtdy;
      const double sr0_0 = sr0 * q[H::IA0];
      const double sr0_1 = sr0 * (1.0 - q[H::IA0]);
      const double su0 = (-u * dux - dpx / r) * dtdx + (-v * duy) * dtdy;
      const double sv0 = (-u * dvx) * dtdx + (-v * dvy - dpy / r) * dtdy;
      const double sp0 = (-u * dpx - dux * r * c * c) * dtdx + (-v * dpy - dvy * r * c * c) * dtdy;
      qr[H::IAD0] += 0.5 * sr0_0;
      qr[H::IAD1] += 0.5 * sr0_1;
      qr[H::IP] += 0.5 * sp0;
      qr[H::IU] += 0.5 * su0;
      qr[H::IV] += 0.5 * sv0;
    }
  }
  else
  {
    const double drz0 = sl[2][H::IAD0], drz1 = sl[2][H::IAD1], dpz = sl[2][H::IP], duz = sl[2][H::IU], dvz = sl[2][H::IV];
    const double dwx = sl[0][H::IW], dwy = sl[1][H::IW], dwz = sl[2][H::IW];
    qr[H::IAD0] = r0 + off[0] * drx0 + off[1] * dry0 + off[2] * drz0;
    qr[H::IAD1] = r1 + off[0] * drx1 + off[1] * dry1 + off[2] * drz1;
    qr[H::IP] = p + off[0] * dpx + off[1] * dpy + off[2] * dpz;
    qr[H::IU] = u + off[0] * dux + off[1] * duy + off[2] * duz;
    qr[H::IV] = v + off[0] * dvx + off[1] * dvy + off[2] * dvz;
    qr[H::IW] = w + off[0] * dwx + off[1] * dwy + off[2] * dwz;
    if (x.prm.integrator == 0)
    {
      const double dtdy = dtdx, dtdz = dtdx;
      const double sr0 = (-u * (drx0 + drx1) - dux * r) * dtdx + (-v * (dry0 + dry1) - dvy * r) * dtdy +
                         (-w * (drz0 + drz1) - dwz * r) * dtdz;
      const double sr0_0 = sr0 * q[H::IA0];
      const double sr0_1 = sr0 * (1.0 - q[H::IA0]);
      const double su0 = (-u * dux - dpx / r) * dtdx + (-v * duy) * dtdy + (-w * duz) * dtdz;
      const double sv0 = (-u * dvx) * dtdx + (-v * dvy - dpy / r) * dtdy + (-w * dvz) * dtdz;
      const double sw0 = (-u * dwx) * dtdx + (-v * dwy) * dtdy + (-w * dwz - dpz / r) * dtdz;
      const double sp0 = (-u * dpx - dux * r * c * c) * dtdx + (-v * dpy - dvy * r * c * c) * dtdy +
                         (-w * dpz - dwz * r * c * c) * dtdz;
      qr[H::IAD0] += 0.5 * sr0_0;
      qr[H::IAD1] += 0.5 * sr0_1;
      qr[H::IP] += 0.5 * sp0;
      qr[H::IU] += 0.5 * su0;
      qr[H::IV] += 0.5 * sv0;
      qr[H::IW] += 0.5 * sw0;
    }
  }
  qr[H::IAD0] = fmax(x.s.smallr, qr[H::IAD0]);
  qr[H::IAD1] = fmax(x.s.smallr, qr[H::IAD1]);
  qr[H::IA0] = q[H::IA0];
}

/* ---------------------------------------------------------------------------
 * THINC reconstruct_state,
 * scheme/ComputeFluxesAndStoreTHINCFunctor.cpp:122-283 (2D), :290-473 (3D).
 * off[] holds -1/0/+1 here (the reference THINC functor's offsets).
 * Qg is the ghosted primitive array of the block, (i,j,k) the cell.
 * ------------------------------------------------------------------------- */
template <int DIM>
static void
reconstruct_thinc(const Ctx &            x,
                  const double *         q,
                  const double * const * sl,
                  const double *         off,
                  double                 dtdx,
                  const double *         Qg,
                  int                    i,
                  int                    j,
                  int                    k,
                  double *               qr)
{
  using H = Ids<DIM>;
  const Geo<DIM> geo(x.b);
  const double * Qa = Qg + (size_t)H::IA0 * geo.nghost();
  const int      dir = off[0] != 0 ? 0 : (off[1] != 0 ? 1 : 2);
  int            uv[3] = { 0, 0, 0 };
  uv[dir] = 1;
  const double aP = Qa[geo.ghost(i + uv[0], j + uv[1], k + uv[2])];
  const double aC = Qa[geo.ghost(i, j, k)];
  const double aM = Qa[geo.ghost(i - uv[0], j - uv[1], k - uv[2])];
  const double monotonicity = (aP - aC) * (aC - aM);
  const double r0 = q[H::IAD0], r1 = q[H::IAD1];
  const bool   thinc_requested = (q[H::IA0] > x.prm.thinc_eps) && (q[H::IA0] < 1.0 - x.prm.thinc_eps) && monotonicity > 0;
  const double drx0 = sl[0][H::IAD0], drx1 = sl[0][H::IAD1];
  const double dry0 = sl[1][H::IAD0], dry1 = sl[1][H::IAD1];
  const double drz0 = DIM == 3 ? sl[2][H::IAD0] : 0.0, drz1 = DIM == 3 ? sl[2][H::IAD1] : 0.0;
  if (thinc_requested)
  {
    double n[3];
    youngs_normal<DIM>(Qa, geo, i, j, k, n);
    const int    bsgn = off[dir] < 0 ? -1 : 1;
    const double beta = x.prm.thinc_beta * fabs(n[dir]) + 0.01;
    const double A = (aP + aM) / 2;
    const double B = (aP - aM) / 2;
    const double C = g5_tanh(0.5 * beta);
    const double phi = aC;
    const double D = g5_tanh(0.5 * beta * (phi - A) / B);
    qr[H::IA0] = A + bsgn * B * (C + bsgn * D / C) / (1.0 + bsgn * D);
    qr[H::IAD0] = r0 + r0 / q[H::IA0] * (qr[H::IA0] - q[H::IA0]);
    qr[H::IAD1] = r1 + r1 / (1.0 - q[H::IA0]) * (q[H::IA0] - qr[H::IA0]);
  }
  else
  {
    qr[H::IA0] = q[H::IA0];
    if (DIM == 2)
    {
      qr[H::IAD0] = r0 + 0.5 * off[0] * drx0 + 0.5 * off[1] * dry0;
      qr[H::IAD1] = r1 + 0.5 * off[0] * drx1 + 0.5 * off[1] * dry1;
    }
    else
    {
      qr[H::IAD0] = r0 + 0.5 * off[0] * drx0 + 0.5 * off[1] * dry0 + 0.5 * off[2] * drz0;
      qr[H::IAD1] = r1 + 0.5 * off[0] * drx1 + 0.5 * off[1] * dry1 + 0.5 * off[2] * drz1;
    }
  }
  const double p = q[H::IP], u = q[H::IU], v = q[H::IV];
  const double w = DIM == 3 ? q[H::IW] : 0.0;
  const double r = r0 + r1;
  const double c = mixture_sound_speed(x.s, r, p, q[H::IA0], 1 - q[H::IA0], r0, r1);
  const double dpx = sl[0][H::IP], dux = sl[0][H::IU], dvx = sl[0][H::IV];
  const double dpy = sl[1][H::IP], duy = sl[1][H::IU], dvy = sl[1][H::IV];
  if (DIM == 2)
  {
    qr[H::IP] = p + 0.5 * off[0] * dpx + 0.5 * off[1] * dpy;
    qr[H::IU] = u + 0.5 * off[0] * dux + 0.5 * off[1] * duy;
    qr[H::IV] = v + 0.5 * off[0] * dvx + 0.5 * off[1] * dvy;
    if (x.prm.integrator == 0)
    {
      const double dtdy = dtdx;
      const double sr0 = (-u * (drx0 + drx1) - dux * r) * dtdx + (-v * (dry0 + dry1) - dvy * r) * dtdy;
      const double sr0_0 = sr0 * q[H::IA0];
      const double sr0_1 = sr0 * (1.0 - q[H::IA0]);
      const double su0 = (-u * dux - dpx / r) * dtdx + (-v * duy) * dtdy;
      const double sv0 = (-u * dvx) * dtdx + (-v * dvy - dpy / r) * dtdy;
      const double sp0 = (-u * dpx - dux * r * c * c) * dtdx + (-v * dpy - dvy * r * c * c) * dtdy;
      qr[H::IAD0] += 0.5 * sr0_0;
      qr[H::IAD1] += 0.5 * sr0_1;
      qr[H::IP] += 0.5 * sp0;
      qr[H::IU] += 0.5 * su0;
      qr[H::IV] += 0.5 * sv0;
    }
  }
  else
  {
    const double dpz = sl[2][H::IP], duz = sl[2][H::IU], dvz = sl[2][H::IV];
    const double dwx = sl[0][H::IW], dwy = sl[1][H::IW], dwz = sl[2][H::IW];
    qr[H::IP] = p + 0.5 * off[0] * dpx + 0.5 * off[1] * dpy + 0.5 * off[2] * dpz;
    qr[H::IU] = u + 0.5 * off[0] * dux + 0.5 * off[1] * duy + 0.5 * off[2] * duz;
    qr[H::IV] = v + 0.5 * off[0] * dvx + 0.5 * off[1] * dvy + 0.5 * off[2] * dvz;
    qr[H::IW] = w + 0.5 * off[0] * dwx + 0.5 * off[1] * dwy + 0.5 * off[2] * dwz;
    if (x.prm.integrator == 0)
    {
      const double dtdy = dtdx, dtdz = dtdx;
      const double sr0 = (-u * (drx0 + drx1) - dux * r) * dtdx + (-v * (dry0 + dry1) - dvy * r) * dtdy +
                         (-w * (drz0 + drz1) - dwz * r) * dtdz;
      const double sr0_0 = sr0 * q[H::IA0];
      const double sr0_1 = sr0 * (1.0 - q[H::IA0]);
      const double su0 = (-u * dux - dpx / r) * dtdx + (-v * duy) * dtdy + (-w * duz) * dtdz;
      const double sv0 = (-u * dvx) * dtdx + (-v * dvy - dpy / r) * dtdy + (-w * dvz) * dtdz;
      const double sw0 = (-u * dwx) * dtdx + (-v * dwy) * dtdy + (-w * dwz - dpz / r) * dtdz;
      const double sp0 = (-u * dpx - dux * r * c * c) * dtdx + (-v * dpy - dvy * r * c * c) * dtdy +
                         (-w * dpz - dwz * r * c * c) * dtdz;
      qr[H::IAD0] += 0.5 * sr0_0;
      qr[H::IAD1] += 0.5 * sr0_1;
      qr[H::IP] += 0.5 * sp0;
      qr[H::IU] += 0.5 * su0;
      qr[H::IV] += 0.5 * sv0;
      qr[H::IW] += 0.5 * sw0;
    }
  }
}

/* ---------------------------------------------------------------------------
 * the step
 * ------------------------------------------------------------------------- */
template <int DIM>
static void
convert_to_primitives(Ctx & x, const double * U) // GodunovImplemV0.cpp:231-279
{
  using H = Ids<DIM>;
  const Geo<DIM> geo(x.b);
  const int      ng = geo.nghost();
  const int      G = geo.G;
#pragma omp parallel for schedule(static) num_threads(x.nthreads)
  for (int n = 0; n < x.n_owned; ++n)
  {
    double * Qn = &x.Q[(size_t)n * H::NV * ng];
    for (int gc = 0; gc < ng; ++gc)
    {
      int g[3] = { gc % G - 2, (gc / G) % G - 2, DIM == 3 ? gc / (G * G) - 2 : 0 };
      double q[H::NV];
      fill_ghost_cell<DIM>(x, U, n, g, q);
      for (int v = 0; v < H::NV; ++v)
        Qn[(size_t)v * ng + gc] = q[v];
    }
  }
}

template <int DIM>
static void
compute_limited_slopes(Ctx & x) // ComputeLimitedSlopesFunctor.cpp:143-193
{
  using H = Ids<DIM>;
  const Geo<DIM> geo(x.b);
  const int      ng = geo.nghost(), ns = geo.nslope(), S = geo.S;
#pragma omp parallel for schedule(static) num_threads(x.nthreads)
  for (int n = 0; n < x.n_owned; ++n)
  {
    const double * Qn = &x.Q[(size_t)n * H::NV * ng];
    for (int sc = 0; sc < ns; ++sc)
    {
      const int i = sc % S - 1, j = (sc / S) % S - 1, k = DIM == 3 ? sc / (S * S) - 1 : 0;
      for (int v = 0; v < H::NV; ++v)
      {
        const double * Qv = Qn + (size_t)v * ng;
        for (int d = 0; d < DIM; ++d)
        {
          const int o[3] = { d == 0, d == 1, d == 2 };
          x.slopes[d][((size_t)n * H::NV + v) * ns + sc] =
            slope_unsplit_scalar(Qv[geo.ghost(i, j, k)],
                                 Qv[geo.ghost(i + o[0], j + o[1], k + o[2])],
                                 Qv[geo.ghost(i - o[0], j - o[1], k - o[2])],
                                 x.s.slope_type);
        }
      }
    }
  }
}

template <int DIM>
static void
compute_fluxes_and_store(Ctx & x, int dir, const double * dt) // ComputeFluxesAndStore*Functor
{
  using H = Ids<DIM>;
  const Geo<DIM> geo(x.b);
  const int      ng = geo.nghost(), ns = geo.nslope(), nf = geo.nflux(dir);
  const int      f0 = geo.fext(dir, 0), f1 = geo.fext(dir, 1);
#pragma omp parallel for schedule(static) num_threads(x.nthreads)
  for (int n = 0; n < x.n_owned; ++n)
  {
    const double * Qn = &x.Q[(size_t)n * H::NV * ng];
    const int      inst = x.inst.empty() ? 0 : x.inst[n];
    const double   dx = x.prm.level_dx[x.level[n]];
    const double   dtdx = dt[inst] / dx;
    for (int fc = 0; fc < nf; ++fc)
    {
      const int i = fc % f0, j = (fc / f0) % f1, k = DIM == 3 ? fc / (f0 * f1) : 0;
      const int o[3] = { dir == 0, dir == 1, dir == 2 };
      const int cl[3] = { i - o[0], j - o[1], k - o[2] };
      const int cr[3] = { i, j, k };
      double    qn[H::NV], qc[H::NV], sln[3][H::NV], slc[3][H::NV];
      const int gl = geo.ghost(cl[0], cl[1], cl[2]), gr = geo.ghost(cr[0], cr[1], cr[2]);
      const int sln_i = geo.slope(cl[0], cl[1], cl[2]), slc_i = geo.slope(cr[0], cr[1], cr[2]);
      for (int v = 0; v < H::NV; ++v)
      {
        qn[v] = Qn[(size_t)v * ng + gl];
        qc[v] = Qn[(size_t)v * ng + gr];
        for (int d = 0; d < DIM; ++d)
        {
          sln[d][v] = x.slopes[d][((size_t)n * H::NV + v) * ns + sln_i];
          slc[d][v] = x.slopes[d][((size_t)n * H::NV + v) * ns + slc_i];
        }
      }
      const double * psln[3] = { sln[0], sln[1], sln[2] };
      const double * pslc[3] = { slc[0], slc[1], slc[2] };
      double         qL[H::NV], qR[H::NV];
      for (int v = 0; v < H::NV; ++v)
        qL[v] = qR[v] = 0.0;
      if (x.prm.thinc)
      {
        double offL[3] = { 0, 0, 0 }, offR[3] = { 0, 0, 0 };
        offL[dir] = 1.0;
        offR[dir] = -1.0;
        reconstruct_thinc<DIM>(x, qn, psln, offL, dtdx, Qn, cl[0], cl[1], cl[2], qL);
        reconstruct_thinc<DIM>(x, qc, pslc, offR, dtdx, Qn, cr[0], cr[1], cr[2], qR);
      }
      else
      {
        double offL[3] = { 0, 0, 0 }, offR[3] = { 0, 0, 0 };
        offL[dir] = 0.5;
        offR[dir] = -0.5;
        reconstruct_muscl<DIM>(x, qn, psln, offL, dtdx, qL);
        reconstruct_muscl<DIM>(x, qc, pslc, offR, dtdx, qR);
      }
      const int iswap = dir == 0 ? -1 : (dir == 1 ? H::IV : H::IW);
      if (iswap >= 0)
      {
        double t = qL[H::IU];
        qL[H::IU] = qL[iswap];
        qL[iswap] = t;
        t = qR[H::IU];
        qR[H::IU] = qR[iswap];
        qR[iswap] = t;
      }
      double flux[H::NV], us, ph0, ph1;
      riemann_hllc<DIM>(qL, qR, x.s, flux, us, ph0, ph1);
      if (iswap >= 0)
      {
        const double t = flux[H::IU];
        flux[H::IU] = flux[iswap];
        flux[iswap] = t;
      }
      flux[H::IA0] = us * ph0;
      flux[H::IA1] = us * ph1;
      for (int v = 0; v < H::NV; ++v)
        x.flux[((size_t)n * H::NV + v) * nf + fc] = flux[v] * dtdx;
      x.ustar[(size_t)n * nf + fc] = us * dtdx;
    }
  }
}

/* sum of the 2^(dim-1) fine face values adjacent to the coarse cell
 * (get_flux_from_fine_neighbor / compute_face_siblings_sum,
 * scheme/ReadFluxesAndConservativeUpdateFunctor.h:256-307).  side = -1:
 * fine neighbour on the min face (its right faces are used). */
template <int DIM>
static double
fine_face_sum(const Ctx & x, int n, const int * cell, int dir, int side, const double * arr, int nvars, int var)
{
  const Geo<DIM> geo(x.b);
  const int      b = x.b;
  int            d[3] = { 0, 0, 0 };
  d[dir] = side;
  const int       s = slot_index(DIM, d);
  const int32_t * nb = &x.nbr[((size_t)n * x.ns + s) * x.nc];
  // coarse-equivalent coordinates of the cell inside the virtual neighbour
  int vcoord[3] = { cell[0], cell[1], cell[2] };
  vcoord[dir] = side < 0 ? b - 1 : 0;
  int ch[3] = { 0, 0, 0 }, fl[3] = { 0, 0, 0 };
  for (int e = 0; e < DIM; ++e)
  {
    int f = 2 * vcoord[e];
    if (e == dir && side < 0)
      f += 1;
    ch[e] = f / b;
    fl[e] = f - ch[e] * b;
  }
  const int child = DIM == 2 ? ch[0] + 2 * ch[1] : ch[0] + 2 * ch[1] + 4 * ch[2];
  const int F = nb[child];
  const int nf = geo.nflux(dir);
  double    sum = 0.0;
  const int e1 = dir == 0 ? 1 : 0;
  const int e2 = DIM == 3 ? (dir == 2 ? 1 : 2) : -1;
  for (int o2 = 0; o2 < (DIM == 3 ? 2 : 1); ++o2)
    for (int o1 = 0; o1 < 2; ++o1)
    {
      int fc[3] = { fl[0], fl[1], fl[2] };
      fc[e1] += o1;
      if (e2 >= 0)
        fc[e2] += o2;
      fc[dir] = side < 0 ? b : 0; // right face of the last fine cell / left face of the first
      const int idx = geo.flux(dir, fc[0], fc[1], fc[2]);
      sum += arr[((size_t)F * nvars + var) * nf + idx];
    }
  return sum;
}

template <int DIM>
static void
read_fluxes_and_update(Ctx & x, const double * Uin, double * Uout, int dir)
{
  using H = Ids<DIM>;
  const Geo<DIM> geo(x.b);
  const int      nc = geo.ncell(), nf = geo.nflux(dir), b = x.b;
  const double   volume_ratio = (double)(1 << DIM);
#pragma omp parallel for schedule(static) num_threads(x.nthreads)
  for (int n = 0; n < x.n_owned; ++n)
  {
    int dmin[3] = { 0, 0, 0 }, dmax[3] = { 0, 0, 0 };
    dmin[dir] = -1;
    dmax[dir] = 1;
    const bool finer_min = x.nbr_rel[(size_t)n * x.ns + slot_index(DIM, dmin)] == 1;
    const bool finer_max = x.nbr_rel[(size_t)n * x.ns + slot_index(DIM, dmax)] == 1;
    for (int c = 0; c < nc; ++c)
    {
      const int cell[3] = { c % b, (c / b) % b, DIM == 3 ? c / (b * b) : 0 };
      auto      U_in = [&](int var) { return Uin[((size_t)n * H::NV + var) * nc + c]; };
      double *  Uo = Uout + (size_t)n * H::NV * nc + c;
      double    st0 = 1.0, st1 = 1.0;
      if (x.prm.source_term == 1)
      {
        // get_source_term_factor (MILLER_PUCKETT), .h:412-443
        double u[H::NV];
        for (int v = 0; v < H::NV; ++v)
          u[v] = U_in(v);
        const double pressure = compute_mixture_pressure<DIM>(u, x.s);
        const double kbar = mixture_bulk_modulus(x.s, pressure, u[H::IA0], u[H::IA1], u[H::IAD0], u[H::IAD1]);
        st0 = 1.0 - kbar / material_bulk_modulus(x.s, 0, pressure, u[H::IA0], u[H::IAD0]);
        st1 = 1.0 - kbar / material_bulk_modulus(x.s, 1, pressure, u[H::IA1], u[H::IAD1]);
      }
      double acc[H::NV];
      for (int v = 0; v < H::NV; ++v)
        acc[v] = 0.0;
      const int  o[3] = { dir == 0, dir == 1, dir == 2 };
      const int  lf = geo.flux(dir, cell[0], cell[1], cell[2]);
      const int  rf = geo.flux(dir, cell[0] + o[0], cell[1] + o[1], cell[2] + o[2]);
      const int  fvars[8] = { H::IAD0, H::IAD1, H::IA0, H::IA1, H::IP, H::IU, H::IV, H::IW };
      const int  nfv = DIM == 2 ? 7 : 8;
      // left coming flux
      if (cell[dir] == 0 && finer_min)
      {
        for (int t = 0; t < nfv; ++t)
          acc[fvars[t]] = acc[fvars[t]] + fine_face_sum<DIM>(x, n, cell, dir, -1, x.flux.data(), H::NV, fvars[t]) / volume_ratio;
        const double us = fine_face_sum<DIM>(x, n, cell, dir, -1, x.ustar.data(), 1, 0);
        acc[H::IA0] -= st0 * us * U_in(H::IA0) / volume_ratio;
        acc[H::IA1] -= st1 * us * U_in(H::IA1) / volume_ratio;
      }
      else
      {
        for (int t = 0; t < nfv; ++t)
          acc[fvars[t]] = acc[fvars[t]] + x.flux[((size_t)n * H::NV + fvars[t]) * nf + lf];
        const double us = x.ustar[(size_t)n * nf + lf];
        acc[H::IA0] -= st0 * us * U_in(H::IA0);
        acc[H::IA1] -= st1 * us * U_in(H::IA1);
      }
      // right coming flux
      if (cell[dir] == b - 1 && finer_max)
      {
        for (int t = 0; t < nfv; ++t)
          acc[fvars[t]] = acc[fvars[t]] - fine_face_sum<DIM>(x, n, cell, dir, +1, x.flux.data(), H::NV, fvars[t]) / volume_ratio;
        const double us = fine_face_sum<DIM>(x, n, cell, dir, +1, x.ustar.data(), 1, 0);
        acc[H::IA0] += st0 * us * U_in(H::IA0) / volume_ratio;
        acc[H::IA1] += st1 * us * U_in(H::IA1) / volume_ratio;
      }
      else
      {
        for (int t = 0; t < nfv; ++t)
          acc[fvars[t]] = acc[fvars[t]] - x.flux[((size_t)n * H::NV + fvars[t]) * nf + rf];
        const double us = x.ustar[(size_t)n * nf + rf];
        acc[H::IA0] += st0 * us * U_in(H::IA0);
        acc[H::IA1] += st1 * us * U_in(H::IA1);
      }
      // update_U, .h:319-393
      const double eps = 1e-12;
      auto         V = [&](int var) -> double & { return Uo[(size_t)var * nc]; };
      V(H::IAD0) += acc[H::IAD0];
      if (V(H::IAD0) < eps)
        V(H::IAD0) = 0.0;
      V(H::IAD1) += acc[H::IAD1];
      if (V(H::IAD1) < eps)
        V(H::IAD1) = 0.0;
      V(H::IA0) += acc[H::IA0];
      if (V(H::IA0) < eps)
        V(H::IA0) = 0.0;
      if (V(H::IA0) > 1.0 - eps)
        V(H::IA0) = 1.0;
      V(H::IA1) += acc[H::IA1];
      if (V(H::IA1) < eps)
        V(H::IA1) = 0.0;
      if (V(H::IA1) > 1.0 - eps)
        V(H::IA1) = 1.0;
      V(H::IP) += acc[H::IP];
      V(H::IU) += acc[H::IU];
      V(H::IV) += acc[H::IV];
      if (DIM == 3)
        V(H::IW) += acc[H::IW];
    }
  }
}

template <int DIM>
static void
fix_volume_fractions(Ctx & x, double * U) // FixVolumeFractionsNormalization.cpp:49-72
{
  using H = Ids<DIM>;
  const int nc = Geo<DIM>(x.b).ncell();
#pragma omp parallel for schedule(static) num_threads(x.nthreads)
  for (int n = 0; n < x.n_owned; ++n)
    for (int c = 0; c < nc; ++c)
    {
      auto V = [&](int var) -> double & { return U[((size_t)n * H::NV + var) * nc + c]; };
      const double sum_alpha = V(H::IA0) + V(H::IA1);
      const double sum_alpha_rho = V(H::IAD0) + V(H::IAD1);
      const double one_over_sum_alpha = 1.0 / sum_alpha;
      V(H::IA0) *= one_over_sum_alpha;
      V(H::IA1) *= one_over_sum_alpha;
      V(H::ID) = sum_alpha_rho;
    }
}

template <int DIM>
static int
do_step(Ctx & x, const double * U, double * U2, const double * dt)
{
  using H = Ids<DIM>;
  const Geo<DIM> geo(x.b);
  const size_t   owned = (size_t)x.n_owned * H::NV * geo.ncell();
  // U2 starts as a copy of U (SolverGodunovFiveEq.cpp:168,494)
  memcpy(U2, U, owned * sizeof(double));
  convert_to_primitives<DIM>(x, U);
  compute_limited_slopes<DIM>(x);
  for (int dir = 0; dir < DIM; ++dir)
  {
    compute_fluxes_and_store<DIM>(x, dir, dt);
    read_fluxes_and_update<DIM>(x, U, U2, dir);
  }
  fix_volume_fractions<DIM>(x, U2);
  return 0;
}

template <int DIM>
static int
do_inv_dt(Ctx & x, const double * U, double * inv_dt) // ComputeDtFiveEqFunctor.cpp:87-134
{
  using H = Ids<DIM>;
  const int nc = Geo<DIM>(x.b).ncell();
  for (int i = 0; i < x.n_inst; ++i)
    inv_dt[i] = 0.0;
  std::vector<double> per_block(x.n_owned, 0.0);
#pragma omp parallel for schedule(static) num_threads(x.nthreads)
  for (int n = 0; n < x.n_owned; ++n)
  {
    const double dx = x.prm.level_dx[x.level[n]];
    double       m = 0.0;
    for (int c = 0; c < nc; ++c)
    {
      double u[H::NV], q[H::NV];
      load_u<DIM>(x, U, n, c, u);
      const double cs = computePrimitives<DIM>(u, q, x.s);
      const double vx = cs + fabs(q[H::IU]);
      const double vy = cs + fabs(q[H::IV]);
      if (DIM == 2)
        m = fmax(m, vx / dx + vy / dx);
      else
      {
        const double vz = cs + fabs(q[H::IW]);
        m = fmax(m, vx / dx + vy / dx + vz / dx);
      }
    }
    per_block[n] = m;
  }
  for (int n = 0; n < x.n_owned; ++n)
  {
    const int i = x.inst.empty() ? 0 : x.inst[n];
    inv_dt[i] = fmax(inv_dt[i], per_block[n]);
  }
  return 0;
}

/* FillOutsideCellFunctor::operator() (border_conditions/FillOutside.cpp:71-170) */
template <int DIM>
static int
do_fill_outside(Ctx & x, double * U)
{
  using H = Ids<DIM>;
  const Geo<DIM> geo(x.b);
  const int      nc = geo.ncell(), b = x.b;
#pragma omp parallel for schedule(static) num_threads(x.nthreads)
  for (int o = 0; o < x.n_outside; ++o)
  {
    const int n_out = x.n_owned + o;
    const int n_in = x.out_src[o];
    for (int c = 0; c < nc; ++c)
    {
      const int co[3] = { c % b, (c / b) % b, DIM == 3 ? c / (b * b) : 0 };
      for (int face = 0; face < 2 * DIM; ++face)
      {
        const int dir = face / 2;
        if (!(x.out_border[(size_t)o * 6 + face] && x.out_normal[(size_t)o * 3 + dir] != 0))
          continue;
        const int bc = x.prm.bc[face];
        int       ci[3] = { co[0], co[1], co[2] };
        if (bc == 2) // ZERO_GRADIENT
          ci[dir] = (face % 2 == 0) ? 0 : b - 1;
        else if (bc == 3) // WALL
          ci[dir] = b - 1 - co[dir];
        else
          continue;
        const int cin = geo.cell(ci[0], ci[1], ci[2]);
        for (int v = 0; v < H::NV; ++v)
          U[((size_t)n_out * H::NV + v) * nc + c] = U[((size_t)n_in * H::NV + v) * nc + cin];
        if (bc == 3)
          U[((size_t)n_out * H::NV + H::IU + dir) * nc + c] *= -1;
      }
    }
  }
  return 0;
}

/* ComputeRefineFlags (scheme/ComputeRefineFlags.cpp:66-368) */
template <int DIM>
static double
neighbor_same_level(const Ctx & x, const double * U, int n, const int * cell, int dir, int side, int var)
{
  using H = Ids<DIM>;
  const Geo<DIM> geo(x.b);
  const int      b = x.b, nc = geo.ncell();
  int            g[3] = { cell[0], cell[1], cell[2] };
  g[dir] += side;
  if (g[dir] >= 0 && g[dir] < b)
    return U[((size_t)n * H::NV + var) * nc + geo.cell(g[0], g[1], g[2])];
  int d[3] = { 0, 0, 0 }, v[3] = { g[0], g[1], g[2] };
  d[dir] = side;
  v[dir] = g[dir] - side * b;
  const int       s = slot_index(DIM, d);
  const int       rel = x.nbr_rel[(size_t)n * x.ns + s];
  const int32_t * nb = &x.nbr[((size_t)n * x.ns + s) * x.nc];
  const int       first = nb[0];
  if (rel <= 0 && first >= x.n_owned) // outside the domain: value of the current cell
    return U[((size_t)n * H::NV + var) * nc + geo.cell(cell[0], cell[1], cell[2])];
  if (rel == 0)
    return U[((size_t)first * H::NV + var) * nc + geo.cell(v[0], v[1], v[2])];
  if (rel < 0)
  {
    int cc[3] = { 0, 0, 0 };
    for (int e = 0; e < DIM; ++e)
    {
      const int vc = x.coord[(size_t)n * 3 + e] + d[e];
      cc[e] = (vc & 1) * (b / 2) + (v[e] >> 1);
    }
    return U[((size_t)first * H::NV + var) * nc + geo.cell(cc[0], cc[1], cc[2])];
  }
  int f0[3] = { 0, 0, 0 }, ch[3] = { 0, 0, 0 };
  for (int e = 0; e < DIM; ++e)
  {
    const int f = 2 * v[e];
    ch[e] = f / b;
    f0[e] = f - ch[e] * b;
  }
  const int child = DIM == 2 ? ch[0] + 2 * ch[1] : ch[0] + 2 * ch[1] + 4 * ch[2];
  const int F = nb[child];
  if (F >= x.n_owned)
    return U[((size_t)n * H::NV + var) * nc + geo.cell(cell[0], cell[1], cell[2])];
  double sum = 0.0;
  for (int oz = 0; oz < (DIM == 3 ? 2 : 1); ++oz)
    for (int oy = 0; oy < 2; ++oy)
      for (int ox = 0; ox < 2; ++ox)
        sum += U[((size_t)F * H::NV + var) * nc + geo.cell(f0[0] + ox, f0[1] + oy, DIM == 3 ? f0[2] + oz : 0)];
  return sum / (double)(1 << DIM);
}

static inline double
normalized_gradient(double v1, double v2)
{
  double vmax = fmax(fabs(v1), fabs(v2));
  if (vmax < 0.001)
    return 0.0;
  vmax = fabs(v1 - v2) / vmax;
  return fmax(fmin(vmax, 1.0), 0.0);
}

template <int DIM>
static int
do_refine_flags(Ctx &          x,
                const double * U,
                int            indicator,
                double         eps_r,
                double         eps_c,
                double         eps_l,
                int            lmin,
                int            lmax,
                int8_t *       flags)
{
  using H = Ids<DIM>;
  const Geo<DIM> geo(x.b);
  const int      nc = geo.ncell(), b = x.b;
#pragma omp parallel for schedule(static) num_threads(x.nthreads)
  for (int n = 0; n < x.n_owned; ++n)
  {
    const int lev = x.level[n];
    int       bflag = -1;
    for (int c = 0; c < nc; ++c)
    {
      const int cell[3] = { c % b, (c / b) % b, DIM == 3 ? c / (b * b) : 0 };
      int       flag = -1;
      auto      update_flag = [&](double ind) {
        int f;
        if (lev < lmax && ind > eps_r)
          f = 2;
        else if (lev > lmin && ind < eps_c)
          f = 0;
        else
          f = 1;
        flag = flag > f ? flag : f;
      };
      const int vars[2] = { H::IAD0, H::IAD1 };
      if (indicator == 2)
      {
        // LOHNER_SPLIT: per direction, var IAD0 then IAD1
        for (int t = 0; t < 2; ++t)
          for (int d = 0; d < DIM; ++d)
          {
            const int    var = vars[t];
            const double L = neighbor_same_level<DIM>(x, U, n, cell, d, -1, var);
            const double R = neighbor_same_level<DIM>(x, U, n, cell, d, +1, var);
            const double C = U[((size_t)n * H::NV + var) * nc + c];
            update_flag(fabs(L - 2 * C + R) / (fabs(R - C) + fabs(C - L) + eps_l * (fabs(L) + 2 * fabs(C) + fabs(R))));
          }
      }
      else
      {
        for (int t = 0; t < 2; ++t)
        {
          const int    var = vars[t];
          const double C = U[((size_t)n * H::NV + var) * nc + c];
          if (indicator == 1)
          {
            double num = 0.0, den = 0.0;
            for (int d = 0; d < DIM; ++d)
            {
              const double L = neighbor_same_level<DIM>(x, U, n, cell, d, -1, var);
              const double R = neighbor_same_level<DIM>(x, U, n, cell, d, +1, var);
              const double a = L - 2 * C + R;
              if (d == 0)
                num = a * a;
              else
                num += a * a;
              const double tmp = fabs(R - C) + fabs(C - L) + eps_l * (fabs(L) + 2 * fabs(C) + fabs(R));
              if (d == 0)
                den = tmp * tmp;
              else
                den += tmp * tmp;
            }
            update_flag(sqrt(num / den));
          }
          else
          {
            double res = -1.7976931348623157e308;
            for (int d = 0; d < DIM; ++d)
            {
              const double L = neighbor_same_level<DIM>(x, U, n, cell, d, -1, var);
              const double R = neighbor_same_level<DIM>(x, U, n, cell, d, +1, var);
              res = fmax(res, normalized_gradient(C, L));
              res = fmax(res, normalized_gradient(C, R));
            }
            update_flag(res);
          }
        }
      }
      bflag = bflag > flag ? bflag : flag;
    }
    flags[n] = (int8_t)bflag;
  }
  return 0;
}

} // namespace

/* ---------------------------------------------------------------------------
 * C API
 * ------------------------------------------------------------------------- */
extern "C" void *
g5o_create(const G5OMesh * mesh, const G5OParams * prm, int nthreads)
{
  if (!mesh || !prm || (prm->dim != 2 && prm->dim != 3) || prm->b < 4 || (prm->b % 2) != 0)
    return nullptr;
  Ctx * x = new Ctx;
  x->prm = *prm;
  x->s = make_settings(prm);
  x->dim = prm->dim;
  x->b = prm->b;
  x->nv = prm->dim == 2 ? 8 : 9;
  x->ns = prm->dim == 2 ? 9 : 27;
  x->nc = prm->dim == 2 ? 4 : 8;
#ifdef _OPENMP
  x->nthreads = nthreads > 0 ? nthreads : omp_get_max_threads();
#else
  (void)nthreads;
  x->nthreads = 1;
#endif
  x->n_owned = mesh->n_owned;
  x->n_outside = mesh->n_outside;
  x->n_total = mesh->n_owned + mesh->n_outside;
  x->n_inst = mesh->n_inst > 0 ? mesh->n_inst : 1;
  x->level.assign(mesh->level, mesh->level + x->n_total);
  x->coord.assign(mesh->coord, mesh->coord + (size_t)x->n_total * 3);
  x->nbr.assign(mesh->nbr, mesh->nbr + (size_t)x->n_owned * x->ns * x->nc);
  x->nbr_rel.assign(mesh->nbr_rel, mesh->nbr_rel + (size_t)x->n_owned * x->ns);
  if (x->n_outside > 0)
  {
    x->out_src.assign(mesh->out_src, mesh->out_src + x->n_outside);
    x->out_normal.assign(mesh->out_normal, mesh->out_normal + (size_t)x->n_outside * 3);
    x->out_border.assign(mesh->out_border, mesh->out_border + (size_t)x->n_outside * 6);
  }
  if (mesh->inst)
    x->inst.assign(mesh->inst, mesh->inst + x->n_total);
  const size_t b = x->b;
  const size_t ng = prm->dim == 2 ? (b + 4) * (b + 4) : (b + 4) * (b + 4) * (b + 4);
  const size_t ns = prm->dim == 2 ? (b + 2) * (b + 2) : (b + 2) * (b + 2) * (b + 2);
  const size_t nf = prm->dim == 2 ? (b + 1) * b : (b + 1) * b * b;
  x->Q.assign((size_t)x->n_owned * x->nv * ng, 0.0);
  for (int d = 0; d < prm->dim; ++d)
    x->slopes[d].assign((size_t)x->n_owned * x->nv * ns, 0.0);
  x->flux.assign((size_t)x->n_owned * x->nv * nf, 0.0);
  x->ustar.assign((size_t)x->n_owned * nf, 0.0);
  return x;
}

extern "C" void
g5o_destroy(void * ctx)
{
  delete static_cast<Ctx *>(ctx);
}

/* conservative state that the ghost fill of owned block n gives ghosted cell
 * g (block cell coordinates, -2 .. b+1; g[2] = 0 in 2D) before the
 * conversion to primitives */
extern "C" int
g5o_ghost_state(void * ctx, const double * U, int n, const int * g, double * u)
{
  Ctx * x = static_cast<Ctx *>(ctx);
  if (n < 0 || n >= x->n_owned)
    return -1;
  for (int e = 0; e < x->dim; ++e)
    if (g[e] < -2 || g[e] >= x->b + 2)
      return -1;
  if (x->dim == 2)
    ghost_state<2>(*x, U, n, g, u, x->prm.prolongation);
  else
    ghost_state<3>(*x, U, n, g, u, x->prm.prolongation);
  return 0;
}

extern "C" int
g5o_step(void * ctx, const double * U, double * U2, const double * dt)
{
  Ctx * x = static_cast<Ctx *>(ctx);
  return x->dim == 2 ? do_step<2>(*x, U, U2, dt) : do_step<3>(*x, U, U2, dt);
}

extern "C" int
g5o_inv_dt(void * ctx, const double * U, double * inv_dt)
{
  Ctx * x = static_cast<Ctx *>(ctx);
  return x->dim == 2 ? do_inv_dt<2>(*x, U, inv_dt) : do_inv_dt<3>(*x, U, inv_dt);
}

extern "C" int
g5o_fill_outside(void * ctx, double * U)
{
  Ctx * x = static_cast<Ctx *>(ctx);
  return x->dim == 2 ? do_fill_outside<2>(*x, U) : do_fill_outside<3>(*x, U);
}

extern "C" int
g5o_refine_flags(void *         ctx,
                 const double * U,
                 int            indicator,
                 double         eps_refine,
                 double         eps_coarsen,
                 double         eps_lohner,
                 int            level_min,
                 int            level_max,
                 int8_t *       flags)
{
  Ctx * x = static_cast<Ctx *>(ctx);
  return x->dim == 2 ? do_refine_flags<2>(*x, U, indicator, eps_refine, eps_coarsen, eps_lohner, level_min, level_max, flags)
                     : do_refine_flags<3>(*x, U, indicator, eps_refine, eps_coarsen, eps_lohner, level_min, level_max, flags);
}

extern "C" double
g5o_compute_primitives(const G5OParams * prm, const double * u, double * q)
{
  const Settings s = make_settings(prm);
  return prm->dim == 2 ? computePrimitives<2>(u, q, s) : computePrimitives<3>(u, q, s);
}

extern "C" void
g5o_riemann_hllc(const G5OParams * prm, const double * qL, const double * qR, double * out)
{
  const Settings s = make_settings(prm);
  const int      nv = prm->dim == 2 ? 8 : 9;
  if (prm->dim == 2)
    riemann_hllc<2>(qL, qR, s, out, out[nv], out[nv + 1], out[nv + 2]);
  else
    riemann_hllc<3>(qL, qR, s, out, out[nv], out[nv + 1], out[nv + 2]);
}

extern "C" double
g5o_slope(const G5OParams * prm, double q, double qp, double qm)
{
  return slope_unsplit_scalar(q, qp, qm, prm->slope_type);
}

extern "C" double
g5o_tanh(double x)
{
  return g5_tanh(x);
}

extern "C" double
g5o_mixture_pressure(const G5OParams * prm, double rho, double eint, double a0, double ar0, double ar1)
{
  const Settings s = make_settings(prm);
  return mixture_pressure(s, rho, eint, a0, 1.0 - a0, ar0, ar1);
}

extern "C" double
g5o_mixture_sound_speed(const G5OParams * prm, double rho, double p, double a0, double ar0, double ar1)
{
  const Settings s = make_settings(prm);
  return mixture_sound_speed(s, rho, p, a0, 1.0 - a0, ar0, ar1);
}

/* ---------------------------------------------------------------------------
 * Block remap after a mesh adaptation (UserDataRemapper::remap_block_data,
 * called from SolverGodunovFiveEq::map_userdata_after_adapt,
 * SolverGodunovFiveEq.cpp:1137-1169; the remapper is external to the
 * reference and restated here with the reference's own ghost-cell rules):
 *   kept block      -> copy;
 *   refined block   -> SIMPLE_COPY prolongation: each fine cell takes the
 *                      parent cell containing its centre (all variables);
 *   coarsened block -> restriction of get_conservative_vars_restriction
 *                      (scheme/ConvertToPrimitivesVariablesFunctor.cpp:208-246):
 *                      mean of the 2^dim fine cells for IE IU IV (IW) IAD0
 *                      IAD1 IA0 (sum in z, y, x order, then / 2^dim),
 *                      IA1 = 1 - IA0, ID = IAD0 + IAD1.
 * ------------------------------------------------------------------------- */
template <int DIM>
static int
do_remap(int b, int n_new, const int8_t * kind, const int32_t * src, const double * Uold, double * Unew)
{
  using H = Ids<DIM>;
  const Geo<DIM> geo(b);
  const int      nc = geo.ncell();
  const int      nch = 1 << DIM;
#pragma omp parallel for schedule(static)
  for (int j = 0; j < n_new; ++j)
  {
    const int32_t * s = src + (size_t)j * nch;
    double *        out = Unew + (size_t)j * H::NV * nc;
    for (int kk = 0; kk < (DIM == 3 ? b : 1); ++kk)
      for (int jj = 0; jj < b; ++jj)
        for (int ii = 0; ii < b; ++ii)
        {
          const int c = geo.cell(ii, jj, kk);
          const int cc[3] = { ii, jj, kk };
          if (kind[j] == 0)
          {
            for (int v = 0; v < H::NV; ++v)
              out[v * nc + c] = Uold[((size_t)s[0] * H::NV + v) * nc + c];
          }
          else if (kind[j] == 1)
          {
            int pc[3] = { 0, 0, 0 };
            for (int e = 0; e < DIM; ++e)
              pc[e] = ((s[1] >> e) & 1) * (b / 2) + (cc[e] >> 1);
            const int cp = geo.cell(pc[0], pc[1], pc[2]);
            for (int v = 0; v < H::NV; ++v)
              out[v * nc + c] = Uold[((size_t)s[0] * H::NV + v) * nc + cp];
          }
          else
          {
            int f0[3] = { 0, 0, 0 }, ch[3] = { 0, 0, 0 };
            for (int e = 0; e < DIM; ++e)
            {
              const int f = 2 * cc[e];
              ch[e] = f / b;
              f0[e] = f - ch[e] * b;
            }
            const int F = s[ch[0] + 2 * ch[1] + 4 * ch[2]];
            const int vars[7] = { H::IE, H::IU, H::IV, H::IW, H::IAD0, H::IAD1, H::IA0 };
            for (int t = 0; t < 7; ++t)
            {
              if (DIM == 2 && t == 3)
                continue;
              const int v = vars[t];
              double    sum = 0.0;
              for (int oz = 0; oz < (DIM == 3 ? 2 : 1); ++oz)
                for (int oy = 0; oy < 2; ++oy)
                  for (int ox = 0; ox < 2; ++ox)
                    sum += Uold[((size_t)F * H::NV + v) * nc + geo.cell(f0[0] + ox, f0[1] + oy, DIM == 3 ? f0[2] + oz : 0)];
              out[v * nc + c] = sum / (double)(1 << DIM);
            }
            out[H::IA1 * nc + c] = 1.0 - out[H::IA0 * nc + c];
            out[H::ID * nc + c] = out[H::IAD0 * nc + c] + out[H::IAD1 * nc + c];
          }
        }
  }
  return 0;
}

extern "C" int
g5o_remap(const G5OParams * prm, int n_new, const int8_t * kind, const int32_t * src, const double * Uold, double * Unew)
{
  return prm->dim == 2 ? do_remap<2>(prm->b, n_new, kind, src, Uold, Unew) : do_remap<3>(prm->b, n_new, kind, src, Uold, Unew);
}

/* refined blocks prolonged with the context's prolongation over the old
 * mesh (the context's mesh): each fine cell from its parent cell and the
 * parent's neighbours at the old level (the stencil the UserDataRemapper
 * keeps the old orchard keys for, SolverGodunovFiveEq.cpp:286-289) */
template <int DIM>
static void
do_remap_refined(const Ctx & x, int n_new, const int8_t * kind, const int32_t * src, const double * Uold, double * Unew)
{
  using H = Ids<DIM>;
  const Geo<DIM> geo(x.b);
  const int      nc = geo.ncell(), nch = 1 << DIM, h = x.b / 2;
#pragma omp parallel for schedule(static)
  for (int j = 0; j < n_new; ++j)
  {
    if (kind[j] != 1)
      continue;
    const int32_t * s = src + (size_t)j * nch;
    double *        out = Unew + (size_t)j * H::NV * nc;
    for (int c = 0; c < nc; ++c)
    {
      const int cc[3] = { c % x.b, (c / x.b) % x.b, DIM == 3 ? c / (x.b * x.b) : 0 };
      int       q[3] = { 0, 0, 0 }, pos[3] = { 0, 0, 0 };
      for (int e = 0; e < DIM; ++e)
      {
        q[e] = ((s[1] >> e) & 1) * h + (cc[e] >> 1);
        pos[e] = cc[e] & 1;
      }
      double u[H::NV];
      prolong_point<DIM>(
        x.prm.prolongation, [&](const int * qq, int var) { return level_cell_value<DIM>(x, Uold, s[0], qq, var); }, q, pos, u);
      for (int v = 0; v < H::NV; ++v)
        out[(size_t)v * nc + c] = u[v];
    }
  }
}

extern "C" int
g5o_remap_mesh(void * ctx, int n_new, const int8_t * kind, const int32_t * src, const double * Uold, double * Unew)
{
  Ctx * x = static_cast<Ctx *>(ctx);
  const int rc = g5o_remap(&x->prm, n_new, kind, src, Uold, Unew);
  if (rc != 0 || x->prm.prolongation == 0)
    return rc;
  for (int j = 0; j < n_new; ++j)
    if (kind[j] == 1 && (src[(size_t)j << x->dim] < 0 || src[(size_t)j << x->dim] >= x->n_owned))
      return -1;
  if (x->dim == 2)
    do_remap_refined<2>(*x, n_new, kind, src, Uold, Unew);
  else
    do_remap_refined<3>(*x, n_new, kind, src, Uold, Unew);
  return 0;
}

/* ---------------------------------------------------------------------------
 * ComputeDerivedQuantities::run (utils/ComputeDerivedQuantities.h:96-180):
 * quantity per cell of blocks [begin, begin + count); out[n_blocks][ncell].
 * ------------------------------------------------------------------------- */
template <int DIM>
static int
do_derived(const G5OParams * prm, const double * U, int quantity, long long begin, long long count, double * out)
{
  using H = Ids<DIM>;
  const Settings s = make_settings(prm);
  const int      b = prm->b;
  const int      nc = DIM == 2 ? b * b : b * b * b;
#pragma omp parallel for schedule(static)
  for (long long oct = begin; oct < begin + count; ++oct)
    for (int c = 0; c < nc; ++c)
    {
      double u[H::NV];
      for (int v = 0; v < H::NV; ++v)
        u[v] = U[(oct * H::NV + v) * nc + c];
      double q[H::NV];
      const double cs = computePrimitives<DIM>(u, q, s);
      double       r = 0.0;
      switch (quantity)
      {
      case 0: r = u[H::ID]; break;
      case 1: r = compute_mixture_pressure<DIM>(u, s); break;
      case 2: r = cs; break;
      case 3: r = compute_mixture_ekin<DIM>(u, s); break;
      case 4:
      {
        double un = q[H::IU] * q[H::IU] + q[H::IV] * q[H::IV];
        if (DIM == 3)
          un += q[H::IW] * q[H::IW];
        un = sqrt(un);
        r = un / cs;
        break;
      }
      case 5: r = q[H::IU]; break;
      case 6: r = q[H::IV]; break;
      default: r = DIM == 3 ? q[H::IW] : 0.0; break;
      }
      out[oct * nc + c] = r;
    }
  return 0;
}

extern "C" int
g5o_derived(const G5OParams * prm, const double * U, int quantity, long long begin, long long count, double * out)
{
  return prm->dim == 2 ? do_derived<2>(prm, U, quantity, begin, count, out) : do_derived<3>(prm, U, quantity, begin, count, out);
}
