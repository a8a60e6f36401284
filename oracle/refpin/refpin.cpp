// refpin.cpp — exposes the reference's own HLLC solver and conservative ->
// primitive conversion (models/RiemannSolvers.h:57-262, models/utils.h:36-250,
// models/HydroSettings.cpp:18-29), compiled from the reference tree against
// the shim headers beside this file, as a C library for generating golden
// vectors (test infrastructure only; never linked by the product).
#include <godunov_five_eq/models/HydroSettings.h>
#include <godunov_five_eq/models/RiemannSolvers.h>
#include <godunov_five_eq/models/utils.h>

#include <string>

using namespace kalypsso;
using namespace kalypsso::godunov_five_eq;

namespace
{
struct Host
{
};

// prm: gamma0, gamma1, pinf0, pinf1, smallr, smallc
ConfigMap
make_config(const double * prm)
{
  ConfigMap c;
  c.set("material0_mie_gruneisen_sg", "gamma", std::to_string(prm[0]));
  c.set("material1_mie_gruneisen_sg", "gamma", std::to_string(prm[1]));
  c.set("material0_mie_gruneisen_sg", "pinf", std::to_string(prm[2]));
  c.set("material1_mie_gruneisen_sg", "pinf", std::to_string(prm[3]));
  c.set("hydro", "riemann", "HLLC");
  return c;
}

template <size_t dim>
void
hllc(const double * prm, const double * ql, const double * qr, double * out)
{
  ConfigMap c = make_config(prm);
  core::eos::MieGruneisenMixture<Host> eos(c);
  // exact parameter values (the ConfigMap round-trips through text)
  for (int k = 0; k < 2; ++k)
  {
    eos.gamma[k] = prm[k];
    eos.pinf[k] = prm[2 + k];
    eos.xi[k] = 1.0 / (eos.gamma[k] - 1.0);
    eos.gpx[k] = eos.gamma[k] * eos.pinf[k] * eos.xi[k];
  }
  HydroSettings s(c);
  s.smallr = prm[4];
  s.smallc = prm[5];
  s.smallp = s.smallc * s.smallc;
  s.smallpp = s.smallr * s.smallp;
  constexpr size_t nv = models::FiveEq<dim>::nbvar();
  HydroState<dim>  qL, qR;
  for (size_t v = 0; v < nv; ++v)
  {
    qL[v] = ql[v];
    qR[v] = qr[v];
  }
  auto r = riemann_hydro<dim>(qL, qR, s, eos);
  for (size_t v = 0; v < nv; ++v)
    out[v] = r.flux[v];
  out[nv] = r.ustar;
  out[nv + 1] = r.phistar0;
  out[nv + 2] = r.phistar1;
}

template <size_t dim>
double
prim(const double * prm, const double * u, double * q)
{
  ConfigMap c = make_config(prm);
  core::eos::MieGruneisenMixture<Host> eos(c);
  for (int k = 0; k < 2; ++k)
  {
    eos.gamma[k] = prm[k];
    eos.pinf[k] = prm[2 + k];
    eos.xi[k] = 1.0 / (eos.gamma[k] - 1.0);
    eos.gpx[k] = eos.gamma[k] * eos.pinf[k] * eos.xi[k];
  }
  HydroSettings s(c);
  s.smallr = prm[4];
  s.smallc = prm[5];
  s.smallp = s.smallc * s.smallc;
  constexpr size_t nv = models::FiveEq<dim>::nbvar();
  HydroState<dim>  U, Q;
  for (size_t v = 0; v < nv; ++v)
    U[v] = u[v];
  const double cs = models::computePrimitives<dim>(U, Q, s, eos);
  for (size_t v = 0; v < nv; ++v)
    q[v] = Q[v];
  return cs;
}
} // namespace

extern "C" void
ref_hllc(int dim, const double * prm, const double * ql, const double * qr, double * out)
{
  if (dim == 2)
    hllc<2>(prm, ql, qr, out);
  else
    hllc<3>(prm, ql, qr, out);
}

extern "C" double
ref_prim(int dim, const double * prm, const double * u, double * q)
{
  return dim == 2 ? prim<2>(prm, u, q) : prim<3>(prm, u, q);
}
