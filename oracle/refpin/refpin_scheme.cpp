// refpin_scheme.cpp — one GodunovImplemV0::do_time_step
// (scheme/GodunovImplemV0.cpp:85-151) of a periodic tile of same-level blocks,
// computed by the reference's own scheme functors compiled in place from the
// reference tree:
//   ComputeLimitedSlopesFunctor          scheme/ComputeLimitedSlopesFunctor.cpp:116-193
//   ComputeFluxesAndStoreFunctor         scheme/ComputeFluxesAndStoreFunctor.cpp:126-664
//   ComputeFluxesAndStoreTHINCFunctor    scheme/ComputeFluxesAndStoreTHINCFunctor.cpp:122-788
//   ReadFluxesAndConservativeUpdate...   scheme/ReadFluxesAndConservativeUpdateFunctor.cpp:115-592,
//                                        .h:319-443 (update_U, source-term factor)
//   FixVolumeFractionsNormalization      scheme/FixVolumeFractionsNormalization.cpp:49-72
//   ComputeDtFiveEqFunctor::compute_cfl  scheme/ComputeDtFiveEqFunctor.cpp:87-134
// with the primitive conversion of models/utils.h:200-250.  The ghost fill of a
// same-level neighbour is a copy of its cell converted to primitives and
// stored as set_primitive_vars stores it
// (scheme/ConvertToPrimitivesVariablesFunctor.cpp:251-271, 494-537), restated
// here because the fill's neighbour search lives in the external core.
//
// Test infrastructure only (golden vectors for the CPU oracle); never linked
// by the product.
#include <godunov_five_eq/models/HydroSettings.h>
#include <godunov_five_eq/models/utils.h>
#include <godunov_five_eq/scheme/ComputeDtFiveEqFunctor.h>
#include <godunov_five_eq/scheme/ComputeFluxesAndStoreFunctor.h>
#include <godunov_five_eq/scheme/ComputeFluxesAndStoreTHINCFunctor.h>
#include <godunov_five_eq/scheme/ComputeLimitedSlopesFunctor.h>
#include <godunov_five_eq/scheme/FixVolumeFractionsNormalization.h>
#include <godunov_five_eq/scheme/ReadFluxesAndConservativeUpdateFunctor.h>

#include <cstdio>
#include <string>

using namespace kalypsso;
using namespace kalypsso::godunov_five_eq;

namespace
{
using Dev = kalypsso::DefaultDevice;

// prm: gamma0 gamma1 pinf0 pinf1 smallr smallc slope_type thinc thinc_beta
//      thinc_eps integrator source_term
// a value as text that reads back to the same double
std::string
num(double x)
{
  char buf[40];
  std::snprintf(buf, sizeof(buf), "%.17g", x);
  return buf;
}

ConfigMap
make_config(const double * prm)
{
  ConfigMap c;
  c.set("material0_mie_gruneisen_sg", "gamma", num(prm[0]));
  c.set("material1_mie_gruneisen_sg", "gamma", num(prm[1]));
  c.set("material0_mie_gruneisen_sg", "pinf", num(prm[2]));
  c.set("material1_mie_gruneisen_sg", "pinf", num(prm[3]));
  c.set("hydro", "riemann", "HLLC");
  c.set("THINC", "enabled", prm[7] != 0.0 ? "true" : "false");
  c.set("THINC", "beta", num(prm[8]));
  c.set("THINC", "epsilon", num(prm[9]));
  c.set("refpin", "integrator", std::to_string((int)prm[10]));
  c.set("refpin", "source_term", std::to_string((int)prm[11]));
  return c;
}

template <size_t dim>
int
step(const double * prm, int b, int nb, int level, const double * Uin, double dt, double * Uout, double * inv_dt)
{
  using Hydro = models::FiveEq<dim>;
  constexpr int nv = (int)Hydro::nbvar();
  ConfigMap     cfg = make_config(prm);

  core::eos::MieGruneisenMixture<Dev> eos(cfg);
  for (int k = 0; k < 2; ++k)
  {
    eos.gamma[k] = prm[k];
    eos.pinf[k] = prm[2 + k];
    eos.xi[k] = 1.0 / (eos.gamma[k] - 1.0);
    eos.gpx[k] = eos.gamma[k] * eos.pinf[k] * eos.xi[k];
  }
  HydroSettings s(cfg);
  s.smallr = prm[4];
  s.smallc = prm[5];
  s.smallp = s.smallc * s.smallc;
  s.smallpp = s.smallr * s.smallp;
  s.slope_type = prm[6];

  const int nblocks = dim == 2 ? nb * nb : nb * nb * nb;
  const int ncell = dim == 2 ? b * b : b * b * b;
  const int n = nb * b; // cells per tile edge

  block_size_t<dim> bs;
  for (size_t e = 0; e < dim; ++e)
    bs[e] = b;
  DataArrayBlock<dim, real_t, Dev>        U(bs, nv, nblocks), U2(bs, nv, nblocks);
  DataArrayGhostedBlock<dim, real_t, Dev> Q(bs, 2, nv, nblocks);
  DataArrayGhostedBlock<dim, real_t, Dev> sx(bs, 1, nv, nblocks), sy(bs, 1, nv, nblocks), sz(bs, 1, nv, nblocks);
  for (size_t i = 0; i < (size_t)nblocks * nv * ncell; ++i)
  {
    (*U.s)[i] = Uin[i];
    (*U2.s)[i] = Uin[i]; // U2 starts as a copy of U (SolverGodunovFiveEq.cpp:494)
  }

  // ghosted primitives: every ghosted cell from the cell of the periodic tile it covers
  const int g = 2, gb = b + 2 * g, ngc = dim == 2 ? gb * gb : gb * gb * gb;
  for (int blk = 0; blk < nblocks; ++blk)
  {
    const int bc[3] = { blk % nb, (blk / nb) % nb, dim == 3 ? blk / (nb * nb) : 0 };
    for (int gc = 0; gc < ngc; ++gc)
    {
      int c[3] = { gc % gb - g, (gc / gb) % gb - g, dim == 3 ? gc / (gb * gb) - g : 0 };
      int src_blk = 0, src_cell = 0, mul = 1, cmul = 1;
      for (int e = 0; e < (int)dim; ++e)
      {
        const int gcoord = ((bc[e] * b + c[e]) % n + n) % n;
        src_blk += (gcoord / b) * mul;
        src_cell += (gcoord % b) * cmul;
        mul *= nb;
        cmul *= b;
      }
      HydroState<dim> u, q;
      for (int v = 0; v < nv; ++v)
        u[v] = U(src_cell, v, src_blk);
      models::computePrimitives<dim>(u, q, s, eos);
      Q(gc, Hydro::ID, blk) = q[Hydro::ID];
      Q(gc, Hydro::IAD0, blk) = q[Hydro::IAD0];
      Q(gc, Hydro::IAD1, blk) = q[Hydro::IAD1];
      Q(gc, Hydro::IA0, blk) = q[Hydro::IA0];
      Q(gc, Hydro::IA1, blk) = ONE_F - q[Hydro::IA0];
      Q(gc, Hydro::IP, blk) = q[Hydro::IP];
      Q(gc, Hydro::IU, blk) = q[Hydro::IU];
      Q(gc, Hydro::IV, blk) = q[Hydro::IV];
      if constexpr (dim == 3)
        Q(gc, Hydro::IW, blk) = q[Hydro::IW];
    }
  }

  ComputeLimitedSlopesFunctor<dim, Dev>::apply_on_group(Q, sx, sy, sz, nblocks, s);

  typename orchard_key_base_t<Dev>::view_t keys("keys", nblocks);
  for (int blk = 0; blk < nblocks; ++blk)
    keys(blk) = (uint64_t)level;
  conformal_status_view_t<dim, Dev> conformal("conformal", nblocks); // all faces same level
  AMRMeshInfo                       info(nblocks, 0);
  typename hashmap_base_t<Dev>::map_t hashmap;
  brick_size_t<dim>                 brick;
  Kokkos::Array<bool, dim>          periodic;
  for (size_t e = 0; e < dim; ++e)
  {
    brick[e] = nb;
    periodic[e] = true;
  }
  DataArrayBlock<dim, real_t, Dev> F(bs, nv, nblocks), ustar(bs, 1, nblocks);
  // room for the largest flux shape ((b+1) b^(dim-1) cells)
  F.s->assign((size_t)(b + 1) * ncell / b * nv * nblocks, 0.0);
  ustar.s->assign((size_t)(b + 1) * ncell / b * nblocks, 0.0);
  for (int dir = 0; dir < (int)dim; ++dir)
  {
    F.reshape(get_flux_block_sizes<dim>(bs, dir));
    ustar.reshape(get_flux_block_sizes<dim>(bs, dir));
    if (prm[7] != 0.0)
      ComputeFluxesAndStoreTHINCFunctor<dim, Dev>::apply(cfg, keys, info, F, ustar, Q, sx, sy, sz, 0, nblocks, dir, s, eos, dt);
    else
      ComputeFluxesAndStoreFunctor<dim, Dev>::apply(cfg, keys, info, F, ustar, Q, sx, sy, sz, 0, nblocks, dir, s, eos, dt);
    ReadFluxesAndConservativeUpdateFunctor<dim, Dev>::apply(
      cfg, hashmap, keys, conformal, info, U, U2, F, ustar, dir, brick, periodic, s, eos, dt);
  }
  FixVolumeFractionsNormalization<dim, Dev>::apply(info, U2);

  real_t inv = 0;
  ComputeDtFiveEqFunctor<dim, Dev>::apply(cfg, keys, nblocks, s, bs, U2, eos, inv);
  *inv_dt = inv;
  for (size_t i = 0; i < (size_t)nblocks * nv * ncell; ++i)
    Uout[i] = (*U2.s)[i];
  return 0;
}

} // namespace

extern "C" int
refpin_scheme_step(const double * prm, int dim, int b, int nb, int level, const double * U, double dt, double * U2, double * inv_dt)
{
  if (b < 4 || nb < 1 || level < 0 || level > 30)
    return -1;
  return dim == 2 ? step<2>(prm, b, nb, level, U, dt, U2, inv_dt) : (dim == 3 ? step<3>(prm, b, nb, level, U, dt, U2, inv_dt) : -1);
}
