// g5_phys.h — device parameter block from the C-ABI parameters (shared by
// the context entry points and the allocation-free step).
#pragma once

#include <cstring>

#include "../../include/g5gpu.h"
#include "g5_common.cuh"

namespace g5
{

// whether the law kinds and their parameters are usable (reference densities
// and Grueneisen coefficients positive)
inline bool
eos_params_valid(const G5Params * prm)
{
  for (int k = 0; k < 2; ++k)
  {
    const int kind = prm->eos[k];
    if (kind < G5_EOS_STIFFENED || kind > G5_EOS_SHOCKWAVE2)
      return false;
    if (kind != G5_EOS_STIFFENED && !(prm->mg[k][0] > 0.0 && prm->mg[k][1] > 0.0))
      return false;
  }
  return true;
}

inline PhysParams
make_phys(const G5Params * params)
{
  PhysParams p;
  std::memset(&p, 0, sizeof(p));
  p.smallr = params->smallr;
  p.smallc = params->smallc;
  p.smallp = params->smallc * params->smallc;
  p.slope_type = params->slope_type;
  for (int k = 0; k < 2; ++k)
  {
    p.gamma[k] = params->gamma[k];
    p.pinf[k] = params->pinf[k];
    p.xi[k] = 1.0 / (params->gamma[k] - 1.0);
    p.gpx[k] = params->gamma[k] * params->pinf[k] * p.xi[k];
  }
  p.cfl = params->cfl;
  p.thinc_beta = params->thinc_beta;
  p.thinc_eps = params->thinc_eps;
  p.integrator = params->integrator;
  p.thinc = params->thinc;
  p.source_term = params->source_term;
  for (int f = 0; f < 6; ++f)
    p.bc[f] = params->bc[f];
  for (int l = 0; l < 32; ++l)
    p.level_dx[l] = params->level_dx[l];
  p.f_smallr = (float)p.smallr;
  p.f_smallc = (float)p.smallc;
  p.f_smallp = (float)p.smallp;
  p.f_slope_type = (float)p.slope_type;
  p.f_thinc_beta = (float)p.thinc_beta;
  p.f_thinc_eps = (float)p.thinc_eps;
  for (int k = 0; k < 2; ++k)
  {
    p.f_xi[k] = (float)p.xi[k];
    p.f_gpx[k] = (float)p.gpx[k];
  }
  p.f_dxi = (float)(p.xi[0] - p.xi[1]);
  p.dgpx = p.gpx[0] - p.gpx[1];
  for (int k = 0; k < 2; ++k)
  {
    p.eos_kind[k] = params->eos[k];
    for (int j = 0; j < 8; ++j)
      p.mg[k][j] = params->mg[k][j];
    p.mg_rho0[k] = params->eos[k] != G5_EOS_STIFFENED ? params->mg[k][0] : 1.0;
  }
  p.mg_any = params->eos[0] != G5_EOS_STIFFENED || params->eos[1] != G5_EOS_STIFFENED;
  p.prolong = params->prolongation;
  return p;
}

} // namespace g5
