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

// Block-table check shared by g5_set_mesh and g5_step_static (the reference
// asserts the same facts in StencilHelper and its hashmap lookups): levels in
// range, instance ids below n_inst, relation codes in {-1, 0, 1}, a valid
// block for every coarser or same-level slot and for every child of a finer
// slot that touches the block (the other children may be -1), outside blocks
// mirroring owned ones.  Array presence is the caller's check.  Returns G5_OK
// or G5_ERR_MESH.
inline int
validate_table(int dim, const G5Mesh * m)
{
  const int n_owned = m->n_owned, n_total = m->n_owned + m->n_outside;
  const int n_inst = m->n_inst > 0 ? m->n_inst : 1;
  const int ns = dim == 2 ? 9 : 27, nch = dim == 2 ? 4 : 8, center = dim == 2 ? 4 : 13;
  for (int n = 0; n < n_total; ++n)
    if (m->level[n] < 0 || m->level[n] > 31)
      return G5_ERR_MESH;
  if (m->inst)
    for (int n = 0; n < n_total; ++n)
      if (m->inst[n] < 0 || m->inst[n] >= n_inst)
        return G5_ERR_MESH;
  for (int n = 0; n < n_owned; ++n)
    for (int s = 0; s < ns; ++s)
    {
      if (s == center)
        continue;
      const int       rel = m->nbr_rel[(size_t)n * ns + s];
      const int32_t * nb = m->nbr + ((size_t)n * ns + s) * nch;
      if (rel < -1 || rel > 1)
        return G5_ERR_MESH;
      if (rel <= 0)
      {
        if (nb[0] < 0 || nb[0] >= n_total)
          return G5_ERR_MESH;
        continue;
      }
      const int d[3] = { s % 3 - 1, (s / 3) % 3 - 1, s / 9 - 1 };
      for (int ch = 0; ch < nch; ++ch)
      {
        bool needed = true;
        for (int e = 0; e < dim; ++e)
        {
          const int ce = (ch >> e) & 1;
          if ((d[e] == -1 && ce != 1) || (d[e] == 1 && ce != 0))
            needed = false;
        }
        if (nb[ch] >= n_total || (needed && nb[ch] < 0))
          return G5_ERR_MESH;
      }
    }
  for (int o = 0; o < m->n_outside; ++o)
    if (m->out_src[o] < 0 || m->out_src[o] >= n_owned)
      return G5_ERR_MESH;
  return G5_OK;
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
    for (int j = 0; j < 8; ++j)
      p.f_mg[k][j] = (float)params->mg[k][j];
    p.f_mg_rho0[k] = (float)p.mg_rho0[k];
    p.f_gm1[k] = (float)(params->gamma[k] - 1.0);
    p.f_gpinf[k] = (float)(params->gamma[k] * params->pinf[k]);
  }
  p.mg_any = params->eos[0] != G5_EOS_STIFFENED || params->eos[1] != G5_EOS_STIFFENED;
  p.prolong = params->prolongation;
  return p;
}

} // namespace g5
