// refpin_flags.cpp — ComputeRefineFlags::run (scheme/ComputeRefineFlags.cpp:18-368)
// on a periodic tile of same-level blocks, the reference's own code compiled
// in place from the reference tree: the Loehner split / unsplit and the
// normalised-gradient indicators on IAD0 and IAD1, and the flag of each
// block (max over its cells of -1 init, 0 coarsen, 1 nothing, 2 refine).
// The neighbour values come through the shims' same-level StencilHelper.
//
// Test infrastructure only (golden vectors for the CPU oracle); never linked
// by the product.
#include <godunov_five_eq/scheme/ComputeRefineFlags.h>

using namespace kalypsso;
using namespace kalypsso::godunov_five_eq;

namespace
{
using Dev = kalypsso::DefaultDevice;

template <size_t dim>
int
flags(int b, int nb, int level, const double * Uin, int indicator, double eps_lohner, double eps_refine, double eps_coarsen, int lmin,
      int lmax, int8_t * out)
{
  using Hydro = models::FiveEq<dim>;
  constexpr int     nv = (int)Hydro::nbvar();
  const int         nblocks = dim == 2 ? nb * nb : nb * nb * nb;
  const int         ncell = dim == 2 ? b * b : b * b * b;
  block_size_t<dim> bs;
  brick_size_t<dim> brick;
  Kokkos::Array<bool, dim> periodic;
  for (size_t e = 0; e < dim; ++e)
  {
    bs[e] = b;
    brick[e] = nb;
    periodic[e] = true;
  }
  DataArrayBlock<dim, real_t, Dev> U(bs, nv, nblocks);
  for (size_t i = 0; i < (size_t)nblocks * nv * ncell; ++i)
    (*U.s)[i] = Uin[i];
  typename orchard_key_base_t<Dev>::view_t keys("keys", nblocks);
  for (int blk = 0; blk < nblocks; ++blk)
    keys(blk) = (uint64_t)level;
  typename AMRContext<dim, Dev>::amrflags_view_t f("flags", nblocks);
  for (int blk = 0; blk < nblocks; ++blk)
    f(blk) = AMRContextBase::KALYPSSO_FLAG_INIT;
  RefineIndicatorData rd;
  rd.indicator = indicator == 1 ? Indicator(Indicator::LOHNER_UNSPLIT)
               : indicator == 2 ? Indicator(Indicator::LOHNER_SPLIT)
                                : Indicator(Indicator::SIMPLE_GRADIENT);
  rd.epsilon = eps_lohner;
  rd.refine_th = eps_refine;
  rd.coarsen_th = eps_coarsen;
  rd.level_min = lmin;
  rd.level_max = lmax;
  typename hashmap_base_t<Dev>::map_t hashmap;
  ComputeRefineFlags<dim, Dev>::run(hashmap, keys, nblocks, brick, periodic, U, f, rd);
  for (int blk = 0; blk < nblocks; ++blk)
    out[blk] = f(blk);
  return 0;
}

} // namespace

// indicator: 0 SIMPLE_GRADIENT, 1 LOHNER_UNSPLIT, 2 LOHNER_SPLIT (the codes of g5_refine_flags)
extern "C" int
refpin_refine_flags(int dim, int b, int nb, int level, const double * U, int indicator, double eps_lohner, double eps_refine,
                    double eps_coarsen, int lmin, int lmax, int8_t * out)
{
  if (b < 4 || nb < 1 || level < 0 || level > 30 || indicator < 0 || indicator > 2)
    return -1;
  return dim == 2 ? flags<2>(b, nb, level, U, indicator, eps_lohner, eps_refine, eps_coarsen, lmin, lmax, out)
                  : (dim == 3 ? flags<3>(b, nb, level, U, indicator, eps_lohner, eps_refine, eps_coarsen, lmin, lmax, out) : -1);
}
