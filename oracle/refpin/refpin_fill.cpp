// refpin_fill.cpp — FillOutsideCellFunctor::apply (border_conditions/
// FillOutside.cpp:44-172), the reference's own boundary fill compiled in place
// from the reference tree: for every cell of every outside quadrant, the faces
// in order whose rule applies (the inside quadrant at the domain border on
// that face and the outside quadrant beyond it in that direction), each
// ZERO_GRADIENT or WALL copy overwriting the previous one.  The inside
// quadrant, the outside normal and the border faces come through the shims'
// refpin_fill keys from the GPU path's block table (out_src, out_normal,
// out_border).
//
// Test infrastructure only (golden vectors for the CPU oracle); never linked
// by the product.
#include <godunov_five_eq/border_conditions/FillOutside.h>

using namespace kalypsso;
using namespace kalypsso::godunov_five_eq;

namespace
{
using Dev = kalypsso::DefaultDevice;

template <size_t dim>
int
fill(int b, int n_owned, int n_outside, const int32_t * out_src, const int8_t * out_normal, const int8_t * out_border, const int32_t * bc,
     double * Uio)
{
  using Hydro = models::FiveEq<dim>;
  constexpr int     nv = (int)Hydro::nbvar();
  const int         ntotal = n_owned + n_outside;
  const size_t      ncell = dim == 2 ? (size_t)b * b : (size_t)b * b * b;
  block_size_t<dim> bs;
  for (size_t e = 0; e < dim; ++e)
    bs[e] = b;
  auto & tb = refpin_fill::table();
  tb.n_owned = n_owned;
  tb.n_outside = n_outside;
  tb.out_src = out_src;
  tb.out_normal = out_normal;
  tb.out_border = out_border;
  tb.border_of.assign((size_t)n_owned * 6, 0);
  for (int o = 0; o < n_outside; ++o)
  {
    if (out_src[o] < 0 || out_src[o] >= n_owned)
      return 2;
    for (int f = 0; f < 6; ++f)
      tb.border_of[(size_t)out_src[o] * 6 + f] = out_border[(size_t)o * 6 + f];
  }
  DataArrayBlock<dim, real_t, Dev> U(bs, nv, ntotal);
  for (size_t i = 0; i < (size_t)ntotal * nv * ncell; ++i)
    (*U.s)[i] = Uio[i];
  typename orchard_key_base_t<Dev>::view_t keys("keys", ntotal);
  for (int blk = 0; blk < ntotal; ++blk)
    keys(blk) = (uint64_t)blk;
  ConfigMap cm;
  for (int f = 0; f < 2 * (int)dim; ++f)
    cm.set("refpin", "bc" + std::to_string(f), std::to_string(bc[f]));
  typename hashmap_base_t<Dev>::map_t hashmap;
  FillOutsideCellFunctor<dim, Dev>::apply(U, AMRMeshInfo(n_owned, 0, n_outside), keys, hashmap, cm, ParallelEnv{});
  for (size_t i = 0; i < (size_t)ntotal * nv * ncell; ++i)
    Uio[i] = (*U.s)[i];
  return 0;
}
} // namespace

// U: [n_owned + n_outside][nv][b^dim]; the outside blocks are overwritten.
// bc[2 dim]: the BC_HYDRO value of each face (2 ZERO_GRADIENT, 3 WALL).
extern "C" int
refpin_fill_outside(int dim, int b, int n_owned, int n_outside, const int32_t * out_src, const int8_t * out_normal, const int8_t * out_border,
                    const int32_t * bc, double * U)
{
  if (dim == 2)
    return fill<2>(b, n_owned, n_outside, out_src, out_normal, out_border, bc, U);
  if (dim == 3)
    return fill<3>(b, n_owned, n_outside, out_src, out_normal, out_border, bc, U);
  return 1;
}
