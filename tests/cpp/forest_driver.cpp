// C++ driver of the host block forest (include/g5gpu.hpp g5::Forest over the
// g5_forest_* C ABI): builds a forest, refines given leaves, balances, adapts
// with given flags and prints the leaves, the old -> new block map and the
// block table as text, for comparison with the Python mesh on the same input.
// Host only (no device call).
//
// stdin: dim bsize nbrick0 nbrick1 nbrick2 periodic0 periodic1 periodic2 lmin lmax
//        n_refine, then n_refine rows "level x y z"
//        n_flags (0: no adaptation), then n_flags codes
#include <cstdio>
#include <vector>

#include "../../include/g5gpu.hpp"

template <typename T>
static void
put(const char * name, const std::vector<T> & v)
{
  std::printf("%s %zu", name, v.size());
  for (const T & x : v)
    std::printf(" %d", (int)x);
  std::printf("\n");
}

int
main()
{
  G5ForestSpec s{};
  if (std::scanf("%d %d %d %d %d %d %d %d %d %d", &s.dim, &s.bsize, &s.nbrick[0], &s.nbrick[1], &s.nbrick[2], &s.periodic[0],
                 &s.periodic[1], &s.periodic[2], &s.level_min, &s.level_max) != 10)
    return 2;
  int nref = 0;
  if (std::scanf("%d", &nref) != 1)
    return 2;
  std::vector<int32_t> keys((size_t)nref * 4);
  for (int i = 0; i < 4 * nref; ++i)
    if (std::scanf("%d", &keys[i]) != 1)
      return 2;
  int nflags = 0;
  if (std::scanf("%d", &nflags) != 1)
    return 2;
  std::vector<int8_t> flags((size_t)nflags);
  for (int i = 0; i < nflags; ++i)
  {
    int f = 0;
    if (std::scanf("%d", &f) != 1)
      return 2;
    flags[i] = (int8_t)f;
  }
  try
  {
    g5::Forest forest(s);
    forest.refine(keys);
    forest.balance();
    put("leaves0", forest.leaves());
    if (nflags > 0)
    {
      std::vector<int8_t>  kind;
      std::vector<int32_t> src;
      const G5Remap        r = forest.adapt(flags, kind, src);
      std::printf("n_new %d\n", r.n_new);
      put("kind", kind);
      put("src", src);
    }
    const g5::BlockTable t = forest.table();
    std::printf("sizes %d %d\n", t.n_owned, t.n_outside);
    put("level", t.level);
    put("coord", t.coord);
    put("nbr", t.nbr);
    put("nbr_rel", t.nbr_rel);
    put("out_src", t.out_src);
    put("out_normal", t.out_normal);
    put("out_border", t.out_border);
  }
  catch (const g5::Error & e)
  {
    std::printf("error %s\n", e.what());
    return 1;
  }
  return 0;
}
