// g5_forest.cpp — the block forest of the dynamic AMR cycle, on the host:
// refinement, 2:1 balance, adaptation from refine flags with the old -> new
// block map, and the block table the kernels read (leaf order, outside twins,
// neighbour slots).  It stands where the reference calls p4est through its
// AMR manager (AMRManager::rebuild_from_context, SolverGodunovFiveEq.cpp:
// 258-314; the hashmap and orchard keys the stencil helpers use).
//
// A leaf is (level, x, y, z) in block units of its level (z = 0 in 2D) on a
// brick of nbrick[0] x nbrick[1] (x nbrick[2]) level-0 trees.  Leaf order:
// brick tree index, then the Morton index of the leaf's origin at the finest
// level present (x lowest bit).  2:1 balance across faces, edges and corners.
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <new>
#include <unordered_map>
#include <unordered_set>
#include <utility>
#include <vector>

#include "../../include/g5gpu.h"

namespace
{

struct Key
{
  int32_t L, x, y, z;
  bool    operator==(const Key & o) const { return L == o.L && x == o.x && y == o.y && z == o.z; }
  int32_t c(int e) const { return e == 0 ? x : (e == 1 ? y : z); }
};

struct KeyHash
{
  size_t operator()(const Key & k) const
  {
    uint64_t h = (uint64_t)(uint32_t)k.L * 0x9E3779B97F4A7C15ull;
    h ^= (uint64_t)(uint32_t)k.x * 0xC2B2AE3D27D4EB4Full;
    h ^= (uint64_t)(uint32_t)k.y * 0x165667B19E3779F9ull;
    h ^= (uint64_t)(uint32_t)k.z * 0xD6E8FEB86659FD93ull;
    return (size_t)(h ^ (h >> 31));
  }
};

using KeySet = std::unordered_set<Key, KeyHash>;
template <typename V>
using KeyMap = std::unordered_map<Key, V, KeyHash>;

Key
make_key(int L, const int * c)
{
  return Key{ L, c[0], c[1], c[2] };
}

// the block table of the current leaves (see g5_forest_table)
struct Table
{
  std::vector<Key>     owned, outside;
  std::vector<int32_t> out_src, nbr;
  std::vector<int8_t>  normal, border, rel;
};

} // namespace

struct G5Forest
{
  int    dim = 2, b = 16, lmin = 0, lmax = 0;
  int    nbrick[3] = { 1, 1, 1 }, periodic[3] = { 0, 0, 0 };
  KeySet leaves;
  Table  table;          // block table of the leaves, built on demand
  bool   table_valid = false;
  // leaf membership per level on a dense grid with a one-block margin (the
  // outside twins' positions), used when the level grids are small; the hash
  // set stays the list of leaves
  bool                 dense = false;
  std::vector<uint8_t> occ[32];
  int64_t              gx[32], gxy[32]; // grid strides per level

  int extent(int L, int e) const { return nbrick[e] << L; }

  void init_dense()
  {
    int64_t total = 0;
    for (int L = lmin; L <= lmax; ++L)
      total += (int64_t)(extent(L, 0) + 2) * (extent(L, 1) + 2) * (dim == 3 ? extent(L, 2) + 2 : 1);
    dense = total <= (int64_t)1 << 26;
    if (!dense)
      return;
    for (int L = lmin; L <= lmax; ++L)
    {
      gx[L] = extent(L, 0) + 2;
      gxy[L] = gx[L] * (extent(L, 1) + 2);
      occ[L].assign((size_t)(gxy[L] * (dim == 3 ? extent(L, 2) + 2 : 1)), 0);
    }
  }

  // position of k on its level's grid, or -1 outside it
  int64_t grid_index(const Key & k) const
  {
    if (k.L < lmin || k.L > lmax)
      return -1;
    for (int e = 0; e < dim; ++e)
      if (k.c(e) < -1 || k.c(e) > extent(k.L, e))
        return -1;
    return (k.x + 1) + gx[k.L] * (k.y + 1) + (dim == 3 ? gxy[k.L] * (k.z + 1) : 0);
  }

  bool has(const Key & k) const
  {
    if (!dense)
      return leaves.count(k) != 0;
    const int64_t i = grid_index(k);
    return i >= 0 && occ[k.L][(size_t)i];
  }
  void add(const Key & k)
  {
    leaves.insert(k);
    const int64_t i = dense ? grid_index(k) : -1;
    if (i >= 0)
      occ[k.L][(size_t)i] = 1;
  }
  void del(const Key & k)
  {
    leaves.erase(k);
    const int64_t i = dense ? grid_index(k) : -1;
    if (i >= 0)
      occ[k.L][(size_t)i] = 0;
  }

  // periodic wrap of same-level coordinates; true when outside a non-periodic face
  bool wrap(int L, const int * c, int * out) const
  {
    bool outside = false;
    out[0] = out[1] = out[2] = 0;
    for (int e = 0; e < dim; ++e)
    {
      const int n = extent(L, e);
      int       v = c[e];
      if (periodic[e])
        v = ((v % n) + n) % n;
      else if (v < 0 || v >= n)
        outside = true;
      out[e] = v;
    }
    return outside;
  }

  int nchild() const { return 1 << dim; }

  // child index x + 2 y + 4 z
  Key child(const Key & k, int ci) const
  {
    return Key{ k.L + 1, 2 * k.x + (ci & 1), 2 * k.y + ((ci >> 1) & 1), dim == 3 ? 2 * k.z + ((ci >> 2) & 1) : 0 };
  }

  Key parent(const Key & k) const { return Key{ k.L - 1, k.x >> 1, k.y >> 1, dim == 3 ? k.z >> 1 : 0 }; }

  // leaf at a level <= L containing the level-L position c (inside the domain)
  bool covering_leaf(int L, const int * c, Key & out) const
  {
    for (int l = L; l >= lmin; --l)
    {
      const int s = L - l;
      const Key k{ l, c[0] >> s, c[1] >> s, dim == 3 ? c[2] >> s : 0 };
      if (has(k))
      {
        out = k;
        return true;
      }
    }
    return false;
  }

  template <typename F>
  void for_offsets(F f) const
  {
    for (int oz = (dim == 3 ? -1 : 0); oz <= (dim == 3 ? 1 : 0); ++oz)
      for (int oy = -1; oy <= 1; ++oy)
        for (int ox = -1; ox <= 1; ++ox)
          if (ox || oy || oz)
            f(ox, oy, oz);
  }

  // leaves coarser than L - 1 next to a leaf of level L (faces, edges, corners)
  KeySet unbalanced() const
  {
    KeySet marked;
    for (const Key & k : leaves)
    {
      if (k.L - lmin < 2)
        continue;
      for_offsets([&](int ox, int oy, int oz) {
        const int c[3] = { k.x + ox, k.y + oy, k.z + oz };
        int       cw[3];
        if (wrap(k.L, c, cw))
          return;
        Key leaf;
        if (covering_leaf(k.L, cw, leaf) && leaf.L < k.L - 1)
          marked.insert(leaf);
      });
    }
    return marked;
  }

  int refine_keys(const std::vector<Key> & keys)
  {
    table_valid = false;
    int n = 0;
    for (const Key & k : keys)
      if (has(k) && k.L < lmax)
      {
        del(k);
        for (int ci = 0; ci < nchild(); ++ci)
          add(child(k, ci));
        ++n;
      }
    return n;
  }

  int balance()
  {
    int total = 0;
    for (;;)
    {
      const KeySet marked = unbalanced();
      if (marked.empty())
        return total;
      total += refine_keys(std::vector<Key>(marked.begin(), marked.end()));
    }
  }

  // a leaf finer than parent level + 1 touches the coarse block P
  bool coarsening_breaks_balance(const Key & P) const
  {
    const int L = P.L + 1;
    int       lo[3] = { 2 * P.x, 2 * P.y, 2 * P.z };
    const int zr = dim == 3 ? 4 : 1;
    for (int iz = 0; iz < zr; ++iz)
      for (int iy = 0; iy < 4; ++iy)
        for (int ix = 0; ix < 4; ++ix)
        {
          const int c[3] = { lo[0] - 1 + ix, lo[1] - 1 + iy, dim == 3 ? lo[2] - 1 + iz : 0 };
          bool      inside = true;
          for (int e = 0; e < dim; ++e)
            inside = inside && c[e] >= lo[e] && c[e] < lo[e] + 2;
          if (inside)
            continue;
          int cw[3];
          if (wrap(L, c, cw))
            continue;
          Key leaf;
          if (!covering_leaf(L, cw, leaf))
            return true;
        }
    return false;
  }

  std::vector<Key> ordered() const
  {
    int Lmax = 0;
    for (const Key & k : leaves)
      Lmax = std::max(Lmax, (int)k.L);
    std::vector<std::pair<std::pair<int64_t, uint64_t>, Key>> tmp;
    tmp.reserve(leaves.size());
    for (const Key & k : leaves)
    {
      int64_t tree[3] = { 0, 0, 0 }, local[3] = { 0, 0, 0 };
      for (int e = 0; e < dim; ++e)
      {
        tree[e] = k.c(e) >> k.L;
        local[e] = (int64_t)(k.c(e) - (tree[e] << k.L)) << (Lmax - k.L);
      }
      const int64_t tidx = tree[0] + nbrick[0] * (tree[1] + (dim == 3 ? nbrick[1] * tree[2] : 0));
      uint64_t      m = 0;
      for (int bit = 0; bit < Lmax; ++bit)
        for (int e = 0; e < dim; ++e)
          m |= (uint64_t)((local[e] >> bit) & 1) << (bit * dim + e);
      tmp.push_back({ { tidx, m }, k });
    }
    std::sort(tmp.begin(), tmp.end(), [](const auto & a, const auto & b) { return a.first < b.first; });
    std::vector<Key> out;
    out.reserve(tmp.size());
    for (auto & t : tmp)
      out.push_back(t.second);
    return out;
  }
};

namespace
{

bool
spec_ok(const G5ForestSpec * s)
{
  if (!s || (s->dim != 2 && s->dim != 3) || s->bsize < 4 || (s->bsize & 1))
    return false;
  if (s->level_min < 0 || s->level_max < s->level_min || s->level_max > 24)
    return false;
  for (int e = 0; e < s->dim; ++e)
    if (s->nbrick[e] < 1 || (int64_t)s->nbrick[e] << s->level_max > (1 << 28))
      return false;
  return true;
}

bool
key_ok(const G5Forest * f, const Key & k)
{
  if (k.L < f->lmin || k.L > f->lmax)
    return false;
  for (int e = 0; e < 3; ++e)
  {
    const int v = k.c(e);
    if (e >= f->dim ? v != 0 : (v < 0 || v >= f->extent(k.L, e)))
      return false;
  }
  return true;
}

} // namespace

extern "C" int
g5_forest_create(const G5ForestSpec * spec, const int32_t * leaves, int64_t n_leaves, G5Forest ** out)
{
  if (!out || !spec_ok(spec) || n_leaves < 0 || (n_leaves > 0 && !leaves))
    return G5_ERR_ARG;
  *out = nullptr;
  G5Forest * f = new (std::nothrow) G5Forest;
  if (!f)
    return G5_ERR_ARG;
  f->dim = spec->dim;
  f->b = spec->bsize;
  f->lmin = spec->level_min;
  f->lmax = spec->level_max;
  for (int e = 0; e < 3; ++e)
  {
    f->nbrick[e] = e < spec->dim ? spec->nbrick[e] : 1;
    f->periodic[e] = e < spec->dim ? (spec->periodic[e] != 0) : 0;
  }
  f->init_dense();
  if (n_leaves == 0)
  {
    // uniform at level_min
    const int L = f->lmin;
    for (int z = 0; z < (f->dim == 3 ? f->extent(L, 2) : 1); ++z)
      for (int y = 0; y < f->extent(L, 1); ++y)
        for (int x = 0; x < f->extent(L, 0); ++x)
          f->add(Key{ L, x, y, z });
  }
  else
  {
    f->leaves.reserve((size_t)n_leaves * 2);
    for (int64_t i = 0; i < n_leaves; ++i)
    {
      const Key k{ leaves[4 * i], leaves[4 * i + 1], leaves[4 * i + 2], leaves[4 * i + 3] };
      if (!key_ok(f, k))
      {
        delete f;
        return G5_ERR_MESH;
      }
      f->add(k);
    }
    // the leaves must tile the brick: no duplicate, no leaf inside another,
    // and the covered volume (in cells of the finest level present) that of
    // the brick
    int Lm = 0;
    for (const Key & k : f->leaves)
      Lm = k.L > Lm ? k.L : Lm;
    bool               ok = (int64_t)f->leaves.size() == n_leaves;
    unsigned __int128  vol = 0, full = 1;
    for (int e = 0; e < f->dim; ++e)
      full *= (unsigned __int128)f->extent(Lm, e);
    for (const Key & k : f->leaves)
    {
      vol += (unsigned __int128)1 << (f->dim * (Lm - k.L));
      Key a = k;
      while (ok && a.L > f->lmin)
      {
        a = f->parent(a);
        ok = !f->has(a);
      }
    }
    if (!ok || vol != full)
    {
      delete f;
      return G5_ERR_MESH;
    }
  }
  *out = f;
  return G5_OK;
}

extern "C" int
g5_forest_destroy(G5Forest * f)
{
  if (!f)
    return G5_ERR_ARG;
  delete f;
  return G5_OK;
}

extern "C" int64_t
g5_forest_num_leaves(const G5Forest * f)
{
  return f ? (int64_t)f->leaves.size() : (int64_t)G5_ERR_ARG;
}

extern "C" int
g5_forest_leaves(const G5Forest * f, int32_t * out)
{
  if (!f || !out)
    return G5_ERR_ARG;
  const std::vector<Key> ord = f->ordered();
  for (size_t i = 0; i < ord.size(); ++i)
  {
    out[4 * i] = ord[i].L;
    out[4 * i + 1] = ord[i].x;
    out[4 * i + 2] = ord[i].y;
    out[4 * i + 3] = ord[i].z;
  }
  return G5_OK;
}

extern "C" int
g5_forest_refine(G5Forest * f, const int32_t * keys, int64_t n)
{
  if (!f || n < 0 || (n > 0 && !keys))
    return G5_ERR_ARG;
  std::vector<Key> v;
  v.reserve((size_t)n);
  for (int64_t i = 0; i < n; ++i)
    v.push_back(Key{ keys[4 * i], keys[4 * i + 1], keys[4 * i + 2], keys[4 * i + 3] });
  return f->refine_keys(v);
}

extern "C" int
g5_forest_balance(G5Forest * f)
{
  if (!f)
    return G5_ERR_ARG;
  return f->balance();
}

extern "C" int64_t
g5_forest_adapt(G5Forest * f, const int8_t * flags, int64_t n_flags, int8_t * kind, int32_t * src, int64_t cap)
{
  if (!f || (n_flags > 0 && !flags) || !kind || !src)
    return G5_ERR_ARG;
  const std::vector<Key> old = f->ordered();
  if (n_flags != (int64_t)old.size())
    return G5_ERR_ARG;
  f->table_valid = false;
  const int    nc = f->nchild();
  KeyMap<int>  old_index;
  old_index.reserve(old.size() * 2);
  for (size_t i = 0; i < old.size(); ++i)
    old_index[old[i]] = (int)i;
  KeyMap<Key> refined_from;
  bool        twice = false;
  auto        refine_one = [&](const Key & k) {
    if (refined_from.count(k))
    {
      twice = true;
      return;
    }
    f->del(k);
    for (int ci = 0; ci < nc; ++ci)
    {
      const Key ch = f->child(k, ci);
      f->add(ch);
      refined_from[ch] = k;
    }
  };
  for (size_t i = 0; i < old.size(); ++i)
    if (flags[i] == 2 && old[i].L < f->lmax)
      refine_one(old[i]);
  // 2:1 balance by refinement
  for (;;)
  {
    const KeySet marked = f->unbalanced();
    if (marked.empty())
      break;
    for (const Key & k : marked)
      if (k.L < f->lmax)
        refine_one(k);
    if (twice)
      return G5_ERR_MESH;
  }
  if (twice)
    return G5_ERR_MESH;
  // coarsening of complete families flagged 0 and not refined
  KeySet parents;
  for (size_t i = 0; i < old.size(); ++i)
    if (flags[i] == 0 && old[i].L > f->lmin)
      parents.insert(f->parent(old[i]));
  KeyMap<std::vector<Key>> families;
  for (const Key & P : parents)
  {
    std::vector<Key> kids;
    bool             all = true;
    for (int ci = 0; ci < nc && all; ++ci)
    {
      const Key ch = f->child(P, ci);
      auto      it = old_index.find(ch);
      all = f->has(ch) && it != old_index.end() && flags[it->second] == 0;
      kids.push_back(ch);
    }
    if (all)
      families[P] = kids;
  }
  for (auto & fam : families)
  {
    for (const Key & ch : fam.second)
      f->del(ch);
    f->add(fam.first);
  }
  for (;;)
  {
    std::vector<Key> undo;
    for (auto & fam : families)
      if (f->coarsening_breaks_balance(fam.first))
        undo.push_back(fam.first);
    if (undo.empty())
      break;
    for (const Key & P : undo)
    {
      f->del(P);
      for (const Key & ch : families[P])
        f->add(ch);
      families.erase(P);
    }
  }
  const std::vector<Key> nw = f->ordered();
  if ((int64_t)nw.size() > cap)
    return G5_ERR_ARG;
  for (size_t j = 0; j < nw.size(); ++j)
  {
    const Key & k = nw[j];
    int32_t *   s = src + j * nc;
    for (int c = 0; c < nc; ++c)
      s[c] = -1;
    kind[j] = 0;
    auto oi = old_index.find(k);
    if (oi != old_index.end())
    {
      s[0] = oi->second;
      continue;
    }
    auto rf = refined_from.find(k);
    if (rf != refined_from.end())
    {
      kind[j] = 1;
      s[0] = old_index.at(rf->second);
      s[1] = (k.x & 1) | ((k.y & 1) << 1) | (f->dim == 3 ? (k.z & 1) << 2 : 0);
      continue;
    }
    auto fm = families.find(k);
    if (fm == families.end())
      return G5_ERR_MESH;
    kind[j] = 2;
    for (int c = 0; c < nc; ++c)
      s[c] = old_index.at(fm->second[c]);
  }
  return (int64_t)nw.size();
}

namespace
{

int
build_table(const G5Forest * f, Table & t)
{
  const int dim = f->dim, ns = dim == 2 ? 9 : 27, nc = f->nchild();
  t.owned = f->ordered();
  // block index by key: the forest's level grids when dense, else a hash map
  KeyMap<int>          hindex;
  std::vector<int32_t> dindex[32];
  if (f->dense)
    for (int L = f->lmin; L <= f->lmax; ++L)
      dindex[L].assign(f->occ[L].size(), -1);
  else
    hindex.reserve(t.owned.size() * 3);
  auto put = [&](const Key & k, int v) {
    if (!f->dense)
      hindex[k] = v;
    else
    {
      const int64_t gi = f->grid_index(k);
      if (gi >= 0)
        dindex[k.L][(size_t)gi] = v;
    }
  };
  auto find = [&](const Key & k) -> int {
    if (!f->dense)
    {
      auto it = hindex.find(k);
      return it == hindex.end() ? -1 : it->second;
    }
    const int64_t gi = f->grid_index(k);
    return gi < 0 ? -1 : dindex[k.L][(size_t)gi];
  };
  for (size_t i = 0; i < t.owned.size(); ++i)
    put(t.owned[i], (int)i);
  // outside twins: per owned block touching a non-periodic face, one twin per
  // non-zero normal over {0} + {-1 at the min face} + {+1 at the max face}
  for (size_t i = 0; i < t.owned.size(); ++i)
  {
    const Key & k = t.owned[i];
    int         choices[3][3], nch[3];
    int8_t      bord[6] = { 0, 0, 0, 0, 0, 0 };
    for (int e = 0; e < 3; ++e)
    {
      nch[e] = 1;
      choices[e][0] = 0;
      if (e >= dim)
        continue;
      const int n = f->extent(k.L, e);
      const bool lo = k.c(e) == 0, hi = k.c(e) == n - 1;
      bord[2 * e] = lo;
      bord[2 * e + 1] = hi;
      if (!f->periodic[e])
      {
        if (lo)
          choices[e][nch[e]++] = -1;
        if (hi)
          choices[e][nch[e]++] = 1;
      }
    }
    // itertools.product order: the last dimension varies fastest
    for (int a = 0; a < nch[0]; ++a)
      for (int bb = 0; bb < nch[1]; ++bb)
        for (int cc = 0; cc < nch[2]; ++cc)
        {
          const int nrm[3] = { choices[0][a], choices[1][bb], choices[2][cc] };
          if (!nrm[0] && !nrm[1] && !nrm[2])
            continue;
          t.outside.push_back(Key{ k.L, k.x + nrm[0], k.y + nrm[1], dim == 3 ? k.z + nrm[2] : 0 });
          for (int e = 0; e < 3; ++e)
            t.normal.push_back((int8_t)nrm[e]);
          for (int fc = 0; fc < 6; ++fc)
            t.border.push_back(bord[fc]);
          t.out_src.push_back((int32_t)i);
        }
  }
  const int n_owned = (int)t.owned.size();
  for (size_t j = 0; j < t.outside.size(); ++j)
  {
    if (f->dense && f->grid_index(t.outside[j]) < 0)
      return G5_ERR_MESH;
    put(t.outside[j], n_owned + (int)j);
  }
  t.nbr.assign((size_t)n_owned * ns * nc, -1);
  t.rel.assign((size_t)n_owned * ns, 0);
  for (int i = 0; i < n_owned; ++i)
  {
    const Key & k = t.owned[i];
    for (int sz = (dim == 3 ? -1 : 0); sz <= (dim == 3 ? 1 : 0); ++sz)
      for (int sy = -1; sy <= 1; ++sy)
        for (int sx = -1; sx <= 1; ++sx)
        {
          if (!sx && !sy && !sz)
            continue;
          const int d[3] = { sx, sy, sz };
          const int s = (sx + 1) + 3 * (sy + 1) + (dim == 3 ? 9 * (sz + 1) : 0);
          int       c[3] = { k.x + sx, k.y + sy, dim == 3 ? k.z + sz : 0 }, cw[3];
          f->wrap(k.L, c, cw);
          int32_t * nb = &t.nbr[((size_t)i * ns + s) * nc];
          int       hit = find(make_key(k.L, cw));
          if (hit >= 0)
          {
            t.rel[(size_t)i * ns + s] = 0;
            nb[0] = hit;
            continue;
          }
          const Key pk{ k.L - 1, cw[0] >> 1, cw[1] >> 1, dim == 3 ? cw[2] >> 1 : 0 };
          hit = find(pk);
          if (hit >= 0)
          {
            t.rel[(size_t)i * ns + s] = -1;
            nb[0] = hit;
            continue;
          }
          bool found = false;
          for (int ci = 0; ci < nc; ++ci)
          {
            const int ch[3] = { ci & 1, (ci >> 1) & 1, (ci >> 2) & 1 };
            bool      touch = true;
            for (int e = 0; e < dim; ++e)
              touch = touch && !((d[e] == -1 && ch[e] != 1) || (d[e] == 1 && ch[e] != 0));
            if (!touch)
              continue;
            const Key ck{ k.L + 1, 2 * cw[0] + ch[0], 2 * cw[1] + ch[1], dim == 3 ? 2 * cw[2] + ch[2] : 0 };
            const int ct = find(ck);
            if (ct < 0)
              return G5_ERR_MESH; // not 2:1 balanced
            nb[ci] = ct;
            found = true;
          }
          if (!found)
            return G5_ERR_MESH;
          t.rel[(size_t)i * ns + s] = 1;
        }
  }
  return G5_OK;
}

} // namespace

namespace
{
int
ensure_table(G5Forest * f)
{
  if (f->table_valid)
    return G5_OK;
  f->table = Table();
  const int rc = build_table(f, f->table);
  f->table_valid = rc == G5_OK;
  return rc;
}
} // namespace

extern "C" int
g5_forest_table_sizes(G5Forest * f, int32_t * n_owned, int32_t * n_outside)
{
  if (!f || !n_owned || !n_outside)
    return G5_ERR_ARG;
  const int rc = ensure_table(f);
  if (rc != G5_OK)
    return rc;
  *n_owned = (int32_t)f->table.owned.size();
  *n_outside = (int32_t)f->table.outside.size();
  return G5_OK;
}

extern "C" int
g5_forest_table(G5Forest *       f,
                int32_t *        level,
                int32_t *        coord,
                int32_t *        nbr,
                int8_t *         nbr_rel,
                int32_t *        out_src,
                int8_t *         out_normal,
                int8_t *         out_border)
{
  if (!f || !level || !coord || !nbr || !nbr_rel)
    return G5_ERR_ARG;
  const int rc = ensure_table(f);
  if (rc != G5_OK)
    return rc;
  const Table & t = f->table;
  const size_t n_owned = t.owned.size(), n_out = t.outside.size();
  if (n_out > 0 && (!out_src || !out_normal || !out_border))
    return G5_ERR_ARG;
  for (size_t i = 0; i < n_owned + n_out; ++i)
  {
    const Key & k = i < n_owned ? t.owned[i] : t.outside[i - n_owned];
    level[i] = k.L;
    coord[3 * i] = k.x;
    coord[3 * i + 1] = k.y;
    coord[3 * i + 2] = k.z;
  }
  std::memcpy(nbr, t.nbr.data(), t.nbr.size() * sizeof(int32_t));
  std::memcpy(nbr_rel, t.rel.data(), t.rel.size());
  if (n_out > 0)
  {
    std::memcpy(out_src, t.out_src.data(), n_out * sizeof(int32_t));
    std::memcpy(out_normal, t.normal.data(), n_out * 3);
    std::memcpy(out_border, t.border.data(), n_out * 6);
  }
  return G5_OK;
}
