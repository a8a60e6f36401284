// g5_prolong.cuh — ghost cells of an owned block that lie in a coarser
// neighbour, prolonged by EXTRAPOLATE_LINEAR_MINMOD or by conservative
// order-2 / order-4 interpolation (ConvertToPrimitivesVariablesFunctor::
// fill_ghosts, scheme/ConvertToPrimitivesVariablesFunctor.cpp:893-917, with
// linear_extrapolate_using_limited_slopes :544-745, extrapol_2d/3d :278-335,
// conservative_interpolation_order2/4 :750-827, interpol_order2/4 :341-488).
//
// One pass before the step kernel, over the blocks the step walks: a CTA
// loads the level-(l-1) values of the coarse cells around its block (the
// patch) into shared memory once, then every ghost cell in a coarser slot
// combines its stencil from the patch and writes its conservative state to
// DevMesh::pg, where the step kernel's gather reads it instead of the coarse
// cell.  FP64, evaluated in the order of the CPU restatement (compiled
// without multiply-add contraction): the result is bit-exact against it.
//
// Stencil semantics (the reference's helpers are in the external kalypsso
// core, restated): a coarse cell's value is the coarser neighbour's cell
// that holds it, the mean of the 2^dim level-l cells covering it (the block
// itself or a same-level neighbour), or in a finer neighbour the mean of the
// 2^dim means of 2^dim level-(l+1) cells (sums x fastest, then / 2^dim).
// Minmod: coarse value + 0.25 (+-1) x the minmod slope per direction
// (slope_type 1); conservative order 2 / 4: half-cell averages of the
// quadratic / quartic with the coarse cell averages, lower half
// (1/8, 1, -1/8) / (-3/128, 22/128, 1, -22/128, 3/128), upper half reversed,
// along x, then y, then z.
//
// Reach: the patch spans r + 1 coarse cells around the block's footprint
// (r = 1 for minmod and order 2, 2 for order 4), so every patch cell lies in
// one of the block's 3^dim neighbour slots; in a finer slot it lies in a
// child that touches the block when r <= b/4 - 1/2.  Order 4 on 8-cell blocks
// also reads the far children of a finer slot, which the block table does not
// list: each is found as the same-level neighbour of its touching sibling
// (owned, with a neighbour table); a far child refined further, or one beyond
// a domain face (an outside twin), raises the mesh status.
#pragma once

#include "g5_common.cuh"

namespace g5
{

template <int DIM, int B, int MODE>
struct ProlongTraits
{
  static constexpr int R = MODE == 3 ? 2 : 1;         // stencil half-width in coarse cells
  static constexpr int P = B / 2 + 2 + 2 * R;         // patch extent per axis
  static constexpr int NP = DIM == 2 ? P * P : P * P * P;
  static constexpr int NVI = DIM == 2 ? 6 : 7;        // prolonged variables
  static constexpr int G = B + 4;
  static constexpr int NG = DIM == 2 ? G * G : G * G * G;
  static constexpr int NC = DIM == 2 ? B * B : B * B * B;
  static constexpr int NS = DIM == 2 ? 9 : 27, NCH = DIM == 2 ? 4 : 8;
  static constexpr int NT = 128;
  static constexpr size_t smem_bytes = sizeof(double) * (size_t)NVI * NP;
};

// where the value of coarse cell q (coarse coordinates relative to block n's
// footprint [0, B/2)^DIM) comes from: kind 0 mean of 2^DIM cells of block src
// from cell c, kind 1 the single cell c of src, kind 2 mean of 2^DIM means of
// 2^DIM cells of src from cell c; kind -1 unresolvable (bad table entry)
template <int DIM, int B>
__device__ __forceinline__ void
coarse_cell_ref(const DevMesh & m, int n, const int * c0, const int * q, int & kind, int & src, int & c)
{
  constexpr int NS = DIM == 2 ? 9 : 27, NCH = DIM == 2 ? 4 : 8, H = B / 2;
  int           s[3] = { 0, 0, 0 }, f[3] = { 0, 0, 0 };
  bool          own = true;
#pragma unroll
  for (int e = 0; e < DIM; ++e)
  {
    s[e] = q[e] < 0 ? -1 : (q[e] >= H ? 1 : 0);
    f[e] = 2 * q[e] - s[e] * B; // first level-l cell of q in the slot's same-level block
    own = own && s[e] == 0;
  }
  auto cell = [&](const int * x) { return DIM == 2 ? x[0] + B * x[1] : x[0] + B * (x[1] + B * x[2]); };
  kind = -1;
  src = -1;
  c = 0;
  if (own)
  {
    kind = 0;
    src = n;
    c = cell(f);
    return;
  }
  const int       slot = DIM == 2 ? (s[0] + 1) + 3 * (s[1] + 1) : (s[0] + 1) + 3 * (s[1] + 1) + 9 * (s[2] + 1);
  const int       rel = m.nbr_rel[(size_t)n * NS + slot];
  const int32_t * nb = m.nbr + ((size_t)n * NS + slot) * NCH;
  if (rel == 0)
  {
    kind = 0;
    src = nb[0];
    c = cell(f);
  }
  else if (rel < 0)
  {
    int cc[3] = { 0, 0, 0 };
#pragma unroll
    for (int e = 0; e < DIM; ++e)
      cc[e] = ((c0[e] + s[e]) & 1) * H + (f[e] >> 1);
    kind = 1;
    src = nb[0];
    c = cell(cc);
  }
  else
  {
    int ch[3] = { 0, 0, 0 }, l[3] = { 0, 0, 0 };
#pragma unroll
    for (int e = 0; e < DIM; ++e)
    {
      ch[e] = f[e] >= H ? 1 : 0;
      l[e] = 2 * (f[e] - ch[e] * H);
    }
    kind = 2;
    src = nb[DIM == 2 ? ch[0] + 2 * ch[1] : ch[0] + 2 * ch[1] + 4 * ch[2]];
    c = cell(l);
    if (src < 0)
    {
      // a child that does not touch the block (order-4 patches of 8-cell
      // blocks reach it): the same-level neighbour of the touching sibling,
      // when that sibling is owned and the child is a leaf
      int ct[3] = { 0, 0, 0 }, dl[3] = { 0, 0, 0 };
#pragma unroll
      for (int e = 0; e < DIM; ++e)
      {
        ct[e] = s[e] == 0 ? ch[e] : (s[e] < 0 ? 1 : 0);
        dl[e] = ch[e] - ct[e];
      }
      const int T = nb[DIM == 2 ? ct[0] + 2 * ct[1] : ct[0] + 2 * ct[1] + 4 * ct[2]];
      const int st = DIM == 2 ? (dl[0] + 1) + 3 * (dl[1] + 1) : (dl[0] + 1) + 3 * (dl[1] + 1) + 9 * (dl[2] + 1);
      src = (T >= 0 && T < m.n_owned && m.nbr_rel[(size_t)T * NS + st] == 0) ? m.nbr[((size_t)T * NS + st) * NCH] : -1;
    }
  }
  if (src < 0 || src >= m.n_total)
    kind = -1;
}

// mean of the 2^DIM cells of one variable's block array p from cell c
template <int DIM, int B>
__device__ __forceinline__ double
mean_cells(const double * p, int c)
{
  double sum = 0.0;
#pragma unroll
  for (int oz = 0; oz < (DIM == 3 ? 2 : 1); ++oz)
#pragma unroll
    for (int oy = 0; oy < 2; ++oy)
#pragma unroll
      for (int ox = 0; ox < 2; ++ox)
        sum += p[c + ox + B * oy + B * B * oz];
  return sum / (double)(1 << DIM);
}

template <int DIM, int B>
__device__ __forceinline__ double
coarse_cell_value(const double * p, int kind, int c)
{
  if (kind == 1)
    return p[c];
  if (kind == 0)
    return mean_cells<DIM, B>(p, c);
  double sum = 0.0;
#pragma unroll
  for (int oz = 0; oz < (DIM == 3 ? 2 : 1); ++oz)
#pragma unroll
    for (int oy = 0; oy < 2; ++oy)
#pragma unroll
      for (int ox = 0; ox < 2; ++ox)
        sum += mean_cells<DIM, B>(p, c + 2 * ox + 2 * B * oy + 2 * B * B * oz);
  return sum / (double)(1 << DIM);
}

__device__ __forceinline__ double
prolong_coef(int mode, int upper, int i)
{
  // lower half; the upper half is the same read backwards
  const int k = upper ? -i : i;
  if (mode == 2)
    return k == 0 ? 1.0 : (k < 0 ? 0.125 : -0.125);
  switch (k)
  {
  case -2: return -3.0 / 128.0;
  case -1: return 22.0 / 128.0;
  case 0: return 1.0;
  case 1: return -22.0 / 128.0;
  default: return 3.0 / 128.0;
  }
}

// linear combination sum_i c(i) v(i), i = -R .. R, left to right
template <int R, typename F>
__device__ __forceinline__ double
prolong_lin(int mode, int upper, F v)
{
  double acc = prolong_coef(mode, upper, -R) * v(-R);
#pragma unroll
  for (int i = -R + 1; i <= R; ++i)
    acc = acc + prolong_coef(mode, upper, i) * v(i);
  return acc;
}

// the 2^dim children of the coarse value at Pv in a shared-memory patch
// (strides 1, P, P^2), child (ux, uy, uz) at ch[ux + 2 uy + 4 uz]: minmod
// slopes, or the x, then y, then z sums of the conservative interpolation
// shared by the children (the same operands and order as the per-child sums
// of the CPU restatement)
template <int DIM, int MODE, int P>
__device__ __forceinline__ void
prolong_children(const double * Pv, double * ch)
{
  constexpr int R = MODE == 3 ? 2 : 1, NCHILD = 1 << DIM;
  auto at = [&](int i, int j, int k) { return Pv[i + P * (j + (DIM == 3 ? P * k : 0))]; };
  if constexpr (MODE == 1)
  {
    const double u0 = at(0, 0, 0);
    double       sl[3];
    sl[0] = slope_scalar<double>(u0, at(1, 0, 0), at(-1, 0, 0), 1.0);
    sl[1] = slope_scalar<double>(u0, at(0, 1, 0), at(0, -1, 0), 1.0);
    if constexpr (DIM == 3)
      sl[2] = slope_scalar<double>(u0, at(0, 0, 1), at(0, 0, -1), 1.0);
#pragma unroll
    for (int c = 0; c < NCHILD; ++c)
    {
      double r = u0;
#pragma unroll
      for (int e = 0; e < DIM; ++e)
        r = r + 0.25 * (double)(((c >> e) & 1) ? 1 : -1) * sl[e];
      ch[c] = r;
    }
  }
  else if constexpr (DIM == 2)
  {
#pragma unroll
    for (int ux = 0; ux < 2; ++ux)
    {
      double X[2 * R + 1];
#pragma unroll
      for (int j = -R; j <= R; ++j)
        X[j + R] = prolong_lin<R>(MODE, ux, [&](int i) { return at(i, j, 0); });
#pragma unroll
      for (int uy = 0; uy < 2; ++uy)
        ch[ux + 2 * uy] = prolong_lin<R>(MODE, uy, [&](int j) { return X[j + R]; });
    }
  }
  else
  {
#pragma unroll
    for (int ux = 0; ux < 2; ++ux)
    {
      double X[2 * R + 1][2 * R + 1]; // [k][j]
#pragma unroll
      for (int k = -R; k <= R; ++k)
#pragma unroll
        for (int j = -R; j <= R; ++j)
          X[k + R][j + R] = prolong_lin<R>(MODE, ux, [&](int i) { return at(i, j, k); });
#pragma unroll
      for (int uy = 0; uy < 2; ++uy)
      {
        double Y[2 * R + 1];
#pragma unroll
        for (int k = -R; k <= R; ++k)
          Y[k + R] = prolong_lin<R>(MODE, uy, [&](int j) { return X[k + R][j + R]; });
#pragma unroll
        for (int uz = 0; uz < 2; ++uz)
          ch[ux + 2 * uy + 4 * uz] = prolong_lin<R>(MODE, uz, [&](int k) { return Y[k + R]; });
      }
    }
  }
}

// One CTA per walked block with a coarser neighbour:
//  1. the coarser slots and the prefix of their coarse-cell counts;
//  2. the patch cells some stencil reads, packed into a list (warp ballots);
//  3. their values for the NVI prolonged variables into shared memory;
//  4. work items (variable, coarse cell): the 2^dim children of the coarse
//     cell for that variable, the per-direction combinations shared by the
//     children (slopes, or the x then y then z sums);
//  5. ID = IAD0 + IAD1 and IA1 = 1 - IA0 per ghost cell.
// FP64 instructions cost the same with idle lanes: the items are packed
// into full warps.
template <int DIM, int B, int MODE>
__global__ void __launch_bounds__(128)
prolong_kernel(StepArgs a)
{
  using T = ProlongTraits<DIM, B, MODE>;
  using H = V<DIM>;
  constexpr int R = T::R, P = T::P, NP = T::NP, G = T::G, NG = T::NG, NC = T::NC, NT = T::NT;
  constexpr int HB = B / 2, NCHILD = 1 << DIM;
  extern __shared__ __align__(16) double sP[]; // [NVI][NP]
  __shared__ int sOff[T::NS + 1];              // coarse cells of the coarser slots before slot k
  __shared__ int sSlot[T::NS];
  __shared__ int sNslot, sCount;
  __shared__ int sList[NP]; // patch cells to load
  const int      vars[7] = { H::IAD0, H::IAD1, H::IA0, H::IE, H::IU, H::IV, H::IW };
  const int      tid = threadIdx.x, lane = tid & 31;
  const int      nwalk = step_count(a);
  // coarse cell (block coarse coordinates) of item w's slot-local index
  auto slot_cell = [&](int js, int loc, int * q) {
    const int sl = sSlot[js];
#pragma unroll
    for (int e = 0, p3 = 1; e < DIM; ++e, p3 *= 3)
    {
      const int d = (sl / p3) % 3 - 1;
      if (d == 0)
      {
        q[e] = loc % HB;
        loc /= HB;
      }
      else
        q[e] = d < 0 ? -1 : HB;
    }
  };
  for (int iw = blockIdx.x; iw < nwalk; iw += gridDim.x)
  {
    const int n = a.work ? a.work[iw] : iw;
    const int ps = a.m.pg_slot[n];
    if (ps < 0)
      continue;
    const int c0[3] = { a.m.coord[n * 3 + 0], a.m.coord[n * 3 + 1], DIM == 3 ? a.m.coord[n * 3 + 2] : 0 };
    __syncthreads(); // the previous block's lists and patch are read
    if (tid == 0)
    {
      int tot = 0, k = 0;
      for (int sl = 0; sl < T::NS; ++sl)
      {
        if (sl == T::NS / 2 || a.m.nbr_rel[(size_t)n * T::NS + sl] >= 0)
          continue;
        int cnt = 1;
#pragma unroll
        for (int e = 0, p3 = 1; e < DIM; ++e, p3 *= 3)
          cnt *= (sl / p3) % 3 == 1 ? HB : 1;
        sSlot[k] = sl;
        sOff[k] = tot;
        tot += cnt;
        ++k;
      }
      sOff[k] = tot;
      sNslot = k;
      sCount = 0;
    }
    __syncthreads();
    const int nslot = sNslot, ncc = sOff[nslot];
    // 2. patch cells within R of a coarse cell of a coarser slot
    for (int base = 0; base < NP; base += NT)
    {
      const int i = base + tid;
      bool      need = false;
      if (i < NP)
      {
        const int q[3] = { i % P - 1 - R, (i / P) % P - 1 - R, DIM == 3 ? i / (P * P) - 1 - R : 0 };
        for (int js = 0; js < nslot && !need; ++js)
        {
          const int sl = sSlot[js];
          bool      in = true;
#pragma unroll
          for (int e = 0, p3 = 1; e < DIM; ++e, p3 *= 3)
          {
            const int d = (sl / p3) % 3 - 1;
            const int lo = d < 0 ? -1 : (d == 0 ? 0 : HB), hi = d < 0 ? -1 : (d == 0 ? HB - 1 : HB);
            in = in && q[e] >= lo - R && q[e] <= hi + R;
          }
          need = in;
        }
      }
      const unsigned mask = __ballot_sync(0xffffffffu, need);
      int            wbase = 0;
      if (lane == 0 && mask)
        wbase = atomicAdd(&sCount, __popc(mask));
      wbase = __shfl_sync(0xffffffffu, wbase, 0);
      if (need)
        sList[wbase + __popc(mask & ((1u << lane) - 1u))] = i;
    }
    __syncthreads();
    // 3. their values
    const int nload = sCount;
    for (int k = tid; k < nload; k += NT)
    {
      const int i = sList[k];
      const int q[3] = { i % P - 1 - R, (i / P) % P - 1 - R, DIM == 3 ? i / (P * P) - 1 - R : 0 };
      int       kind, src, c;
      coarse_cell_ref<DIM, B>(a.m, n, c0, q, kind, src, c);
      if (kind < 0)
        raise_status(a.status, STATUS_MESH);
#pragma unroll
      for (int t = 0; t < T::NVI; ++t)
        sP[t * NP + i] = kind < 0 ? 0.0 : coarse_cell_value<DIM, B>(a.U + ((size_t)src * H::NV + vars[t]) * NC, kind, c);
    }
    __syncthreads();
    // 4. items (variable t, coarse cell cc): the cell's 2^dim children
    double * out = a.m.pg + (size_t)ps * H::NV * NG;
    for (int w = tid; w < T::NVI * ncc; w += NT)
    {
      const int t = w / ncc, cc = w - t * ncc;
      int       js = 0;
      while (js + 1 < nslot && sOff[js + 1] <= cc)
        ++js;
      int q[3] = { 0, 0, 0 };
      slot_cell(js, cc - sOff[js], q);
      const double * Pv = sP + t * NP + (q[0] + 1 + R) + P * ((q[1] + 1 + R) + (DIM == 3 ? P * (q[2] + 1 + R) : 0));
      double ch[NCHILD];
      prolong_children<DIM, MODE, P>(Pv, ch);
      double * o = out + (size_t)vars[t] * NG;
#pragma unroll
      for (int c = 0; c < NCHILD; ++c)
      {
        const int gx = 2 * q[0] + (c & 1), gy = 2 * q[1] + ((c >> 1) & 1), gz = DIM == 3 ? 2 * q[2] + ((c >> 2) & 1) : 0;
        o[DIM == 2 ? (gx + 2) + G * (gy + 2) : (gx + 2) + G * ((gy + 2) + G * (gz + 2))] = ch[c];
      }
    }
    __syncthreads();
    // 5. the two derived variables of every ghost cell
    for (int w = tid; w < ncc * NCHILD; w += NT)
    {
      const int cc = w / NCHILD, c = w - cc * NCHILD;
      int       js = 0;
      while (js + 1 < nslot && sOff[js + 1] <= cc)
        ++js;
      int q[3] = { 0, 0, 0 };
      slot_cell(js, cc - sOff[js], q);
      const int gx = 2 * q[0] + (c & 1), gy = 2 * q[1] + ((c >> 1) & 1), gz = DIM == 3 ? 2 * q[2] + ((c >> 2) & 1) : 0;
      double *  o = out + (DIM == 2 ? (gx + 2) + G * (gy + 2) : (gx + 2) + G * ((gy + 2) + G * (gz + 2)));
      o[(size_t)H::ID * NG] = o[(size_t)H::IAD0 * NG] + o[(size_t)H::IAD1 * NG];
      o[(size_t)H::IA1 * NG] = 1.0 - o[(size_t)H::IA0 * NG];
    }
  }
}

// ---------------------------------------------------------------------------
// Refined blocks of a mesh adaptation prolonged with the same types
// (map_userdata_after_adapt, SolverGodunovFiveEq.cpp:1137-1169: the
// UserDataRemapper keeps the old orchard keys for the stencil of this
// prolongation, :286-289): every fine cell of the children of an old block
// from its parent cell and the parent's neighbours at the old level, over the
// old block table.  A stencil point q (old-level cell coordinates relative to
// the old block, -R .. b+R-1) is the old block's cell, a same-level
// neighbour's cell, the coarser neighbour's cell holding it, or the mean of
// the 2^dim cells of a finer neighbour covering it — the values the ghost
// fill gives those cells.
// ---------------------------------------------------------------------------
template <int DIM, int B>
__device__ __forceinline__ void
level_cell_ref(const DevMesh & m, int n, const int * c0, const int * q, int & kind, int & src, int & c)
{
  constexpr int NS = DIM == 2 ? 9 : 27, NCH = DIM == 2 ? 4 : 8, H = B / 2;
  int           s[3] = { 0, 0, 0 }, v[3] = { 0, 0, 0 };
  bool          own = true;
#pragma unroll
  for (int e = 0; e < DIM; ++e)
  {
    s[e] = q[e] < 0 ? -1 : (q[e] >= B ? 1 : 0);
    v[e] = q[e] - s[e] * B;
    own = own && s[e] == 0;
  }
  auto cell = [&](const int * x) { return DIM == 2 ? x[0] + B * x[1] : x[0] + B * (x[1] + B * x[2]); };
  kind = 1;
  src = n;
  c = cell(v);
  if (own)
    return;
  const int       slot = DIM == 2 ? (s[0] + 1) + 3 * (s[1] + 1) : (s[0] + 1) + 3 * (s[1] + 1) + 9 * (s[2] + 1);
  const int       rel = m.nbr_rel[(size_t)n * NS + slot];
  const int32_t * nb = m.nbr + ((size_t)n * NS + slot) * NCH;
  if (rel == 0)
    src = nb[0];
  else if (rel < 0)
  {
    int cc[3] = { 0, 0, 0 };
#pragma unroll
    for (int e = 0; e < DIM; ++e)
      cc[e] = ((c0[e] + s[e]) & 1) * H + (v[e] >> 1);
    src = nb[0];
    c = cell(cc);
  }
  else
  {
    int ch[3] = { 0, 0, 0 }, l[3] = { 0, 0, 0 };
#pragma unroll
    for (int e = 0; e < DIM; ++e)
    {
      const int f = 2 * v[e];
      ch[e] = f >= B ? 1 : 0;
      l[e] = f - ch[e] * B;
    }
    kind = 0;
    src = nb[DIM == 2 ? ch[0] + 2 * ch[1] : ch[0] + 2 * ch[1] + 4 * ch[2]];
    c = cell(l);
  }
  if (src < 0 || src >= m.n_total)
    kind = -1;
}

template <int DIM, int B, int MODE>
struct RefineTraits
{
  static constexpr int R = MODE == 3 ? 2 : 1;
  static constexpr int P = B + 2 * R; // patch: the old block and R cells around it
  static constexpr int NP = DIM == 2 ? P * P : P * P * P;
  static constexpr int NVI = DIM == 2 ? 6 : 7;
  static constexpr int NC = DIM == 2 ? B * B : B * B * B;
  static constexpr int NT = 256;
  static constexpr size_t smem_bytes = sizeof(double) * (size_t)NVI * NP;
  static_assert(2 * R <= B, "the patch reaches past the children of a finer slot that touch the block");
};

// list[r * (1 + 2^DIM)]: the refined old block, then the new block of each
// of its children (child index x + 2 y + 4 z)
template <int DIM, int B, int MODE>
__global__ void __launch_bounds__(256)
prolong_refine_kernel(const double * __restrict__ Uold, double * __restrict__ Unew, DevMesh m, const int32_t * __restrict__ list,
                      int n_ref, unsigned int * status)
{
  using T = RefineTraits<DIM, B, MODE>;
  using H = V<DIM>;
  constexpr int R = T::R, P = T::P, NP = T::NP, NC = T::NC, NT = T::NT, HB = B / 2, NCHILD = 1 << DIM;
  extern __shared__ __align__(16) double sP[]; // [NVI][NP]
  const int vars[7] = { H::IAD0, H::IAD1, H::IA0, H::IE, H::IU, H::IV, H::IW };
  for (int r = blockIdx.x; r < n_ref; r += gridDim.x)
  {
    const int32_t * row = list + (size_t)r * (1 + NCHILD);
    const int       n = row[0];
    const int       c0[3] = { m.coord[n * 3 + 0], m.coord[n * 3 + 1], DIM == 3 ? m.coord[n * 3 + 2] : 0 };
    __syncthreads(); // the previous block's patch is read
    for (int i = threadIdx.x; i < NP; i += NT)
    {
      const int q[3] = { i % P - R, (i / P) % P - R, DIM == 3 ? i / (P * P) - R : 0 };
      int       kind, src, c;
      level_cell_ref<DIM, B>(m, n, c0, q, kind, src, c);
      if (kind < 0)
        raise_status(status, STATUS_MESH);
#pragma unroll
      for (int t = 0; t < T::NVI; ++t)
        sP[t * NP + i] = kind < 0 ? 0.0 : coarse_cell_value<DIM, B>(Uold + ((size_t)src * H::NV + vars[t]) * NC, kind, c);
    }
    __syncthreads();
    // items (variable t, old cell): the cell's 2^dim fine cells
    for (int w = threadIdx.x; w < T::NVI * NC; w += NT)
    {
      const int t = w / NC, oc = w - t * NC;
      const int q[3] = { oc % B, (oc / B) % B, DIM == 3 ? oc / (B * B) : 0 };
      double    ch[NCHILD];
      prolong_children<DIM, MODE, P>(sP + t * NP + (q[0] + R) + P * ((q[1] + R) + (DIM == 3 ? P * (q[2] + R) : 0)), ch);
      const int cb = (q[0] >= HB ? 1 : 0) + (q[1] >= HB ? 2 : 0) + (DIM == 3 && q[2] >= HB ? 4 : 0);
      double *  o = Unew + ((size_t)row[1 + cb] * H::NV + vars[t]) * NC;
      const int f0 = 2 * (q[0] % HB), f1 = 2 * (q[1] % HB), f2 = DIM == 3 ? 2 * (q[2] % HB) : 0;
#pragma unroll
      for (int c = 0; c < NCHILD; ++c)
        o[(f0 + (c & 1)) + B * ((f1 + ((c >> 1) & 1)) + (DIM == 3 ? B * (f2 + ((c >> 2) & 1)) : 0))] = ch[c];
    }
    __syncthreads();
    for (int w = threadIdx.x; w < NCHILD * NC; w += NT)
    {
      double * o = Unew + (size_t)row[1 + w / NC] * H::NV * NC + (w % NC);
      o[(size_t)H::ID * NC] = o[(size_t)H::IAD0 * NC] + o[(size_t)H::IAD1 * NC];
      o[(size_t)H::IA1 * NC] = 1.0 - o[(size_t)H::IA0 * NC];
    }
  }
}

} // namespace g5
