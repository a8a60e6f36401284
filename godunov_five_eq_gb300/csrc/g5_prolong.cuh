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
// child that touches the block when r <= b/4 - 1/2 (order 4 therefore needs
// 16-cell blocks: the block table lists only the touching children).
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
  static_assert(B >= 4 + 4 * R, "the patch reaches past the children of a finer slot that touch the block");
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

template <int DIM, int B, int MODE>
__global__ void __launch_bounds__(128)
prolong_kernel(StepArgs a)
{
  using T = ProlongTraits<DIM, B, MODE>;
  using H = V<DIM>;
  constexpr int R = T::R, P = T::P, NP = T::NP, G = T::G, NG = T::NG, NC = T::NC;
  extern __shared__ __align__(16) double sP[]; // [NVI][NP]
  const int vars[7] = { H::IAD0, H::IAD1, H::IA0, H::IE, H::IU, H::IV, H::IW };
  const int nwalk = step_count(a);
  for (int iw = blockIdx.x; iw < nwalk; iw += gridDim.x)
  {
    const int n = a.work ? a.work[iw] : iw;
    const int ps = a.m.pg_slot[n];
    if (ps < 0)
      continue;
    const int c0[3] = { a.m.coord[n * 3 + 0], a.m.coord[n * 3 + 1], DIM == 3 ? a.m.coord[n * 3 + 2] : 0 };
    __syncthreads(); // the previous block's patch is read
    for (int i = threadIdx.x; i < NP; i += T::NT)
    {
      int q[3] = { i % P - 1 - R, (i / P) % P - 1 - R, DIM == 3 ? i / (P * P) - 1 - R : 0 };
      int kind, src, c;
      coarse_cell_ref<DIM, B>(a.m, n, c0, q, kind, src, c);
      if (kind < 0)
        raise_status(a.status, STATUS_MESH);
#pragma unroll
      for (int t = 0; t < T::NVI; ++t)
        sP[t * NP + i] = kind < 0 ? 0.0 : coarse_cell_value<DIM, B>(a.U + ((size_t)src * H::NV + vars[t]) * NC, kind, c);
    }
    __syncthreads();
    double * out = a.m.pg + (size_t)ps * H::NV * NG;
    for (int gi = threadIdx.x; gi < NG; gi += T::NT)
    {
      int g[3] = { gi % G - 2, (gi / G) % G - 2, DIM == 3 ? gi / (G * G) - 2 : 0 };
      int s[3] = { 0, 0, 0 };
      bool inner = true;
#pragma unroll
      for (int e = 0; e < DIM; ++e)
      {
        s[e] = g[e] < 0 ? -1 : (g[e] >= B ? 1 : 0);
        inner = inner && s[e] == 0;
      }
      if (inner)
        continue;
      const int slot = DIM == 2 ? (s[0] + 1) + 3 * (s[1] + 1) : (s[0] + 1) + 3 * (s[1] + 1) + 9 * (s[2] + 1);
      if (a.m.nbr_rel[(size_t)n * T::NS + slot] >= 0)
        continue;
      int pc[3] = { 0, 0, 0 }, up[3] = { 0, 0, 0 };
#pragma unroll
      for (int e = 0; e < DIM; ++e)
      {
        pc[e] = (g[e] + 2) / 2 - 1 + 1 + R; // holding coarse cell, in patch coordinates
        up[e] = (g[e] + 2) & 1;
      }
      double u[H::NV];
#pragma unroll
      for (int t = 0; t < T::NVI; ++t)
      {
        const double * Pv = sP + t * NP;
        auto at = [&](int i, int j, int k) { return Pv[(pc[0] + i) + P * ((pc[1] + j) + (DIM == 3 ? P * (pc[2] + k) : 0))]; };
        double r;
        if constexpr (MODE == 1)
        {
          const double u0 = at(0, 0, 0);
          const double sx = slope_scalar<double>(u0, at(1, 0, 0), at(-1, 0, 0), 1.0);
          const double sy = slope_scalar<double>(u0, at(0, 1, 0), at(0, -1, 0), 1.0);
          r = u0;
          r = r + 0.25 * (double)(up[0] ? 1 : -1) * sx;
          r = r + 0.25 * (double)(up[1] ? 1 : -1) * sy;
          if constexpr (DIM == 3)
          {
            const double sz = slope_scalar<double>(u0, at(0, 0, 1), at(0, 0, -1), 1.0);
            r = r + 0.25 * (double)(up[2] ? 1 : -1) * sz;
          }
        }
        else
        {
          double valy[2 * R + 1];
#pragma unroll
          for (int k = (DIM == 3 ? -R : 0); k <= (DIM == 3 ? R : 0); ++k)
          {
            double valx[2 * R + 1];
#pragma unroll
            for (int j = -R; j <= R; ++j)
            {
              double acc = prolong_coef(MODE, up[0], -R) * at(-R, j, k);
#pragma unroll
              for (int i = -R + 1; i <= R; ++i)
                acc = acc + prolong_coef(MODE, up[0], i) * at(i, j, k);
              valx[j + R] = acc;
            }
            double acc = prolong_coef(MODE, up[1], -R) * valx[0];
#pragma unroll
            for (int j = -R + 1; j <= R; ++j)
              acc = acc + prolong_coef(MODE, up[1], j) * valx[j + R];
            valy[DIM == 3 ? k + R : 0] = acc;
          }
          if constexpr (DIM == 3)
          {
            double acc = prolong_coef(MODE, up[2], -R) * valy[0];
#pragma unroll
            for (int k = -R + 1; k <= R; ++k)
              acc = acc + prolong_coef(MODE, up[2], k) * valy[k + R];
            r = acc;
          }
          else
            r = valy[0];
        }
        u[vars[t]] = r;
      }
      u[H::ID] = u[H::IAD0] + u[H::IAD1];
      u[H::IA1] = 1.0 - u[H::IA0];
#pragma unroll
      for (int v = 0; v < H::NV; ++v)
        out[(size_t)v * NG + gi] = u[v];
    }
  }
}

} // namespace g5
