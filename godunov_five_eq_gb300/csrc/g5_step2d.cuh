// g5_step2d.cuh — fused 2D block timestep (one CTA per 16x16 or 8x8 block,
// persistent over the block list).
//
// Per block, entirely in shared memory:
//   1. gather the block and its 2-cell halo from U (same level: copy,
//      finer neighbour: mean of 4 fine cells, coarser neighbour: the coarse
//      cell) and convert to primitives                         (a2, a3)
//   2. per cell of the (b+2)^2 ring: limited slopes, sound speed and the
//      Hancock half-step source                                  (a5, a6)
//   3. per face: reconstruct both sides (MUSCL or THINC), HLLC, scale by
//      dt/dx                                                     (a6-a9)
//   4. per owned cell: X update + clamps, Y update + clamps, volume-fraction
//      renormalisation, write U2, CFL reduction of the new state  (a10-a12)
// Cells next to a finer face are deferred to the reflux kernel; fine blocks
// next to a coarser face publish their face fluxes for it.
#pragma once

#include "g5_common.cuh"

namespace g5
{

template <int B, bool MIXED>
struct Step2DTraits
{
  using R = typename std::conditional<MIXED, float, double>::type;
  static constexpr int NT = B * B;
  static constexpr int G = B + 4;  // ghosted extent
  static constexpr int S = B + 2;  // ring extent
  static constexpr int NQ = 6;     // r0 r1 p u v a0
  static constexpr int NREC = 15;  // dqx[5] dqy[5] hS[5] (the THINC normal is evaluated on demand)
  static constexpr int NFF = B * (B + 1);
  static constexpr size_t smem_bytes = sizeof(R) * (size_t)(NQ * G * G + NREC * S * S + 2 * 8 * NFF) + 64;
};

// halo cell h (0 .. G*G - B*B - 1) -> ghosted coordinates
template <int B>
__device__ __forceinline__ void
halo_coords(int h, int & gx, int & gy)
{
  constexpr int G = B + 4;
  if (h < 2 * G)
  {
    gx = h % G - 2;
    gy = h / G - 2;
    return;
  }
  h -= 2 * G;
  if (h < 2 * G)
  {
    gx = h % G - 2;
    gy = B + h / G;
    return;
  }
  h -= 2 * G;
  // side columns: 4 per row, rows 0..B-1
  const int r = h >> 2, c = h & 3;
  gy = r;
  gx = c < 2 ? c - 2 : B + (c - 2);
}

// load the conservative state seen by ghost cell (gx, gy) of block n.
// Returns false (and raises the mesh status) on a bad neighbour index.
// (cx0, cy0): the block's coordinates.  The slot's relation and its four
// neighbour entries are read in one wave (a 16-byte row), not one after the
// other: the gather is latency-bound.
template <int B>
__device__ __forceinline__ bool
gather_ghost_2d(const StepArgs & a, int n, int cx0, int cy0, int gx, int gy, double * u)
{
  using H = V<2>;
  constexpr int NC = B * B;
  const int     dxs = gx < 0 ? -1 : (gx >= B ? 1 : 0);
  const int     dys = gy < 0 ? -1 : (gy >= B ? 1 : 0);
  const int     vx = gx - dxs * B, vy = gy - dys * B;
  const int     s = (dxs + 1) + 3 * (dys + 1);
  const int     rel = a.m.nbr_rel[n * 9 + s];
  const int4    nb4 = *reinterpret_cast<const int4 *>(a.m.nbr + (n * 9 + s) * 4);
  const int     nb[4] = { nb4.x, nb4.y, nb4.z, nb4.w };
  if (rel == 0)
  {
    const int src = nb[0];
    if (src < 0 || src >= a.m.n_total)
      return false;
    const double * base = a.U + (size_t)src * H::NV * NC + vx + B * vy;
#pragma unroll
    for (int v = 0; v < H::NV; ++v)
      u[v] = base[v * NC];
    return true;
  }
  if (rel < 0)
  {
    if (a.m.pg)
    {
      // prolonged by the pre-pass (minmod extrapolation or conservative interpolation)
      constexpr int GG = (B + 4) * (B + 4);
      const int     ps = a.m.pg_slot[n];
      if (ps < 0)
        return false;
      const double * base = a.m.pg + (size_t)ps * H::NV * GG + (gx + 2) + (B + 4) * (gy + 2);
#pragma unroll
      for (int v = 0; v < H::NV; ++v)
        u[v] = base[v * GG];
      return true;
    }
    const int src = nb[0];
    if (src < 0 || src >= a.m.n_total)
      return false;
    const int cx = ((cx0 + dxs) & 1) * (B / 2) + (vx >> 1);
    const int cy = ((cy0 + dys) & 1) * (B / 2) + (vy >> 1);
    const double * base = a.U + (size_t)src * H::NV * NC + cx + B * cy;
#pragma unroll
    for (int v = 0; v < H::NV; ++v)
      u[v] = base[v * NC];
    return true;
  }
  // finer: mean of the 4 fine cells (sum in x-fastest order, then / 4)
  const int fx = 2 * vx, fy = 2 * vy;
  const int chx = fx / B, chy = fy / B;
  const int src = nb[chx + 2 * chy];
  if (src < 0 || src >= a.m.n_total)
    return false;
  const int      lx = fx - chx * B, ly = fy - chy * B;
  const double * base = a.U + (size_t)src * H::NV * NC + lx + B * ly;
  const int      vars[6] = { H::IE, H::IU, H::IV, H::IAD0, H::IAD1, H::IA0 };
  // lx is even: each pair of fine cells in x is one 16-byte load
#pragma unroll
  for (int t = 0; t < 6; ++t)
  {
    const double2 * p = reinterpret_cast<const double2 *>(base + vars[t] * NC);
    const double2   r0 = p[0], r1 = p[B / 2];
    double          sum = 0.0;
    sum += r0.x;
    sum += r0.y;
    sum += r1.x;
    sum += r1.y;
    u[vars[t]] = sum / 4.0;
  }
  u[H::IA1] = 1.0 - u[H::IA0];
  u[H::ID] = u[H::IAD0] + u[H::IAD1];
  return true;
}

template <int B, bool MIXED>
__device__ __forceinline__ void
store_prim(typename Step2DTraits<B, MIXED>::R * sQ, int gidx, const double * u, const PhysParams & P, int eosk)
{
  constexpr int GG = (B + 4) * (B + 4);
  if constexpr (MIXED)
  {
    float q[6];
    prim_mixed<2>(u, q, P, eosk);
#pragma unroll
    for (int k = 0; k < 6; ++k)
      sQ[k * GG + gidx] = q[k];
  }
  else
  {
    double q[6];
    prim_fp64<2>(u, q, P);
#pragma unroll
    for (int k = 0; k < 6; ++k)
      sQ[k * GG + gidx] = q[k];
  }
}

// Youngs normal (restated: (1,2,1)-weighted central differences), |n_x|, |n_y|
template <typename R, int G>
__device__ __forceinline__ void
youngs_abs_2d(const R * A, int gi, R & nx, R & ny)
{
  auto a = [&](int dx, int dy) { return A[gi + dx + G * dy]; };
  const R gx = (a(1, -1) + R(2) * a(1, 0) + a(1, 1)) - (a(-1, -1) + R(2) * a(-1, 0) + a(-1, 1));
  const R gy = (a(-1, 1) + R(2) * a(0, 1) + a(1, 1)) - (a(-1, -1) + R(2) * a(0, -1) + a(1, -1));
  R       nrm = gx * gx + gy * gy;
  nrm = sqrt(nrm);
  nx = (nrm > R(0)) ? fabs(-gx / nrm) : R(0);
  ny = (nrm > R(0)) ? fabs(-gy / nrm) : R(0);
}

// reconstruct one side of a face from cell (ci, cj) (ghosted-ring coordinates)
// dir: 0 X, 1 Y; side: +1 -> right face of the cell (qL), -1 -> left face (qR)
template <int B, bool MIXED>
__device__ __forceinline__ void
face_state(const typename Step2DTraits<B, MIXED>::R * sQ,
           const typename Step2DTraits<B, MIXED>::R * sRec,
           int                                          ci,
           int                                          cj,
           int                                          dir,
           int                                          side,
           const PhysParams &                           P,
           typename Step2DTraits<B, MIXED>::R *         q)
{
  using T = Step2DTraits<B, MIXED>;
  using R = typename T::R;
  constexpr int G = T::G, S = T::S, GG = G * G, SS = S * S;
  const int     gi = (ci + 2) + G * (cj + 2);
  const int     si = (ci + 1) + S * (cj + 1);
  const R       offx = dir == 0 ? R(0.5) * R(side) : R(0);
  const R       offy = dir == 1 ? R(0.5) * R(side) : R(0);
  const bool    hancock = P.integrator == 0;
  R             thinc_eps, thinc_beta, smallr;
  if constexpr (MIXED)
  {
    thinc_eps = P.f_thinc_eps;
    thinc_beta = P.f_thinc_beta;
    smallr = P.f_smallr;
  }
  else
  {
    thinc_eps = P.thinc_eps;
    thinc_beta = P.thinc_beta;
    smallr = P.smallr;
  }
  R qc[5], dqx[5], dqy[5], hs[5];
#pragma unroll
  for (int k = 0; k < 5; ++k)
  {
    qc[k] = sQ[k * GG + gi];
    dqx[k] = sRec[k * SS + si];
    dqy[k] = sRec[(5 + k) * SS + si];
    hs[k] = sRec[(10 + k) * SS + si];
  }
  const R a0 = sQ[5 * GG + gi];
#pragma unroll
  for (int k = 0; k < 5; ++k)
  {
    if constexpr (MIXED)
      q[k] = qc[k] + offx * dqx[k] + offy * dqy[k] + (hancock ? hs[k] : R(0));
    else
    {
      q[k] = qc[k] + offx * dqx[k] + offy * dqy[k];
      if (hancock)
        q[k] += hs[k];
    }
  }
  q[5] = a0;
  if (P.thinc)
  {
    // THINC (scheme/ComputeFluxesAndStoreTHINCFunctor.cpp:122-283): alpha
    // and the partial densities from the hyperbolic-tangent profile
    const int  o = dir == 0 ? 1 : G;
    const R *  A = sQ + 5 * GG;
    const R    aP = A[gi + o], aM = A[gi - o];
    const R    mono = (aP - a0) * (a0 - aM);
    const bool req = (a0 > thinc_eps) && (a0 < R(1) - thinc_eps) && mono > R(0);
    if (req)
    {
      R nxa, nya;
      youngs_abs_2d<R, G>(A, gi, nxa, nya);
      const R nd = dir == 0 ? nxa : nya;
      const R beta = thinc_beta * nd + R(0.01);
      const R Aa = (aP + aM) / R(2);
      const R Bb = (aP - aM) / R(2);
      R       C, D;
      if constexpr (MIXED)
      {
        C = tanhf(R(0.5) * beta);
        D = tanhf(R(0.5) * beta * (a0 - Aa) / Bb);
      }
      else
      {
        C = tanh_d(R(0.5) * beta);
        D = tanh_d(R(0.5) * beta * (a0 - Aa) / Bb);
      }
      const R bs = R(side);
      const R af = Aa + bs * Bb * (C + bs * D / C) / (R(1) + bs * D);
      const R r0 = qc[0], r1 = qc[1];
      R       q0 = r0 + r0 / a0 * (af - a0);
      R       q1 = r1 + r1 / (R(1) - a0) * (a0 - af);
      if (hancock)
      {
        q0 += hs[0];
        q1 += hs[1];
      }
      q[0] = q0;
      q[1] = q1;
      q[5] = af;
    }
    // THINC functor: no smallr clamp on the partial densities
  }
  else
  {
    q[0] = fmax(smallr, q[0]);
    q[1] = fmax(smallr, q[1]);
  }
}

// The mixed form of face_state for a face direction known at compile time:
// q = (q + hs) + off * dq_dir, with q + hs stored by the slope phase, so a
// face side reads 11 values of shared memory instead of 21.
template <int B, int DIR, bool THINC>
__device__ __forceinline__ void
face_state_mixed(const float * sQ, const float * sRec, int ci, int cj, int side, const PhysParams & P, float * q)
{
  using T = Step2DTraits<B, true>;
  constexpr int G = T::G, S = T::S, GG = G * G, SS = S * S;
  const int     gi = (ci + 2) + G * (cj + 2);
  const int     si = (ci + 1) + S * (cj + 1);
  const float   off = 0.5f * (float)side;
  const float * dq = sRec + (DIR == 0 ? 0 : 5 * SS);
#pragma unroll
  for (int k = 0; k < 5; ++k)
    q[k] = sRec[(10 + k) * SS + si] + off * dq[k * SS + si];
  const float a0 = sQ[5 * GG + gi];
  q[5] = a0;
  if constexpr (THINC)
  {
    // THINC (scheme/ComputeFluxesAndStoreTHINCFunctor.cpp:122-283)
    constexpr int o = DIR == 0 ? 1 : G;
    const float * A = sQ + 5 * GG;
    const float   aP = A[gi + o], aM = A[gi - o];
    const float   mono = (aP - a0) * (a0 - aM);
    const float   eps = P.f_thinc_eps;
    if ((a0 > eps) && (a0 < 1.0f - eps) && mono > 0.0f)
    {
      float nxa, nya;
      youngs_abs_2d<float, G>(A, gi, nxa, nya);
      const float nd = DIR == 0 ? nxa : nya;
      const float beta = P.f_thinc_beta * nd + 0.01f;
      const float Aa = (aP + aM) / 2.0f;
      const float Bb = (aP - aM) / 2.0f;
      const float C = tanhf(0.5f * beta);
      const float D = tanhf(0.5f * beta * (a0 - Aa) / Bb);
      const float bs = (float)side;
      const float af = Aa + bs * Bb * (C + bs * D / C) / (1.0f + bs * D);
      const float r0 = sQ[0 * GG + gi], r1 = sQ[1 * GG + gi];
      // (r + hs) + r / a0 (af - a0): the partial densities rescaled (eq. 45)
      q[0] = sRec[10 * SS + si] + r0 / a0 * (af - a0);
      q[1] = sRec[11 * SS + si] + r1 / (1.0f - a0) * (a0 - af);
      q[5] = af;
    }
  }
  else
  {
    q[0] = fmaxf(P.f_smallr, q[0]);
    q[1] = fmaxf(P.f_smallr, q[1]);
  }
}

// HLLC flux of one face of the mixed form, scaled by dt/dx into the shared
// flux arrays; DIR selects the face set (X faces (B+1) x B, Y faces B x (B+1))
template <int B, int DIR, bool THINC, bool MG>
__device__ __forceinline__ void
face_flux_mixed(const float * sQ, const float * sRec, float * sF, int ff, float dtdx, const PhysParams & P)
{
  using H = V<2>;
  constexpr int NFF = B * (B + 1);
  int           li, lj, ri, rj;
  if (DIR == 0)
  {
    const int fi = ff % (B + 1), fj = ff / (B + 1);
    li = fi - 1;
    lj = fj;
    ri = fi;
    rj = fj;
  }
  else
  {
    const int fi = ff % B, fj = ff / B;
    li = fi;
    lj = fj - 1;
    ri = fi;
    rj = fj;
  }
  float qL[6], qR[6], fl[8];
  face_state_mixed<B, DIR, THINC>(sQ, sRec, li, lj, +1, P, qL);
  face_state_mixed<B, DIR, THINC>(sQ, sRec, ri, rj, -1, P, qR);
  if (DIR == 1)
  {
    float t = qL[3];
    qL[3] = qL[4];
    qL[4] = t;
    t = qR[3];
    qR[3] = qR[4];
    qR[4] = t;
  }
  hllc_fp32<2>(qL, qR, P.f_xi[0], P.f_xi[1], P.f_gpx[0], P.f_gpx[1], P.f_smallr, P.f_smallp, P.f_smallc, fl, MG ? &P : nullptr);
  if (DIR == 1)
  {
    const float t = fl[H::FU];
    fl[H::FU] = fl[H::FV];
    fl[H::FV] = t;
  }
#pragma unroll
  for (int k = 0; k < 8; ++k)
    sF[k * NFF + ff] = fl[k] * dtdx;
}

// ReadFluxesAndConservativeUpdateFunctor (X then Y, update_U with the
// per-direction clamps, .cpp:115-305, .h:319-349), FixVolumeFractionsNormalization
// (.cpp:49-72) and the CFL rate of the new state (ComputeDtFiveEqFunctor.cpp:87-134),
// FP64 in the reference's operation order.  Returns the cell's CFL rate (or 0).
template <int B>
__device__ __forceinline__ double
update_fp64(const double * uin, double * u2, const double * sFx, const double * sFy, int ci, int cj, double dx, const PhysParams & P, bool want_dt)
{
  using H = V<2>;
  constexpr int NFF = B * (B + 1);
#pragma unroll
  for (int v = 0; v < H::NV; ++v)
    u2[v] = uin[v];
  const double a0n = uin[H::IA0], a1n = uin[H::IA1];
  double       st0, st1;
  source_factors_fp64<2>(uin, P, st0, st1);
#pragma unroll
  for (int dir = 0; dir < 2; ++dir)
  {
    const double * F = dir == 0 ? sFx : sFy;
    const int      il = dir == 0 ? ci + (B + 1) * cj : ci + B * cj;
    const int      ir = dir == 0 ? il + 1 : il + B;
    double         acc[7];
#pragma unroll
    for (int k = 0; k < 7; ++k)
      acc[k] = 0.0 + F[k * NFF + il];
    const double usl = F[7 * NFF + il];
    acc[H::FA0] -= st0 * usl * a0n;
    acc[H::FA1] -= st1 * usl * a1n;
#pragma unroll
    for (int k = 0; k < 7; ++k)
      acc[k] = acc[k] - F[k * NFF + ir];
    const double usr = F[7 * NFF + ir];
    acc[H::FA0] += st0 * usr * a0n;
    acc[H::FA1] += st1 * usr * a1n;
    const double eps = 1e-12;
    u2[H::IAD0] += acc[H::FR0];
    if (u2[H::IAD0] < eps)
      u2[H::IAD0] = 0.0;
    u2[H::IAD1] += acc[H::FR1];
    if (u2[H::IAD1] < eps)
      u2[H::IAD1] = 0.0;
    u2[H::IA0] += acc[H::FA0];
    if (u2[H::IA0] < eps)
      u2[H::IA0] = 0.0;
    if (u2[H::IA0] > 1.0 - eps)
      u2[H::IA0] = 1.0;
    u2[H::IA1] += acc[H::FA1];
    if (u2[H::IA1] < eps)
      u2[H::IA1] = 0.0;
    if (u2[H::IA1] > 1.0 - eps)
      u2[H::IA1] = 1.0;
    u2[H::IE] += acc[H::FE];
    u2[H::IU] += acc[H::FU];
    u2[H::IV] += acc[H::FV];
  }
  const double sum_alpha = u2[H::IA0] + u2[H::IA1];
  const double sum_alpha_rho = u2[H::IAD0] + u2[H::IAD1];
  const double inv = 1.0 / sum_alpha;
  u2[H::IA0] *= inv;
  u2[H::IA1] *= inv;
  u2[H::ID] = sum_alpha_rho;
  if (!want_dt)
    return 0.0;
  double       q[6];
  const double c = prim_fp64<2>(u2, q, P);
  return (c + fabs(q[H::QU])) / dx + (c + fabs(q[H::QV])) / dx;
}

// The same update in the FP32-bulk form.  FP64 is used only for the adds
// into the stored state: the face fluxes of both directions are summed as a
// float-float pair (error-free differences and sums), turned into a double on
// the integer pipe (ff_to_d, exact but for bits below 2^-53 of the sum) and
// added with one FP64 add, so per-material mass is conserved to FP64
// round-off; the clamps run on the integer pipe; the renormalisation divides
// by 1 + d as a multiply by (1 - d) when |d| < 1e-8 (exact to FP64 rounding).
//
// apply_mixed_2d takes the per-direction increments: h + l (float pairs) of
// r0 r1 e u v and dA (floats, source term included) of alpha0 alpha1; u2 holds
// the old state on entry.  Returns the CFL rate of the new state (or 0).
__device__ __forceinline__ float
apply_mixed_2d(const double * uin, double * u2, const float (&h)[2][5], const float (&l)[2][5], const float (&dA)[2][2], float dx,
               const PhysParams & P, int eosk, bool want_dt)
{
  using H = V<2>;
  const double eps = 1e-12, one_m_eps = 1.0 - 1e-12;
  // partial densities: clamp after X cannot trigger when the state dominates
  // the X decrease (checked in FP32 with a factor-2 margin); then both
  // directions are summed in float-float and added with one FP64 add,
  // otherwise the X and Y increments are applied one after the other.
#pragma unroll
  for (int k = 0; k < 2; ++k)
  {
    const int   iv = k == 0 ? H::IAD0 : H::IAD1;
    const float uf = d2f_fast(u2[iv]);
    if (uf > 2.0f * fabsf(h[0][k]) + 2e-12f)
    {
      float s, t;
      two_sum(h[0][k], h[1][k], s, t);
      two_sum(s, t + (l[0][k] + l[1][k]), s, t);
      u2[iv] += ff_to_d(s, t);
      if (dlt_pos(u2[iv], eps))
        u2[iv] = 0.0;
    }
    else
    {
#pragma unroll
      for (int dir = 0; dir < 2; ++dir)
      {
        u2[iv] = (u2[iv] + f2d_exact(h[dir][k])) + f2d_exact(l[dir][k]);
        if (dlt_pos(u2[iv], eps))
          u2[iv] = 0.0;
      }
    }
  }
  // volume fractions: the same test against both clamp bounds
#pragma unroll
  for (int k = 0; k < 2; ++k)
  {
    const int   iv = k == 0 ? H::IA0 : H::IA1;
    const float af = d2f_fast(uin[iv]);
    const float m = 2.0f * fabsf(dA[0][k]) + 2e-12f;
    if (af > m && af + m < 1.0f)
    {
      u2[iv] += f2d_exact(dA[0][k] + dA[1][k]);
      if (dlt_pos(u2[iv], eps))
        u2[iv] = 0.0;
      if (dgt_pos(u2[iv], one_m_eps))
        u2[iv] = 1.0;
    }
    else
    {
#pragma unroll
      for (int dir = 0; dir < 2; ++dir)
      {
        u2[iv] += f2d_exact(dA[dir][k]);
        if (dlt_pos(u2[iv], eps))
          u2[iv] = 0.0;
        if (dgt_pos(u2[iv], one_m_eps))
          u2[iv] = 1.0;
      }
    }
  }
  // energy and momentum: no clamps, one float-float sum of both directions
  const int ive[3] = { H::IE, H::IU, H::IV };
#pragma unroll
  for (int e = 0; e < 3; ++e)
  {
    float s, t;
    two_sum(h[0][2 + e], h[1][2 + e], s, t);
    two_sum(s, t + (l[0][2 + e] + l[1][2 + e]), s, t);
    u2[ive[e]] += ff_to_d(s, t);
  }
  // renormalisation
  const double sa = u2[H::IA0] + u2[H::IA1];
  const double d = sa - 1.0;
  if (d != 0.0)
  {
    if ((__double_as_longlong(d) & 0x7FFFFFFFFFFFFFFFLL) < __double_as_longlong(1e-8))
    {
      u2[H::IA0] = fma(-u2[H::IA0], d, u2[H::IA0]);
      u2[H::IA1] = fma(-u2[H::IA1], d, u2[H::IA1]);
    }
    else
    {
      const double inv = 1.0 / sa;
      u2[H::IA0] *= inv;
      u2[H::IA1] *= inv;
    }
  }
  u2[H::ID] = u2[H::IAD0] + u2[H::IAD1];
  if (!want_dt)
    return 0.0f;
  float       df, ux, uy, uz, a0;
  const float p = pressure_mixed<2>(u2, P, eosk, df, ux, uy, uz, a0);
  const float a0s = fmaxf(0.0f, fminf(1.0f, a0));
  const float c = sound_speed_eos(P, eosk, df, p, a0s, d2f_fast(u2[H::IAD0]), d2f_fast(u2[H::IAD1]));
  return ((c + fabsf(ux)) + (c + fabsf(uy))) * __frcp_rn(dx);
}

template <int B>
__device__ __forceinline__ float
update_mixed(const double * uin, double * u2, const float * sFx, const float * sFy, int ci, int cj, float dx, const PhysParams & P, int eosk, bool want_dt)
{
  using H = V<2>;
  constexpr int NFF = B * (B + 1);
#pragma unroll
  for (int v = 0; v < H::NV; ++v)
    u2[v] = uin[v];
  float        a0f = d2f_fast(uin[H::IA0]), a1f = d2f_fast(uin[H::IA1]);
  {
    float st0, st1;
    source_factors_mixed<2>(uin, P, eosk, st0, st1);
    a0f *= st0;
    a1f *= st1;
  }
  const int    ilx = ci + (B + 1) * cj, irx = ilx + 1;
  const int    ily = ci + B * cj, iry = ily + B;
  // error-free per-direction increments of the conserved quantities:
  // d[dir] = F_left - F_right = h + l exactly
  float h[2][5], l[2][5];
  const int ks[5] = { H::FR0, H::FR1, H::FE, H::FU, H::FV };
#pragma unroll
  for (int k = 0; k < 5; ++k)
  {
    // both directions in one packed transformation
    float2 hi, lo;
    two_diff2(make_float2(sFx[ks[k] * NFF + ilx], sFy[ks[k] * NFF + ily]), make_float2(sFx[ks[k] * NFF + irx], sFy[ks[k] * NFF + iry]), hi, lo);
    h[0][k] = hi.x;
    h[1][k] = hi.y;
    l[0][k] = lo.x;
    l[1][k] = lo.y;
  }
  float dA[2][2];
  {
    const float uslx = sFx[H::FUS * NFF + ilx], usrx = sFx[H::FUS * NFF + irx];
    const float usly = sFy[H::FUS * NFF + ily], usry = sFy[H::FUS * NFF + iry];
    dA[0][0] = ((sFx[H::FA0 * NFF + ilx] - uslx * a0f) - sFx[H::FA0 * NFF + irx]) + usrx * a0f;
    dA[0][1] = ((sFx[H::FA1 * NFF + ilx] - uslx * a1f) - sFx[H::FA1 * NFF + irx]) + usrx * a1f;
    dA[1][0] = ((sFy[H::FA0 * NFF + ily] - usly * a0f) - sFy[H::FA0 * NFF + iry]) + usry * a0f;
    dA[1][1] = ((sFy[H::FA1 * NFF + ily] - usly * a1f) - sFy[H::FA1 * NFF + iry]) + usry * a1f;
  }
  return apply_mixed_2d(uin, u2, h, l, dA, dx, P, eosk, want_dt);
}


template <int B>
__device__ __forceinline__ void reflux2d_lanes(const StepArgs & a, int rec, int pos, bool act);

// Reflux in the step kernel's tail (FP32-bulk form): the deferred cells of
// deferred block j (its records fin_rec[j * 4 ..]) on the NT threads of the
// calling CTA, eight lanes per cell (whole warps: B * 8 lanes per record)
template <int B, int NT>
__device__ __forceinline__ void
finish_deferred_2d(const StepArgs & a, int j)
{
  constexpr int PER = B * 8;
  static_assert(PER % 32 == 0 && NT % 32 == 0, "whole warps per record");
  const int4 rr = *reinterpret_cast<const int4 *>(a.m.fin_rec + (size_t)j * 4);
  const int  nrec = (rr.x >= 0) + (rr.y >= 0) + (rr.z >= 0) + (rr.w >= 0);
  for (int base = 0; base < nrec * PER; base += NT)
  {
    const int  item = base + (int)threadIdx.x;
    const bool act = item < nrec * PER;
    const int  slot = act ? item / PER : 0;
    const int  rec = slot == 0 ? rr.x : (slot == 1 ? rr.y : (slot == 2 ? rr.z : rr.w));
    reflux2d_lanes<B>(a, rec, (item >> 3) % B, act);
  }
}

// 4 CTAs per SM in the FP32-bulk form (64 registers), so that CTAs in the
// FP64-heavy update overlap with CTAs in the FP32 face phase; 2 CTAs per SM
// (128 registers) in the FP64 form
// THINC, STIFF: the FP32-bulk form is compiled with and without the THINC
// reconstruction and the stiffened-gas pressure path (P picks the kernel), so
// a kernel carries only the code its case runs; the FP64 form tests both at
// run time (STIFF = -1).  FUSED: the FP32-bulk form finishing the coarse/fine
// records in its tail (m.fin_tgt set; the kernel without it keeps the plain
// block loop)
template <int B, bool MIXED, bool THINC = false, int STIFF = -1, bool FUSED = false>
__global__ void __launch_bounds__(B * B, MIXED ? (B == 16 ? 4 : 8) : (B == 16 ? 2 : 8))
step2d_kernel(StepArgs a)
{
  using T = Step2DTraits<B, MIXED>;
  using R = typename T::R;
  using H = V<2>;
  constexpr int NT = T::NT, G = T::G, S = T::S, GG = G * G, SS = S * S, NC = B * B;
  constexpr int NFF = T::NFF;
  constexpr int NHALO = GG - NC;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  R *          sQ = reinterpret_cast<R *>(smem_raw);
  R *          sRec = sQ + T::NQ * GG;
  R *          sFx = sRec + T::NREC * SS; // [8][NFF]  X faces (B+1) x B
  R *          sFy = sFx + 8 * NFF;       // [8][NFF]  Y faces B x (B+1)
  using DtT = typename std::conditional<MIXED, float, double>::type;
  __shared__ DtT sRed[NT / 32];
  __shared__ int sSlot[10]; // the block's reflux slots (faces 0-3), its defer slots, its outside-twin range
  __shared__ int sNext;     // the CTA's next block
  __shared__ int sFin[6];   // reflux in the tail: deferred blocks to finish, end of the claims
  static_assert(T::NREC * T::S * T::S * sizeof(R) >= H::NV * B * B * sizeof(double), "twin staging does not fit the slope area");
  const int         tid = threadIdx.x;
  const PhysParams & P = a.p;
  // the equation of state: 0 ideal gases, 1 a stiffened-gas constant (the
  // pressure numerator cancels: FP64 there), 2 Mie-Grueneisen laws
  const int eosk = STIFF < 0 ? (P.mg_any ? 2 : ((P.gpx[0] != 0.0 || P.gpx[1] != 0.0) ? 1 : 0)) : STIFF;

  const int nwalk = step_count(a);
  // reflux in the tail (FP32-bulk form, FUSED, m.fin_tgt set): after its step a
  // block counts itself off the counters of the deferred blocks whose records
  // it completes (its own and those of the coarser blocks it publishes to);
  // a CTA out of blocks claims deferred blocks by ticket and counts a claim
  // off; whoever brings a counter to zero finishes that block's deferred
  // cells.  Release: the barrier orders the CTA's writes before the counting
  // thread's device-scope fence and atomic; acquire: that thread's fence
  // after the atomic, then the barrier.
  constexpr bool fused = MIXED && FUSED;
  for (int iw = blockIdx.x;;)
  {
    int next = iw;
    if (iw < nwalk)
    {
      const int    n = a.work ? a.work[iw] : iw;
      const int    fin_v = (fused && tid >= 16 && tid < 21) ? a.m.fin_tgt[n * 5 + tid - 16] : -1;
      // (a block with no counter to count off skips the tail's barriers)
      const bool   counts = fused && a.m.fin_tgt[n * 5] >= 0;
      const int    lev = a.m.level[n];
      const int    cx0 = a.m.coord[n * 3 + 0], cy0 = a.m.coord[n * 3 + 1];
      // the next block is claimed now (the ticket's latency hides behind the gather)
      const int    next_v = tid == 10 ? claim_next(a, iw, nwalk) : 0;
      // coarse/fine slots: loaded now, stored to shared memory at the end of the
      // gather (their latency hides behind it)
      int slot_v = -1;
      if (a.m.reflux_slot && tid < 8)
        slot_v = tid < 4 ? a.m.reflux_slot[n * 4 + tid] : a.m.defer_slot[n * 4 + tid - 4];
      if (tid == 8 || tid == 9)
        slot_v = a.fill_twins ? a.m.twin_first[n + tid - 8] : 0;
      const int    ins = a.m.inst ? a.m.inst[n] : 0;
      const double dx = P.level_dx[lev];
      R            dtdx_r;
      if constexpr (MIXED)
        dtdx_r = d2f_fast(a.dt[ins]) * __frcp_rn(d2f_fast(dx));
      else
        dtdx_r = a.dt[ins] / dx;

      // ---------------- phase 1: own cell (coalesced) + halo gather -> primitives
      // (the own cell's loads are in flight while the halo gather runs; its
      // primitives are stored last)
      const int ci = tid % B, cj = tid / B;
      double    uin[H::NV];
      {
        const double * base = a.U + (size_t)n * H::NV * NC + tid;
#pragma unroll
        for (int v = 0; v < H::NV; ++v)
          uin[v] = base[v * NC];
      }
      for (int h = tid; h < NHALO; h += NT)
      {
        int gx, gy;
        halo_coords<B>(h, gx, gy);
        double u[H::NV];
        if (!gather_ghost_2d<B>(a, n, cx0, cy0, gx, gy, u))
        {
          raise_status(a.status, STATUS_MESH);
#pragma unroll
          for (int v = 0; v < H::NV; ++v)
            u[v] = uin[v];
        }
        store_prim<B, MIXED>(sQ, (gx + 2) + G * (gy + 2), u, P, eosk);
      }
      store_prim<B, MIXED>(sQ, (ci + 2) + G * (cj + 2), uin, P, eosk);
      if (tid < 10)
        sSlot[tid] = slot_v;
      if (tid == 10)
        sNext = next_v;
      __syncthreads();
      // the next block of this CTA: its own cells and table rows into L2 while
      // this block computes (its gather then hits L2 instead of HBM)
      if (tid < 3 && sNext < nwalk)
      {
        const int nn = a.work ? a.work[sNext] : sNext;
        if (tid == 0)
          prefetch_l2_range(a.U + (size_t)nn * H::NV * NC, (unsigned)(H::NV * NC * sizeof(double)));
        else if (tid == 1)
          prefetch_l2_line(a.m.nbr + (size_t)nn * 36);
        else
          prefetch_l2_line(a.m.nbr_rel + (size_t)nn * 9);
      }

      // ---------------- phase 2: per face-neighbour cell slopes + Hancock source
      // (the block, then the row or column beyond each face, without gaps: the
      // ring's corners are never a face neighbour; r: the cell's index in the
      // ring layout)
      for (int h = tid; h < NC + 4 * B; h += NT)
      {
        int ri, rj;
        if (h < NC)
        {
          ri = h % B;
          rj = h / B;
        }
        else
        {
          const int i = h - NC, f = i / B, pa = i % B;
          const int side = (f & 1) ? B : -1;
          ri = f < 2 ? side : pa;
          rj = f < 2 ? pa : side;
        }
        const int r = (ri + 1) + S * (rj + 1);
        const int gi = (ri + 2) + G * (rj + 2);
        R         q[5], dqx[5], dqy[5];
        R st;
        if constexpr (MIXED)
          st = P.f_slope_type;
        else
          st = P.slope_type;
#pragma unroll
        for (int k = 0; k < 5; ++k)
        {
          const R * Qk = sQ + k * GG;
          q[k] = Qk[gi];
          dqx[k] = slope_scalar<R>(q[k], Qk[gi + 1], Qk[gi - 1], st);
          dqy[k] = slope_scalar<R>(q[k], Qk[gi + G], Qk[gi - G], st);
          sRec[k * SS + r] = dqx[k];
          sRec[(5 + k) * SS + r] = dqy[k];
        }
        const R a0 = sQ[5 * GG + gi];
        if (P.integrator == 0)
        {
          // Hancock half-step source (ComputeFluxesAndStoreFunctor.cpp:174-199)
          const R r0 = q[0], r1 = q[1], p = q[2], u = q[3], v = q[4];
          const R rr = r0 + r1;
          R       c;
          if constexpr (MIXED)
            c = sound_speed_eos(P, eosk, rr, p, a0, r0, r1);
          else
            c = sound_speed_mix(P, rr, p, a0, 1 - a0, r0, r1);
          const R drx0 = dqx[0], drx1 = dqx[1], dpx = dqx[2], dux = dqx[3], dvx = dqx[4];
          const R dry0 = dqy[0], dry1 = dqy[1], dpy = dqy[2], duy = dqy[3], dvy = dqy[4];
          const R dtdy = dtdx_r;
          const R sr0 = (-u * (drx0 + drx1) - dux * rr) * dtdx_r + (-v * (dry0 + dry1) - dvy * rr) * dtdy;
          const R sr0_0 = sr0 * a0;
          const R sr0_1 = sr0 * (R(1) - a0);
          const R su0 = (-u * dux - dpx / rr) * dtdx_r + (-v * duy) * dtdy;
          const R sv0 = (-u * dvx) * dtdx_r + (-v * dvy - dpy / rr) * dtdy;
          const R sp0 = (-u * dpx - dux * rr * c * c) * dtdx_r + (-v * dpy - dvy * rr * c * c) * dtdy;
          if constexpr (MIXED)
          {
            // the mixed form stores the predicted centre value q + hs
            sRec[10 * SS + r] = q[0] + R(0.5) * sr0_0;
            sRec[11 * SS + r] = q[1] + R(0.5) * sr0_1;
            sRec[12 * SS + r] = q[2] + R(0.5) * sp0;
            sRec[13 * SS + r] = q[3] + R(0.5) * su0;
            sRec[14 * SS + r] = q[4] + R(0.5) * sv0;
          }
          else
          {
            sRec[10 * SS + r] = R(0.5) * sr0_0;
            sRec[11 * SS + r] = R(0.5) * sr0_1;
            sRec[12 * SS + r] = R(0.5) * sp0;
            sRec[13 * SS + r] = R(0.5) * su0;
            sRec[14 * SS + r] = R(0.5) * sv0;
          }
        }
        else if constexpr (MIXED)
        {
#pragma unroll
          for (int k = 0; k < 5; ++k)
            sRec[(10 + k) * SS + r] = q[k];
        }
      }
      __syncthreads();

      // ---------------- phase 3: faces (X then Y) -> HLLC -> shared fluxes
      if constexpr (MIXED)
      {
        for (int f = tid; f < 2 * NFF; f += NT)
        {
          if (f < NFF)
            face_flux_mixed<B, 0, THINC, STIFF == 2>(sQ, sRec, sFx, f, dtdx_r, P);
          else
            face_flux_mixed<B, 1, THINC, STIFF == 2>(sQ, sRec, sFy, f - NFF, dtdx_r, P);
        }
      }
      else
      for (int f = tid; f < 2 * NFF; f += NT)
      {
        const int dir = f >= NFF ? 1 : 0;
        const int ff = f - dir * NFF;
        int       li, lj, ri, rj;
        if (dir == 0)
        {
          const int fi = ff % (B + 1), fj = ff / (B + 1);
          li = fi - 1;
          lj = fj;
          ri = fi;
          rj = fj;
        }
        else
        {
          const int fi = ff % B, fj = ff / B;
          li = fi;
          lj = fj - 1;
          ri = fi;
          rj = fj;
        }
        R qL[6], qR[6], fl[8];
        face_state<B, MIXED>(sQ, sRec, li, lj, dir, +1, P, qL);
        face_state<B, MIXED>(sQ, sRec, ri, rj, dir, -1, P, qR);
        if (dir == 1)
        {
          R t = qL[3];
          qL[3] = qL[4];
          qL[4] = t;
          t = qR[3];
          qR[3] = qR[4];
          qR[4] = t;
        }
        if constexpr (MIXED)
          hllc_fp32<2>(qL, qR, P.f_xi[0], P.f_xi[1], P.f_gpx[0], P.f_gpx[1], P.f_smallr, P.f_smallp, P.f_smallc, fl);
        else
          hllc_fp64<2>(qL, qR, P, fl);
        if (dir == 1)
        {
          const R t = fl[H::FU];
          fl[H::FU] = fl[H::FV];
          fl[H::FV] = t;
        }
        R * dst = dir == 0 ? sFx : sFy;
#pragma unroll
        for (int k = 0; k < 8; ++k)
          dst[k * NFF + ff] = fl[k] * dtdx_r;
      }
      // the own cell's state for the update: the FP32-bulk form without the
      // tail reflux reads it again (an L2 hit, in flight while the CTA waits at
      // the barrier) instead of holding its eight doubles in registers through
      // the slope and face phases (-2 % on the droplet batch; the tail-reflux
      // kernel, with its few rounds of blocks, was 0.4 % slower with it)
      double uown[H::NV];
      if constexpr (MIXED && !FUSED)
      {
        const double * base = a.U + (size_t)n * H::NV * NC + tid;
#pragma unroll
        for (int v = 0; v < H::NV; ++v)
          uown[v] = __ldcg(base + v * NC);
      }
      else
      {
#pragma unroll
        for (int v = 0; v < H::NV; ++v)
          uown[v] = uin[v];
      }
      __syncthreads();

      // ---------------- publish coarse/fine records (AMR only)
      if (a.m.reflux_slot)
      {
#pragma unroll
        for (int face = 0; face < 4; ++face)
        {
          const int rs = sSlot[face];
          if (rs >= 0 && tid < B)
          {
            // fine block face next to a coarser neighbour: publish its B face fluxes
            const int dir = face >> 1, side = face & 1;
            const int idx = dir == 0 ? (side ? B : 0) + (B + 1) * tid : tid + B * (side ? B : 0);
            const R * src = dir == 0 ? sFx : sFy;
            // the mixed form keeps the float fluxes (the buffer read as floats)
            R * dst = reinterpret_cast<R *>(a.reflux_buf) + ((size_t)rs * B + tid) * 8;
#pragma unroll
            for (int k = 0; k < 8; ++k)
              dst[k] = src[k * NFF + idx];
          }
          const int ds = sSlot[4 + face];
          if (ds >= 0 && tid < B)
          {
            // coarse cell next to a finer face: save its four own face fluxes
            const int dir = face >> 1, side = face & 1;
            const int cx = dir == 0 ? (side ? B - 1 : 0) : tid;
            const int cy = dir == 0 ? tid : (side ? B - 1 : 0);
            R *       dst = reinterpret_cast<R *>(a.defer_buf) + ((size_t)ds * B + tid) * 32;
            const int fxl = cx + (B + 1) * cy, fyl = cx + B * cy;
#pragma unroll
            for (int k = 0; k < 8; ++k)
            {
              dst[0 * 8 + k] = sFx[k * NFF + fxl];
              dst[1 * 8 + k] = sFx[k * NFF + fxl + 1];
              dst[2 * 8 + k] = sFy[k * NFF + fyl];
              dst[3 * 8 + k] = sFy[k * NFF + fyl + B];
            }
          }
        }
      }

      // ---------------- phase 4: update of the owned cell (tid)
      bool deferred = false;
      if (a.m.defer_slot)
      {
        const int * dsl = sSlot + 4;
        deferred = (ci == 0 && dsl[0] >= 0) || (ci == B - 1 && dsl[1] >= 0) || (cj == 0 && dsl[2] >= 0) ||
                   (cj == B - 1 && dsl[3] >= 0);
      }
      DtT    m_inv = DtT(0);
      double u2[H::NV];
      if (!deferred)
      {
        if constexpr (MIXED)
          m_inv = update_mixed<B>(uown, u2, sFx, sFy, ci, cj, d2f_fast(dx), P, eosk, a.invdt != nullptr);
        else
          m_inv = update_fp64<B>(uown, u2, sFx, sFy, ci, cj, dx, P, a.invdt != nullptr);
        double * out = a.U2 + (size_t)n * H::NV * NC + tid;
        bool     finite = true;
#pragma unroll
        for (int v = 0; v < H::NV; ++v)
        {
          out[v * NC] = u2[v];
          finite = finite && finite_bits(u2[v]);
        }
        if (!finite)
          raise_status(a.status, STATUS_NONPHYSICAL);
      }
      else
      {
#pragma unroll
        for (int v = 0; v < H::NV; ++v)
          u2[v] = uown[v]; // the reflux pass finishes the cell (and its twin cells)
      }
      if (sSlot[9] > sSlot[8])
      {
        // the solver loop's boundary fill of the outside blocks mirroring this
        // block (FillOutside: the last applicable face's copy rule), from the
        // new state staged in the (now free) slope area
        double * sTw = reinterpret_cast<double *>(sRec);
#pragma unroll
        for (int v = 0; v < H::NV; ++v)
          sTw[v * NC + tid] = u2[v];
        __syncthreads();
        for (int t = sSlot[8]; t < sSlot[9]; ++t)
        {
          const int e = a.m.twin_list[t];
          const int o = e >> 3, face = e & 7, dir = face >> 1, bc = P.bc[face];
          const int edge = (face & 1) ? B - 1 : 0;
          const int sx = dir == 0 ? (bc == 2 ? edge : B - 1 - ci) : ci;
          const int sy = dir == 1 ? (bc == 2 ? edge : B - 1 - cj) : cj;
          const double * src = sTw + sx + B * sy;
          double *       dst = a.U2 + (size_t)o * H::NV * NC + tid;
#pragma unroll
          for (int v = 0; v < H::NV; ++v)
          {
            const double val = src[v * NC];
            dst[v * NC] = (bc == 3 && v == H::IU + dir) ? -val : val;
          }
        }
      }
      if (a.invdt)
      {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
          m_inv = fmax(m_inv, __shfl_xor_sync(0xffffffffu, m_inv, o));
        if ((tid & 31) == 0)
          sRed[tid >> 5] = m_inv;
        __syncthreads();
        if (tid == 0)
        {
          DtT mm = DtT(0);
          for (int w = 0; w < NT / 32; ++w)
            mm = fmax(mm, sRed[w]);
          atomic_max_pos(a.invdt + ins, (double)mm);
        }
      }
      if (counts)
      {
        __syncthreads(); // every output of the block is written
        if (tid >= 16 && tid < 21)
        {
          int ready = -1;
          if (fin_v >= 0)
          {
            __threadfence();
            if (atomicSub(a.m.fin_cnt + fin_v, 1u) == 1u)
            {
              __threadfence();
              ready = fin_v;
            }
          }
          sFin[tid - 16] = ready;
        }
        if (tid == 0)
          sFin[5] = 0;
      }
      next = sNext; // read before the barrier: the next block's claim overwrites it
      if (!counts)
      {
        __syncthreads();
        iw = next;
        continue;
      }
    }
    else
    {
      if (!fused)
        break;
      if (tid == 0)
      {
        // claim the next deferred block; the launch's last draw resets the ticket
        const unsigned d = atomicAdd(a.m.fin_ticket, 1u);
        int            ready = -1;
        if (d < (unsigned)a.m.n_fin)
        {
          __threadfence();
          if (atomicSub(a.m.fin_cnt + d, 1u) == 1u)
          {
            __threadfence();
            ready = (int)d;
          }
        }
        else if (d == (unsigned)a.m.n_fin + gridDim.x - 1u)
          *a.m.fin_ticket = 0u;
        sFin[0] = ready;
        sFin[1] = sFin[2] = sFin[3] = sFin[4] = -1;
        sFin[5] = d >= (unsigned)a.m.n_fin;
      }
    }
    if (fused)
    {
      __syncthreads();
      if constexpr (MIXED)
      {
#pragma unroll 1
        for (int t = 0; t < 5; ++t)
        {
          const int j = sFin[t];
          if (j >= 0)
          {
            finish_deferred_2d<B, NT>(a, j);
            if (tid == 0)
              a.m.fin_cnt[j] = a.m.fin_init[j];
          }
        }
      }
      if (iw >= nwalk && sFin[5])
        break;
    }
    __syncthreads();
    iw = next;
  }
}

// ---------------------------------------------------------------------------
// reflux: coarse cells next to finer faces (one thread per deferred record
// entry).  Replays update_U with the fine face sums of
// get_flux_from_fine_neighbor (ReadFluxesAndConservativeUpdateFunctor.h:256-307).
// ---------------------------------------------------------------------------
// The outside-block cells that copy the refluxed cell (ci, cj) of block n in
// the solver loop's boundary fill (the step kernel filled them from the
// pre-reflux state): ZERO_GRADIENT copies the boundary row into every layer,
// WALL mirrors one cell and negates the normal momentum.
template <int B>
__device__ __forceinline__ void
patch_twins_2d(const StepArgs & a, int n, int ci, int cj, const double * u2)
{
  using H = V<2>;
  constexpr int NC = B * B;
  const int     t0 = a.m.twin_first[n], t1 = a.m.twin_first[n + 1];
  for (int t = t0; t < t1; ++t)
  {
    const int e = a.m.twin_list[t];
    const int o = e >> 3, face = e & 7, dir = face >> 1, bc = a.p.bc[face];
    double *  base = a.U2 + (size_t)o * H::NV * NC;
    if (bc == 2)
    {
      if ((dir == 0 ? ci : cj) != ((face & 1) ? B - 1 : 0))
        continue;
      for (int k = 0; k < B; ++k)
      {
        const int c = dir == 0 ? k + B * cj : ci + B * k;
#pragma unroll
        for (int v = 0; v < H::NV; ++v)
          base[v * NC + c] = u2[v];
      }
    }
    else
    {
      const int c = dir == 0 ? (B - 1 - ci) + B * cj : ci + B * (B - 1 - cj);
#pragma unroll
      for (int v = 0; v < H::NV; ++v)
        base[v * NC + c] = v == H::IU + dir ? -u2[v] : u2[v];
    }
  }
}

// The same patches for one state variable (the value `val` of variable `var`
// of the cell), so that the lanes of a cell's group each write their own
template <int B>
__device__ __forceinline__ void
patch_twins_2d_var(const StepArgs & a, int n, int ci, int cj, int var, double val)
{
  using H = V<2>;
  constexpr int NC = B * B;
  const int     t0 = a.m.twin_first[n], t1 = a.m.twin_first[n + 1];
  for (int t = t0; t < t1; ++t)
  {
    const int e = a.m.twin_list[t];
    const int o = e >> 3, face = e & 7, dir = face >> 1, bc = a.p.bc[face];
    double *  base = a.U2 + ((size_t)o * H::NV + var) * NC;
    if (bc == 2)
    {
      if ((dir == 0 ? ci : cj) != ((face & 1) ? B - 1 : 0))
        continue;
      for (int k = 0; k < B; ++k)
        base[dir == 0 ? k + B * cj : ci + B * k] = val;
    }
    else
      base[dir == 0 ? (B - 1 - ci) + B * cj : ci + B * (B - 1 - cj)] = var == H::IU + dir ? -val : val;
  }
}

// MIXED selects the FP32-bulk form of the mixed mode (float-pair increments
// applied by apply_mixed_2d); the FP64 form replays the reference arithmetic.
// A thread of this pass is latency-bound, so its loads come in two waves: the
// record's DeferInfo row (slots, fine-face reflux slots, level, instance),
// then the cell's old state and all face fluxes it needs.
template <int B, bool MIXED>
__global__ void
reflux2d_kernel(StepArgs a)
{
  using H = V<2>;
  using D = DeferInfo<2>;
  constexpr int NC = B * B;
  const int     gid = blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= a.m.n_defer * B)
    return;
  const int   rec = gid / B, pos = gid % B;
  const int4 * row = reinterpret_cast<const int4 *>(a.m.defer_info + (size_t)rec * D::STRIDE);
  const int4  r0 = row[0], r1 = row[1], r2 = row[2], r3 = row[3];
  const int   code = r0.x;
  const int   dsl[4] = { r0.y, r0.z, r0.w, r1.x };
  const int   rsf[4][2] = { { r1.y, r1.z }, { r1.w, r2.x }, { r2.y, r2.z }, { r2.w, r3.x } };
  const int   n = code >> 3, face = code & 7;
  const int   ins = r3.z;
  if (a.inst_active && !a.inst_active[ins])
    return;
  const double dx = a.p.level_dx[r3.y];
  const int   dirf = face >> 1, sidef = face & 1;
  const int   ci = dirf == 0 ? (sidef ? B - 1 : 0) : pos;
  const int   cj = dirf == 0 ? pos : (sidef ? B - 1 : 0);
  const int   cell = ci + B * cj;
  // a cell next to two finer faces is handled by the lower face index
#pragma unroll
  for (int f2 = 0; f2 < 4; ++f2)
    if (f2 < face && dsl[f2] >= 0 && (f2 >> 1 == 0 ? ci : cj) == ((f2 & 1) ? B - 1 : 0))
      return;
  bool fine[4];
  int  rs[4];
#pragma unroll
  for (int f = 0; f < 4; ++f)
  {
    const int cd = (f >> 1) == 0 ? ci : cj, ct = (f >> 1) == 0 ? cj : ci;
    fine[f] = cd == ((f & 1) ? B - 1 : 0) && dsl[f] >= 0;
    rs[f] = fine[f] ? ((2 * ct) / B ? rsf[f][1] : rsf[f][0]) : -1;
    if (fine[f] && rs[f] < 0)
    {
      raise_status(a.status, STATUS_MESH);
      return;
    }
  }
  double uin[H::NV], u2[H::NV];
  {
    const double * ub = a.U + (size_t)n * H::NV * NC + cell;
#pragma unroll
    for (int v = 0; v < H::NV; ++v)
      u2[v] = uin[v] = ub[v * NC];
  }
  // second wave (with the state): the face fluxes, own faces from the
  // record, fine faces from the two fine faces' published fluxes (floats in
  // the mixed form, doubles in the FP64 form)
  // (rows of 8 fluxes start on 32-byte boundaries: 16-byte vector loads)
  using R = typename std::conditional<MIXED, float, double>::type;
  using R2 = typename std::conditional<MIXED, float4, double2>::type;
  constexpr int RV = sizeof(R2) / sizeof(R);
  const int dslf = face == 0 ? dsl[0] : face == 1 ? dsl[1] : face == 2 ? dsl[2] : dsl[3];
  const R * own = reinterpret_cast<const R *>(a.defer_buf) + ((size_t)dslf * B + pos) * 32;
  R         F0[4][8], F1[4][8];
#pragma unroll
  for (int f = 0; f < 4; ++f)
  {
    const int  ct = (f >> 1) == 0 ? cj : ci;
    const int  fl = 2 * ct - ((2 * ct) / B) * B;
    const R *  p0 = fine[f] ? reinterpret_cast<const R *>(a.reflux_buf) + ((size_t)rs[f] * B + fl) * 8 : own + f * 8;
    const R2 * q = reinterpret_cast<const R2 *>(p0);
#pragma unroll
    for (int k = 0; k < 8 / RV; ++k)
    {
      const R2 x = q[k];
      const R2 y = fine[f] ? q[8 / RV + k] : R2{};
      F0[f][RV * k] = x.x;
      F0[f][RV * k + 1] = x.y;
      F1[f][RV * k] = y.x;
      F1[f][RV * k + 1] = y.y;
      if constexpr (RV == 4)
      {
        F0[f][RV * k + 2] = x.z;
        F0[f][RV * k + 3] = x.w;
        F1[f][RV * k + 2] = y.z;
        F1[f][RV * k + 3] = y.w;
      }
    }
  }
  if constexpr (MIXED)
  {
    // FP32-bulk form: per-direction increments as float pairs (a fine face
    // side is the exact float-float sum of its two fine faces, / 4), applied
    // as in the step kernel
    const int  eosk = a.p.mg_any ? 2 : ((a.p.gpx[0] != 0.0 || a.p.gpx[1] != 0.0) ? 1 : 0);
    float      a0f = d2f_fast(uin[H::IA0]), a1f = d2f_fast(uin[H::IA1]);
    {
      float st0f, st1f;
      source_factors_mixed<2>(uin, a.p, eosk, st0f, st1f);
      a0f *= st0f;
      a1f *= st1f;
    }
    float     h[2][5], l[2][5], dA[2][2];
    const int ks[5] = { H::FR0, H::FR1, H::FE, H::FU, H::FV };
#pragma unroll
    for (int dir = 0; dir < 2; ++dir)
    {
      float Fh[2][8], Fl[2][8];
#pragma unroll
      for (int side = 0; side < 2; ++side)
      {
        const int f = 2 * dir + side;
#pragma unroll
        for (int k = 0; k < 8; ++k)
        {
          if (fine[f])
          {
            float sh, sl;
            two_sum(F0[f][k], F1[f][k], sh, sl);
            Fh[side][k] = 0.25f * sh;
            Fl[side][k] = 0.25f * sl;
          }
          else
          {
            Fh[side][k] = F0[f][k];
            Fl[side][k] = 0.0f;
          }
        }
      }
#pragma unroll
      for (int k = 0; k < 5; ++k)
      {
        float hh, ll;
        two_diff(Fh[0][ks[k]], Fh[1][ks[k]], hh, ll);
        h[dir][k] = hh;
        l[dir][k] = ll + (Fl[0][ks[k]] - Fl[1][ks[k]]);
      }
      const float usl = Fh[0][H::FUS] + Fl[0][H::FUS], usr = Fh[1][H::FUS] + Fl[1][H::FUS];
      dA[dir][0] = (((Fh[0][H::FA0] + Fl[0][H::FA0]) - usl * a0f) - (Fh[1][H::FA0] + Fl[1][H::FA0])) + usr * a0f;
      dA[dir][1] = (((Fh[0][H::FA1] + Fl[0][H::FA1]) - usl * a1f) - (Fh[1][H::FA1] + Fl[1][H::FA1])) + usr * a1f;
    }
    const float m_inv = apply_mixed_2d(uin, u2, h, l, dA, d2f_fast(dx), a.p, eosk, a.invdt != nullptr);
    double *    out = a.U2 + (size_t)n * H::NV * NC + cell;
    bool        finite = true;
#pragma unroll
    for (int v = 0; v < H::NV; ++v)
    {
      out[v * NC] = u2[v];
      finite = finite && finite_bits(u2[v]);
    }
    if (!finite)
      raise_status(a.status, STATUS_NONPHYSICAL);
    if (a.fill_twins)
      patch_twins_2d<B>(a, n, ci, cj, u2);
    if (a.invdt)
      atomic_max_pos_warp(a.invdt, ins, (double)m_inv);
  }
  else
  {
    // update_U with the fine face sums of get_flux_from_fine_neighbor
    // (ReadFluxesAndConservativeUpdateFunctor.h:256-307), X then Y
    const double a0n = uin[H::IA0], a1n = uin[H::IA1];
    double       st0, st1;
    source_factors_fp64<2>(uin, a.p, st0, st1);
#pragma unroll
    for (int dir = 0; dir < 2; ++dir)
    {
      double acc[7];
#pragma unroll
      for (int k = 0; k < 7; ++k)
        acc[k] = 0.0;
#pragma unroll
      for (int side = 0; side < 2; ++side)
      {
        const int f = 2 * dir + side;
        if (fine[f])
        {
          double fv[8];
#pragma unroll
          for (int k = 0; k < 8; ++k)
          {
            double sum = 0.0;
            sum += F0[f][k];
            sum += F1[f][k];
            fv[k] = sum;
          }
#pragma unroll
          for (int k = 0; k < 7; ++k)
            acc[k] = side == 0 ? acc[k] + fv[k] / 4.0 : acc[k] - fv[k] / 4.0;
          const double us = fv[7];
          if (side == 0)
          {
            acc[H::FA0] -= st0 * us * a0n / 4.0;
            acc[H::FA1] -= st1 * us * a1n / 4.0;
          }
          else
          {
            acc[H::FA0] += st0 * us * a0n / 4.0;
            acc[H::FA1] += st1 * us * a1n / 4.0;
          }
        }
        else
        {
#pragma unroll
          for (int k = 0; k < 7; ++k)
            acc[k] = side == 0 ? acc[k] + F0[f][k] : acc[k] - F0[f][k];
          const double us = F0[f][7];
          if (side == 0)
          {
            acc[H::FA0] -= st0 * us * a0n;
            acc[H::FA1] -= st1 * us * a1n;
          }
          else
          {
            acc[H::FA0] += st0 * us * a0n;
            acc[H::FA1] += st1 * us * a1n;
          }
        }
      }
      const double eps = 1e-12;
      u2[H::IAD0] += acc[H::FR0];
      if (u2[H::IAD0] < eps)
        u2[H::IAD0] = 0.0;
      u2[H::IAD1] += acc[H::FR1];
      if (u2[H::IAD1] < eps)
        u2[H::IAD1] = 0.0;
      u2[H::IA0] += acc[H::FA0];
      if (u2[H::IA0] < eps)
        u2[H::IA0] = 0.0;
      if (u2[H::IA0] > 1.0 - eps)
        u2[H::IA0] = 1.0;
      u2[H::IA1] += acc[H::FA1];
      if (u2[H::IA1] < eps)
        u2[H::IA1] = 0.0;
      if (u2[H::IA1] > 1.0 - eps)
        u2[H::IA1] = 1.0;
      u2[H::IE] += acc[H::FE];
      u2[H::IU] += acc[H::FU];
      u2[H::IV] += acc[H::FV];
    }
    const double sum_alpha = u2[H::IA0] + u2[H::IA1];
    const double sum_alpha_rho = u2[H::IAD0] + u2[H::IAD1];
    const double inv = 1.0 / sum_alpha;
    u2[H::IA0] *= inv;
    u2[H::IA1] *= inv;
    u2[H::ID] = sum_alpha_rho;
    double * out = a.U2 + (size_t)n * H::NV * NC + cell;
    bool     finite = true;
#pragma unroll
    for (int v = 0; v < H::NV; ++v)
    {
      out[v * NC] = u2[v];
      finite = finite && isfinite(u2[v]);
    }
    if (!finite)
      raise_status(a.status, STATUS_NONPHYSICAL);
    if (a.fill_twins)
      patch_twins_2d<B>(a, n, ci, cj, u2);
    if (a.invdt)
    {
      double       q[6];
      const double c = prim_fp64<2>(u2, q, a.p);
      atomic_max_pos_warp(a.invdt, ins, (c + fabs(q[V<2>::QU])) / dx + (c + fabs(q[V<2>::QV])) / dx);
    }
  }
}

// ---------------------------------------------------------------------------
// The FP32-bulk reflux pass with 8 lanes per deferred cell.  One thread per
// cell ran a serial chain of about a thousand instructions with one warp per
// SM (latency-bound at ~8 us on the shock-bubble); here lane k of a cell's
// group of 8 handles face-flux component k (r0 r1 a0 a1 e u v u*) and the
// state variable it updates (IAD0 IAD1 IA0 IA1 IE IU IV ID), and the lanes
// exchange what couples them (u* for the volume-fraction source term, the two
// volume fractions for the renormalisation, the partial densities for ID, the
// new state for the CFL rate) by shuffles; each lane writes its variable to
// the cell and to the cell's outside twins.  Every value is computed with the
// arithmetic of apply_mixed_2d in the same order, so the pass gives the same
// bits as the one-thread form.  All lanes of a warp reach every shuffle:
// inactive cells (past the end, skipped, or of a stopped instance) compute on
// zeros and write nothing.
// ---------------------------------------------------------------------------
// cell `pos` of record `rec` on the 8 lanes of the calling thread's group
// (lane k = threadIdx.x % 8); every lane of the warp calls it.  The face
// fluxes are read past L1 (ld.global.cg): in the step kernel's tail other CTAs
// of the same launch wrote them.
template <int B>
__device__ __forceinline__ void
reflux2d_lanes(const StepArgs & a, int rec, int pos, bool act)
{
  using H = V<2>;
  using D = DeferInfo<2>;
  constexpr int NC = B * B;
  const int     k = (int)(threadIdx.x & 7u);       // flux component of this lane
  const int     gb = (int)(threadIdx.x & 31u) & ~7; // first lane of the cell's group
  int4          r0 = make_int4(0, -1, -1, -1), r1 = make_int4(-1, -1, -1, -1), r2 = make_int4(-1, -1, -1, -1), r3 = make_int4(-1, 0, 0, 0);
  if (act)
  {
    const int4 * row = reinterpret_cast<const int4 *>(a.m.defer_info + (size_t)rec * D::STRIDE);
    r0 = row[0];
    r1 = row[1];
    r2 = row[2];
    r3 = row[3];
  }
  const int code = r0.x;
  const int dsl[4] = { r0.y, r0.z, r0.w, r1.x };
  const int rsf[4][2] = { { r1.y, r1.z }, { r1.w, r2.x }, { r2.y, r2.z }, { r2.w, r3.x } };
  const int n = code >> 3, face = code & 7;
  const int ins = act ? r3.z : 0;
  if (act && a.inst_active && !a.inst_active[ins])
    act = false;
  const int dirf = face >> 1, sidef = face & 1;
  const int ci = dirf == 0 ? (sidef ? B - 1 : 0) : pos;
  const int cj = dirf == 0 ? pos : (sidef ? B - 1 : 0);
  const int cell = ci + B * cj;
  // a cell next to two finer faces is handled by the lower face index
#pragma unroll
  for (int f2 = 0; f2 < 4; ++f2)
    if (f2 < face && dsl[f2] >= 0 && (f2 >> 1 == 0 ? ci : cj) == ((f2 & 1) ? B - 1 : 0))
      act = false;
  bool fine[4];
  int  rs[4];
#pragma unroll
  for (int f = 0; f < 4; ++f)
  {
    const int cd = (f >> 1) == 0 ? ci : cj, ct = (f >> 1) == 0 ? cj : ci;
    fine[f] = cd == ((f & 1) ? B - 1 : 0) && dsl[f] >= 0;
    rs[f] = fine[f] ? ((2 * ct) / B ? rsf[f][1] : rsf[f][0]) : -1;
    if (act && fine[f] && rs[f] < 0)
    {
      if (k == 0)
        raise_status(a.status, STATUS_MESH);
      act = false;
    }
  }
  // the state variable this lane updates (flux component k -> variable)
  // (component k -> variable: r0 IAD0, r1 IAD1, a0 IA0, a1 IA1, e IE, u IU,
  // v IV, u* ID, packed as nibbles)
  static_assert(H::FR0 == 0 && H::FR1 == 1 && H::FA0 == 2 && H::FA1 == 3 && H::FE == 4 && H::FU == 5 && H::FV == 6 && H::FUS == 7, "2D face record order");
  static_assert(H::ID == 0 && H::IE == 1 && H::IU == 2 && H::IV == 3 && H::IA0 == 4 && H::IAD0 == 5 && H::IA1 == 6 && H::IAD1 == 7, "2D variable order");
  const int     var = (int)((0x03216475u >> (4 * k)) & 15u);
  constexpr int lane_of[8] = { 7, 4, 5, 6, 2, 0, 3, 1 }; // variable -> lane (inverse of the map above)
  const double  u_own = act ? a.U[((size_t)n * H::NV + var) * NC + cell] : 0.0;
  // component k of the face fluxes: own faces from the record, fine faces
  // from the two fine faces' published fluxes
  const int     dslf = face == 0 ? dsl[0] : face == 1 ? dsl[1] : face == 2 ? dsl[2] : dsl[3];
  float         F0[4], F1[4];
#pragma unroll
  for (int f = 0; f < 4; ++f)
  {
    F0[f] = 0.0f;
    F1[f] = 0.0f;
    if (act)
    {
      const int ct = (f >> 1) == 0 ? cj : ci;
      const int fl = 2 * ct - ((2 * ct) / B) * B;
      if (fine[f])
      {
        const float * p0 = reinterpret_cast<const float *>(a.reflux_buf) + ((size_t)rs[f] * B + fl) * 8;
        F0[f] = __ldcg(p0 + k);
        F1[f] = __ldcg(p0 + 8 + k);
      }
      else
        F0[f] = __ldcg(reinterpret_cast<const float *>(a.defer_buf) + ((size_t)dslf * B + pos) * 32 + f * 8 + k);
    }
  }
  // the whole old state in every lane of the group
  double uin[H::NV];
#pragma unroll
  for (int v = 0; v < H::NV; ++v)
    uin[v] = __shfl_sync(0xffffffffu, u_own, gb + lane_of[v]);
  const int  eosk = a.p.mg_any ? 2 : ((a.p.gpx[0] != 0.0 || a.p.gpx[1] != 0.0) ? 1 : 0);
  float      a0f = d2f_fast(uin[H::IA0]), a1f = d2f_fast(uin[H::IA1]);
  {
    float st0f, st1f;
    source_factors_mixed<2>(uin, a.p, eosk, st0f, st1f);
    a0f *= st0f;
    a1f *= st1f;
  }
  // per direction: this component's side values (a fine side is the exact
  // float-float sum of its two fine faces, / 4)
  float Fh[2][2], Fl[2][2];
#pragma unroll
  for (int dir = 0; dir < 2; ++dir)
#pragma unroll
    for (int side = 0; side < 2; ++side)
    {
      const int f = 2 * dir + side;
      if (fine[f])
      {
        float sh, sl;
        two_sum(F0[f], F1[f], sh, sl);
        Fh[dir][side] = 0.25f * sh;
        Fl[dir][side] = 0.25f * sl;
      }
      else
      {
        Fh[dir][side] = F0[f];
        Fl[dir][side] = 0.0f;
      }
    }
  // u* of both sides (lane FUS) for the volume-fraction source term
  float usl[2], usr[2];
#pragma unroll
  for (int dir = 0; dir < 2; ++dir)
  {
    usl[dir] = __shfl_sync(0xffffffffu, Fh[dir][0] + Fl[dir][0], gb + H::FUS);
    usr[dir] = __shfl_sync(0xffffffffu, Fh[dir][1] + Fl[dir][1], gb + H::FUS);
  }
  const double eps = 1e-12, one_m_eps = 1.0 - 1e-12;
  double       u2v = u_own;
  if (k == H::FR0 || k == H::FR1 || k == H::FE || k == H::FU || k == H::FV)
  {
    float h[2], l[2];
#pragma unroll
    for (int dir = 0; dir < 2; ++dir)
    {
      float hh, ll;
      two_diff(Fh[dir][0], Fh[dir][1], hh, ll);
      h[dir] = hh;
      l[dir] = ll + (Fl[dir][0] - Fl[dir][1]);
    }
    const bool  clamp = k == H::FR0 || k == H::FR1;
    const float uf = d2f_fast(u2v);
    if (!clamp || uf > 2.0f * fabsf(h[0]) + 2e-12f)
    {
      float s, t;
      two_sum(h[0], h[1], s, t);
      two_sum(s, t + (l[0] + l[1]), s, t);
      u2v += ff_to_d(s, t);
      if (clamp && dlt_pos(u2v, eps))
        u2v = 0.0;
    }
    else
    {
#pragma unroll
      for (int dir = 0; dir < 2; ++dir)
      {
        u2v = (u2v + f2d_exact(h[dir])) + f2d_exact(l[dir]);
        if (dlt_pos(u2v, eps))
          u2v = 0.0;
      }
    }
  }
  else if (k == H::FA0 || k == H::FA1)
  {
    const float af_src = k == H::FA0 ? a0f : a1f;
    float       dA[2];
#pragma unroll
    for (int dir = 0; dir < 2; ++dir)
      dA[dir] = (((Fh[dir][0] + Fl[dir][0]) - usl[dir] * af_src) - (Fh[dir][1] + Fl[dir][1])) + usr[dir] * af_src;
    const float af = d2f_fast(u_own); // the lane's own variable, IA0 or IA1
    const float m = 2.0f * fabsf(dA[0]) + 2e-12f;
    if (af > m && af + m < 1.0f)
    {
      u2v += f2d_exact(dA[0] + dA[1]);
      if (dlt_pos(u2v, eps))
        u2v = 0.0;
      if (dgt_pos(u2v, one_m_eps))
        u2v = 1.0;
    }
    else
    {
#pragma unroll
      for (int dir = 0; dir < 2; ++dir)
      {
        u2v += f2d_exact(dA[dir]);
        if (dlt_pos(u2v, eps))
          u2v = 0.0;
        if (dgt_pos(u2v, one_m_eps))
          u2v = 1.0;
      }
    }
  }
  // renormalisation of the volume fractions (lanes FA0 and FA1)
  {
    const double a0n = __shfl_sync(0xffffffffu, u2v, gb + H::FA0);
    const double a1n = __shfl_sync(0xffffffffu, u2v, gb + H::FA1);
    const double sa = a0n + a1n;
    const double d = sa - 1.0;
    if ((k == H::FA0 || k == H::FA1) && d != 0.0)
    {
      if ((__double_as_longlong(d) & 0x7FFFFFFFFFFFFFFFLL) < __double_as_longlong(1e-8))
        u2v = fma(-u2v, d, u2v);
      else
        u2v *= 1.0 / sa;
    }
  }
  // ID = IAD0 + IAD1 (lane FUS)
  {
    const double r0n = __shfl_sync(0xffffffffu, u2v, gb + H::FR0);
    const double r1n = __shfl_sync(0xffffffffu, u2v, gb + H::FR1);
    if (k == H::FUS)
      u2v = r0n + r1n;
  }
  // the new state in every lane: CFL rate of the cell
  double u2[H::NV];
#pragma unroll
  for (int v = 0; v < H::NV; ++v)
    u2[v] = __shfl_sync(0xffffffffu, u2v, gb + lane_of[v]);
  if (act)
  {
    a.U2[((size_t)n * H::NV + var) * NC + cell] = u2v;
    if (!finite_bits(u2v))
      raise_status(a.status, STATUS_NONPHYSICAL);
    if (a.fill_twins)
      patch_twins_2d_var<B>(a, n, ci, cj, var, u2v);
  }
  if (a.invdt)
  {
    float m_inv = 0.0f;
    if (act && k == 0)
    {
      float       df, ux, uy, uz, a0;
      const float p = pressure_mixed<2>(u2, a.p, eosk, df, ux, uy, uz, a0);
      const float a0s = fmaxf(0.0f, fminf(1.0f, a0));
      const float c = sound_speed_eos(a.p, eosk, df, p, a0s, d2f_fast(u2[H::IAD0]), d2f_fast(u2[H::IAD1]));
      m_inv = ((c + fabsf(ux)) + (c + fabsf(uy))) * __frcp_rn(d2f_fast(a.p.level_dx[r3.y]));
    }
    atomic_max_pos_warp(a.invdt, ins, (double)m_inv);
  }
}

template <int B>
__global__ void __launch_bounds__(128)
reflux2d_mixed_lanes_kernel(StepArgs a)
{
  const int  cslot = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 3);
  const bool act = cslot < a.m.n_defer * B;
  reflux2d_lanes<B>(a, act ? cslot / B : 0, cslot % B, act);
}

} // namespace g5
