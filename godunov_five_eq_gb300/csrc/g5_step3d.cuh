// g5_step3d.cuh — fused 3D block timestep (one CTA of 512 threads per 8^3
// block, persistent over the block list).
//
// Shared memory holds the 12^3 ghosted primitives, the Hancock half-step
// source of the 10^3 ring, and the face fluxes of ONE direction (the THINC
// normal is evaluated on demand, at interface cells only).  The update runs direction by direction (X, Y, Z: the
// reference's order, GodunovImplemV0.cpp:121-139, with update_U's clamps after
// each direction), the running state of each owned cell in registers.
// Cells next to a finer face are deferred to reflux3d_kernel; fine blocks
// next to a coarser face publish their face fluxes for it.
#pragma once

#include <type_traits>

#include "g5_common.cuh"

namespace g5
{

template <bool MIXED>
struct Step3DTraits
{
  using R = typename std::conditional<MIXED, float, double>::type;
  static constexpr int B = 8;
  static constexpr int NT = 512;
  static constexpr int G = B + 4, GG = G * G, GGG = G * G * G; // ghosted extent
  static constexpr int S = B + 2, SS = S * S, SSS = S * S * S; // ring extent
  static constexpr int NQ = 7;                                  // r0 r1 p u v w a0
  static constexpr int NHS = 6;                                 // Hancock source r0 r1 p u v w
  static constexpr int NFF = (B + 1) * B * B;                   // faces of one direction
  static constexpr int NF = 9;                                  // r0 r1 a0 a1 e u v w ustar
  // face-flux buffers: the FP32-bulk form computes the X and Y faces in one
  // pass (1,152 faces over 512 threads: 3 rounds instead of 2 + 2), Z alone
  static constexpr int NBUF = MIXED ? 2 : 1;
  static constexpr size_t smem_bytes = sizeof(R) * (size_t)(NQ * GGG + NHS * SSS + NBUF * NF * NFF) + 64;
};

__device__ __forceinline__ bool
neg_zero(double x)
{
  return __double_as_longlong(x) == (long long)0x8000000000000000ULL;
}
__device__ __forceinline__ bool
neg_zero(float x)
{
  return __float_as_uint(x) == 0x80000000u;
}

// The halo cells of an 8^3 block that the step reads, as ghosted offsets
// (-2 .. 9); the other 128 cells of the 12^3 ghosted cube (two coordinates
// two cells out) are never read.  h < HALO3_FULL: cells whose primitive state
// the slopes read: the two layers beyond each face (z faces, then y, then x;
// x fastest, the x layers as pairs of adjacent cells, so that a warp reads
// contiguous runs of a neighbour), then the 96 cells along the block's edges
// (one cell out in two coordinates).  HALO3_FULL <= h < HALO3_FULL +
// HALO3_ALPHA (THINC only): cells whose volume fraction only the Youngs
// normal of a face-neighbour cell reads: two coordinates out (one by two
// cells), then three coordinates out (at most one by two cells).
constexpr int HALO3_FULL = 864, HALO3_ALPHA = 224;

__device__ __forceinline__ void
halo_coords_3d(int h, int * g)
{
  if (h < 768)
  {
    if (h < 256)
    {
      const int zi = h >> 6;
      g[2] = zi < 2 ? zi - 2 : zi + 6;
      g[1] = (h >> 3) & 7;
      g[0] = h & 7;
    }
    else if (h < 512)
    {
      const int i = h - 256, yi = i >> 6;
      g[2] = (i >> 3) & 7;
      g[1] = yi < 2 ? yi - 2 : yi + 6;
      g[0] = i & 7;
    }
    else
    {
      const int i = h - 512, xs = i & 3;
      g[2] = i >> 5;
      g[1] = (i >> 2) & 7;
      g[0] = xs < 2 ? xs - 2 : xs + 6;
    }
    return;
  }
  if (h < HALO3_FULL + 192)
  {
    // 12 lines along axis A (line >> 2) at one cell (h < HALO3_FULL) or at
    // one and two cells (in either order) out in the two other axes
    // (selects, not g[A] = ...: a run-time index would put g in local memory)
    const bool full = h < HALO3_FULL;
    const int  i = full ? h - 768 : h - HALO3_FULL;
    const int  line = full ? i >> 3 : i >> 4;
    const int  A = line >> 2;
    const int  e1 = full ? 1 : (((i >> 3) & 1) ? 1 : 2), e2 = full ? 1 : 3 - e1;
    const int  vA = i & 7, v1 = (line & 1) ? 7 + e1 : -e1, v2 = (line & 2) ? 7 + e2 : -e2;
    // the first other axis is 1 for A = 0, else 0; the second is 1 for A = 2, else 2
    g[0] = A == 0 ? vA : v1;
    g[1] = A == 1 ? vA : (A == 0 ? v1 : v2);
    g[2] = A == 2 ? vA : v2;
    return;
  }
  // 8 corners x (all one cell out, or one axis two cells out)
  const int j = h - (HALO3_FULL + 192), corner = j >> 2, combo = j & 3;
#pragma unroll
  for (int k = 0; k < 3; ++k)
  {
    const int e = combo == k + 1 ? 2 : 1;
    g[k] = ((corner >> k) & 1) ? 7 + e : -e;
  }
}

// HLLC flux of face f of direction DIR (normal velocity swapped into u and
// back), scaled by dt/dx into the face buffer sFd ([9][NFF])
template <bool MIXED, int DIR, int THINC, bool MG = false>
__device__ __forceinline__ void face_flux3(const typename Step3DTraits<MIXED>::R * sQ, const typename Step3DTraits<MIXED>::R * sHS,
                                           int f, typename Step3DTraits<MIXED>::R * sFd, typename Step3DTraits<MIXED>::R dtdx_r,
                                           const PhysParams & P);

// conservative state seen by ghost cell g of block n (3D); false on a bad
// index.  ALPHA_ONLY: u[IA0] only (the same loads and sums for that variable)
template <bool ALPHA_ONLY = false>
__device__ __forceinline__ bool
gather_ghost_3d(const StepArgs & a, int n, const int * c0, const int * g, double * u)
{
  using H = V<3>;
  constexpr int B = 8, NC = 512;
  int           d[3], v[3];
#pragma unroll
  for (int e = 0; e < 3; ++e)
  {
    d[e] = g[e] < 0 ? -1 : (g[e] >= B ? 1 : 0);
    v[e] = g[e] - d[e] * B;
  }
  const int   s = (d[0] + 1) + 3 * (d[1] + 1) + 9 * (d[2] + 1);
  // relation and the 8 neighbour entries in one wave (two 16-byte loads)
  const int   rel = a.m.nbr_rel[n * 27 + s];
  const int4  nb_lo = *reinterpret_cast<const int4 *>(a.m.nbr + (n * 27 + s) * 8);
  const int4  nb_hi = *reinterpret_cast<const int4 *>(a.m.nbr + (n * 27 + s) * 8 + 4);
  const int   nb[8] = { nb_lo.x, nb_lo.y, nb_lo.z, nb_lo.w, nb_hi.x, nb_hi.y, nb_hi.z, nb_hi.w };
  if (rel < 0 && a.m.pg)
  {
    // prolonged by the pre-pass (minmod extrapolation or conservative interpolation)
    constexpr int G = B + 4, GGG = G * G * G;
    const int     ps = a.m.pg_slot[n];
    if (ps < 0)
      return false;
    const double * base = a.m.pg + (size_t)ps * H::NV * GGG + (g[0] + 2) + G * ((g[1] + 2) + G * (g[2] + 2));
#pragma unroll
    for (int k = 0; k < H::NV; ++k)
      if (!ALPHA_ONLY || k == H::IA0)
        u[k] = base[k * GGG];
    return true;
  }
  if (rel <= 0)
  {
    const int src = nb[0];
    if (src < 0 || src >= a.m.n_total)
      return false;
    int c[3];
#pragma unroll
    for (int e = 0; e < 3; ++e)
      c[e] = rel == 0 ? v[e] : ((c0[e] + d[e]) & 1) * (B / 2) + (v[e] >> 1);
    const double * base = a.U + (size_t)src * H::NV * NC + c[0] + B * (c[1] + B * c[2]);
#pragma unroll
    for (int k = 0; k < H::NV; ++k)
      if (!ALPHA_ONLY || k == H::IA0)
        u[k] = base[k * NC];
    return true;
  }
  int ch[3], f0[3];
#pragma unroll
  for (int e = 0; e < 3; ++e)
  {
    const int f = 2 * v[e];
    ch[e] = f / B;
    f0[e] = f - ch[e] * B;
  }
  const int src = nb[ch[0] + 2 * ch[1] + 4 * ch[2]];
  if (src < 0 || src >= a.m.n_total)
    return false;
  const double * base = a.U + (size_t)src * H::NV * NC + f0[0] + B * (f0[1] + B * f0[2]);
  const int      vars[7] = { H::IE, H::IU, H::IV, H::IW, H::IAD0, H::IAD1, H::IA0 };
  // f0[0] is even: each pair of fine cells in x is one 16-byte load
#pragma unroll
  for (int t = 0; t < 7; ++t)
  {
    if (ALPHA_ONLY && vars[t] != H::IA0)
      continue;
    const double * p = base + vars[t] * NC;
    double         sum = 0.0;
#pragma unroll
    for (int oz = 0; oz < 2; ++oz)
#pragma unroll
      for (int oy = 0; oy < 2; ++oy)
      {
        const double2 r = *reinterpret_cast<const double2 *>(p + B * (oy + B * oz));
        sum += r.x;
        sum += r.y;
      }
    u[vars[t]] = sum / 8.0;
  }
  if (!ALPHA_ONLY)
  {
    u[H::IA1] = 1.0 - u[H::IA0];
    u[H::ID] = u[H::IAD0] + u[H::IAD1];
  }
  return true;
}

// the volume-fraction primitive of store_prim3 (prim_mixed / prim_fp64) from
// the conservative volume fraction alone
template <bool MIXED>
__device__ __forceinline__ typename Step3DTraits<MIXED>::R
alpha_prim(double ia0)
{
  if constexpr (MIXED)
  {
    float a0 = fmaxf(0.0f, fminf(1.0f, d2f_nan(ia0)));
    if (a0 < 1e-12f)
      a0 = 0.0f;
    if (a0 > 1.0f - 1e-12f)
      a0 = 1.0f;
    return a0;
  }
  else
  {
    double a0 = fmax(0.0, fmin(1.0, ia0));
    if (a0 < 1e-12)
      a0 = 0.0;
    if (a0 > 1.0 - 1e-12)
      a0 = 1.0;
    return a0;
  }
}

template <bool MIXED>
__device__ __forceinline__ void
store_prim3(typename Step3DTraits<MIXED>::R * sQ, int gidx, const double * u, const PhysParams & P, int eosk)
{
  constexpr int GGG = Step3DTraits<MIXED>::GGG;
  if constexpr (MIXED)
  {
    float q[7];
    prim_mixed<3>(u, q, P, eosk);
#pragma unroll
    for (int k = 0; k < 7; ++k)
      sQ[k * GGG + gidx] = q[k];
  }
  else
  {
    double q[7];
    prim_fp64<3>(u, q, P);
#pragma unroll
    for (int k = 0; k < 7; ++k)
      sQ[k * GGG + gidx] = q[k];
  }
}

// limited slope of component k at ghosted index gi along the stride o
template <typename R>
__device__ __forceinline__ R
slope_at(const R * Qk, int gi, int o, R st)
{
  return slope_scalar<R>(Qk[gi], Qk[gi + o], Qk[gi - o], st);
}

// reconstructed state of cell (ci,cj,ck) at its face in direction dir
// (side +1: right face, side -1: left face); q[7] = r0 r1 p u v w a0
// |n_dir| of the Youngs normal of the alpha field at ghosted index gi
// ((1,2,1) x (1,2,1) weighted central differences, unit cell, n = -grad/|grad|),
// evaluated where THINC needs it (interface cells only)
template <typename R, int G, int GG>
__device__ __forceinline__ R
youngs_abs_3d(const R * A, int gi, int dir)
{
  const R w[3] = { R(1), R(2), R(1) };
  R       g0 = R(0), g1 = R(0), g2 = R(0);
  for (int cc = -1; cc <= 1; ++cc)
    for (int bb = -1; bb <= 1; ++bb)
    {
      const R ww = w[bb + 1] * w[cc + 1];
      g0 += ww * (A[gi + 1 + G * bb + GG * cc] - A[gi - 1 + G * bb + GG * cc]);
      g1 += ww * (A[gi + bb + G + GG * cc] - A[gi + bb - G + GG * cc]);
      g2 += ww * (A[gi + bb + G * cc + GG] - A[gi + bb + G * cc - GG]);
    }
  R nrm = g0 * g0 + g1 * g1;
  nrm += g2 * g2;
  nrm = sqrt(nrm);
  const R gd = dir == 0 ? g0 : (dir == 1 ? g1 : g2);
  return (nrm > R(0)) ? fabs(-gd / nrm) : R(0);
}

template <bool MIXED, int THINC = -1>
__device__ __forceinline__ void
face_state3(const typename Step3DTraits<MIXED>::R * sQ,
            const typename Step3DTraits<MIXED>::R * sHS,
            int                                     ci,
            int                                     cj,
            int                                     ck,
            int                                     dir,
            int                                     side,
            const PhysParams &                      P,
            typename Step3DTraits<MIXED>::R *       q)
{
  using T = Step3DTraits<MIXED>;
  using R = typename T::R;
  constexpr int G = T::G, GG = T::GG, GGG = T::GGG, S = T::S, SS = T::SS, SSS = T::SSS;
  const int     gi = (ci + 2) + G * (cj + 2) + GG * (ck + 2);
  const int     si = (ci + 1) + S * (cj + 1) + SS * (ck + 1);
  const int     strides[3] = { 1, G, GG };
  const int     o = strides[dir];
  R             st, smallr, thinc_eps, thinc_beta;
  if constexpr (MIXED)
  {
    st = P.f_slope_type;
    smallr = P.f_smallr;
    thinc_eps = P.f_thinc_eps;
    thinc_beta = P.f_thinc_beta;
  }
  else
  {
    st = P.slope_type;
    smallr = P.smallr;
    thinc_eps = P.thinc_eps;
    thinc_beta = P.thinc_beta;
  }
  const bool hancock = P.integrator == 0;
  const R    off = R(0.5) * R(side);
  if constexpr (MIXED)
  {
    // two components per packed slope evaluation
#pragma unroll
    for (int k = 0; k < 6; k += 2)
    {
      const R *    Q0 = sQ + k * GGG;
      const R *    Q1 = Q0 + GGG;
      const float2 qc = make_float2(Q0[gi], Q1[gi]);
      const float2 dq = slope_pair(qc, make_float2(Q0[gi + o], Q1[gi + o]), make_float2(Q0[gi - o], Q1[gi - o]), st);
      q[k] = qc.x + off * dq.x;
      q[k + 1] = qc.y + off * dq.y;
      if (hancock)
      {
        q[k] += sHS[k * SSS + si];
        q[k + 1] += sHS[(k + 1) * SSS + si];
      }
    }
  }
  else
  {
#pragma unroll
    for (int k = 0; k < 6; ++k)
    {
      const R * Qk = sQ + k * GGG;
      const R   qc = Qk[gi];
      const R   dq = slope_at<R>(Qk, gi, o, st);
      R         t = qc + off * dq;
      // the reference adds the zero-offset terms of the other directions,
      // ((q + o_x dq_x) + o_y dq_y) + o_z dq_z; they can only change the sign
      // of a zero, so they are evaluated only when a negative zero occurs
      if (neg_zero(qc) || neg_zero(t))
      {
        R dd[3];
#pragma unroll
        for (int e = 0; e < 3; ++e)
          dd[e] = slope_at<R>(Qk, gi, strides[e], st);
        const R o0 = dir == 0 ? off : R(0), o1 = dir == 1 ? off : R(0), o2 = dir == 2 ? off : R(0);
        t = qc + o0 * dd[0] + o1 * dd[1] + o2 * dd[2];
      }
      q[k] = t;
      if (hancock)
        q[k] += sHS[k * SSS + si];
    }
  }
  const R a0 = sQ[6 * GGG + gi];
  q[6] = a0;
  if (THINC < 0 ? P.thinc != 0 : THINC == 1)
  {
    const R *  A = sQ + 6 * GGG;
    const R    aP = A[gi + o], aM = A[gi - o];
    const R    mono = (aP - a0) * (a0 - aM);
    const bool req = (a0 > thinc_eps) && (a0 < R(1) - thinc_eps) && mono > R(0);
    if (req)
    {
      const R nd = youngs_abs_3d<R, G, GG>(A, gi, dir);
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
      const R r0 = sQ[0 * GGG + gi], r1 = sQ[1 * GGG + gi];
      R       q0 = r0 + r0 / a0 * (af - a0);
      R       q1 = r1 + r1 / (R(1) - a0) * (a0 - af);
      if (hancock)
      {
        q0 += sHS[0 * SSS + si];
        q1 += sHS[1 * SSS + si];
      }
      q[0] = q0;
      q[1] = q1;
      q[6] = af;
    }
  }
  else
  {
    q[0] = fmax(smallr, q[0]);
    q[1] = fmax(smallr, q[1]);
  }
}

template <bool MIXED, int DIR, int THINC, bool MG>
__device__ __forceinline__ void
face_flux3(const typename Step3DTraits<MIXED>::R * sQ, const typename Step3DTraits<MIXED>::R * sHS, int f,
           typename Step3DTraits<MIXED>::R * sFd, typename Step3DTraits<MIXED>::R dtdx_r, const PhysParams & P)
{
  using T = Step3DTraits<MIXED>;
  using R = typename T::R;
  using H = V<3>;
  constexpr int B = T::B, NFF = T::NFF;
  int           fi, fj, fk;
  if (DIR == 0)
  {
    fi = f % (B + 1);
    fj = (f / (B + 1)) % B;
    fk = f / ((B + 1) * B);
  }
  else if (DIR == 1)
  {
    fi = f % B;
    fj = (f / B) % (B + 1);
    fk = f / (B * (B + 1));
  }
  else
  {
    fi = f % B;
    fj = (f / B) % B;
    fk = f / (B * B);
  }
  R qL[7], qR[7], fl[9];
  face_state3<MIXED, THINC>(sQ, sHS, fi - (DIR == 0), fj - (DIR == 1), fk - (DIR == 2), DIR, +1, P, qL);
  face_state3<MIXED, THINC>(sQ, sHS, fi, fj, fk, DIR, -1, P, qR);
  if (DIR > 0)
  {
    constexpr int iw = DIR == 1 ? 4 : 5; // component swapped with u
    R             t = qL[3];
    qL[3] = qL[iw];
    qL[iw] = t;
    t = qR[3];
    qR[3] = qR[iw];
    qR[iw] = t;
  }
  if constexpr (MIXED)
    hllc_fp32<3>(qL, qR, P.f_xi[0], P.f_xi[1], P.f_gpx[0], P.f_gpx[1], P.f_smallr, P.f_smallp, P.f_smallc, fl, MG ? &P : nullptr);
  else
    hllc_fp64<3>(qL, qR, P, fl);
  if (DIR > 0)
  {
    constexpr int fw = DIR == 1 ? H::FV : H::FW;
    const R       t = fl[H::FU];
    fl[H::FU] = fl[fw];
    fl[fw] = t;
  }
#pragma unroll
  for (int k = 0; k < 9; ++k)
    sFd[k * NFF + f] = fl[k] * dtdx_r;
}

// one direction of update_U (FP64, reference order); returns nothing, u2 updated
__device__ __forceinline__ void
apply_dir_fp64(double * u2, const double * acc)
{
  using H = V<3>;
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
  u2[H::IW] += acc[H::FW];
}

// The FP32-bulk form's update of a cell's state u2 (old state on entry) from
// its per-direction increments: hh + ll (exact float pairs) of the partial
// densities, dA (source term included) of the volume fractions, the running
// float-float sums es + et of energy and momentum, and the old volume
// fractions af0, af1 as floats.  The partial densities and volume fractions
// take the three directions combined when no per-direction clamp can trigger
// (FP32 test with margin), otherwise direction by direction; then the
// renormalisation and ID = IAD0 + IAD1.
__device__ __forceinline__ void
apply_mixed_3d(double * u2, const float (&hh)[3][2], const float (&ll)[3][2], const float (&dA)[3][2], const float (&es)[4],
               const float (&et)[4], float af0, float af1)
{
  using H = V<3>;
  const double eps = 1e-12, one_m_eps = 1.0 - 1e-12;
#pragma unroll
  for (int k = 0; k < 2; ++k)
  {
    const int   iv = k == 0 ? H::IAD0 : H::IAD1;
    const float uf = d2f_fast(u2[iv]);
    if (uf > 2.0f * (fabsf(hh[0][k]) + fabsf(hh[1][k])) + 2e-12f)
    {
      float s, t, s2, t2;
      two_sum(hh[0][k], hh[1][k], s, t);
      two_sum(s, hh[2][k], s2, t2);
      two_sum(s2, t2 + (t + ll[0][k] + ll[1][k] + ll[2][k]), s2, t2);
      u2[iv] += ff_to_d(s2, t2);
      if (dlt_pos(u2[iv], eps))
        u2[iv] = 0.0;
    }
    else
    {
#pragma unroll
      for (int d = 0; d < 3; ++d)
      {
        u2[iv] = (u2[iv] + f2d_exact(hh[d][k])) + f2d_exact(ll[d][k]);
        if (dlt_pos(u2[iv], eps))
          u2[iv] = 0.0;
      }
    }
  }
#pragma unroll
  for (int k = 0; k < 2; ++k)
  {
    const int   iv = k == 0 ? H::IA0 : H::IA1;
    const float af = k == 0 ? af0 : af1;
    const float m = 2.0f * (fabsf(dA[0][k]) + fabsf(dA[1][k])) + 2e-12f;
    if (af > m && af + m < 1.0f)
    {
      u2[iv] += f2d_exact((dA[0][k] + dA[1][k]) + dA[2][k]);
      if (dlt_pos(u2[iv], eps))
        u2[iv] = 0.0;
      if (dgt_pos(u2[iv], one_m_eps))
        u2[iv] = 1.0;
    }
    else
    {
#pragma unroll
      for (int d = 0; d < 3; ++d)
      {
        u2[iv] += f2d_exact(dA[d][k]);
        if (dlt_pos(u2[iv], eps))
          u2[iv] = 0.0;
        if (dgt_pos(u2[iv], one_m_eps))
          u2[iv] = 1.0;
      }
    }
  }
  const int ive[4] = { H::IE, H::IU, H::IV, H::IW };
#pragma unroll
  for (int e = 0; e < 4; ++e)
  {
    float s, t;
    two_sum(es[e], et[e], s, t);
    u2[ive[e]] += ff_to_d(s, t);
  }
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
}

// THINC, STIFF: compile-time cases of the FP32-bulk form (-1: tested at run
// time, the FP64 form)
template <bool MIXED, int THINC = -1, int STIFF = -1>
__global__ void __launch_bounds__(512, MIXED ? 2 : 1)
step3d_kernel(StepArgs a)
{
  using T = Step3DTraits<MIXED>;
  using R = typename T::R;
  using H = V<3>;
  constexpr int B = T::B, NT = T::NT, G = T::G, GG = T::GG, GGG = T::GGG, S = T::S, SS = T::SS, SSS = T::SSS, NC = 512;
  constexpr int NFF = T::NFF;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  R *          sQ = reinterpret_cast<R *>(smem_raw);
  R *          sHS = sQ + T::NQ * GGG;
  R *          sF = sHS + T::NHS * SSS; // [9][NFF] faces of the current direction
  using DtT = typename std::conditional<MIXED, float, double>::type;
  __shared__ DtT     sRed[NT / 32];
  __shared__ int     sSlot[12]; // the block's reflux slots (faces 0-5), then its defer slots
  __shared__ int     sNext;     // the CTA's next block
  const int          tid = threadIdx.x;
  const PhysParams & P = a.p;
  const int          eosk = STIFF < 0 ? (P.mg_any ? 2 : ((P.gpx[0] != 0.0 || P.gpx[1] != 0.0) ? 1 : 0)) : STIFF;
  const int          ci = tid % B, cj = (tid / B) % B, ck = tid / (B * B);

  const int nwalk = step_count(a);
  for (int iw = blockIdx.x; iw < nwalk;)
  {
    const int    n = a.work ? a.work[iw] : iw;
    // the next block is claimed now (the ticket's latency hides behind the gather)
    const int    next_v = tid == 12 ? claim_next(a, iw, nwalk) : 0;
    const int    ins = a.m.inst ? a.m.inst[n] : 0;
    const double dx = P.level_dx[a.m.level[n]];
    const int    c0[3] = { a.m.coord[n * 3 + 0], a.m.coord[n * 3 + 1], a.m.coord[n * 3 + 2] };
    int          slot_v = -1; // coarse/fine slots, stored to shared memory after the gather
    if (a.m.reflux_slot && tid < 12)
      slot_v = tid < 6 ? a.m.reflux_slot[n * 6 + tid] : a.m.defer_slot[n * 6 + tid - 6];
    R            dtdx_r;
    if constexpr (MIXED)
      dtdx_r = d2f_fast(a.dt[ins]) * __frcp_rn(d2f_fast(dx));
    else
      dtdx_r = a.dt[ins] / dx;

    // ---------------- phase 1: own cell (coalesced) + halo -> primitives
    // (the own cell first, so that its nine doubles are dead before the halo
    // gather: at 64 registers a live own cell spilled)
    double uin[H::NV];
    {
      const double * base = a.U + (size_t)n * H::NV * NC + tid;
#pragma unroll
      for (int v = 0; v < H::NV; ++v)
        uin[v] = base[v * NC];
    }
    store_prim3<MIXED>(sQ, (ci + 2) + G * (cj + 2) + GG * (ck + 2), uin, P, eosk);
    // FP32-bulk form: the owned cell's volume-fraction source-term factors
    // and its volume fractions as floats, taken now so that the nine doubles
    // of the cell do not stay live through the gather, slope and face phases;
    // the final update reads the cell from U again
    float a0f = 0.0f, a1f = 0.0f, af0 = 0.0f, af1 = 0.0f;
    if constexpr (MIXED)
    {
      float fst0, fst1;
      source_factors_mixed<3>(uin, P, eosk, fst0, fst1);
      af0 = d2f_fast(uin[H::IA0]);
      af1 = d2f_fast(uin[H::IA1]);
      a0f = af0 * fst0;
      a1f = af1 * fst1;
    }
    const int nhalo = HALO3_FULL + ((THINC < 0 ? P.thinc != 0 : THINC == 1) ? HALO3_ALPHA : 0);
    for (int h = tid; h < nhalo; h += NT)
    {
      int g[3];
      halo_coords_3d(h, g);
      const int gidx = (g[0] + 2) + G * (g[1] + 2) + GG * (g[2] + 2);
      double    u[H::NV];
      if (h < HALO3_FULL)
      {
        if (!gather_ghost_3d(a, n, c0, g, u))
        {
          raise_status(a.status, STATUS_MESH);
          const double * own = a.U + (size_t)n * H::NV * NC + tid;
#pragma unroll
          for (int v = 0; v < H::NV; ++v)
            u[v] = own[v * NC];
        }
        store_prim3<MIXED>(sQ, gidx, u, P, eosk);
      }
      else
      {
        if (!gather_ghost_3d<true>(a, n, c0, g, u))
        {
          raise_status(a.status, STATUS_MESH);
          u[H::IA0] = a.U[((size_t)n * H::NV + H::IA0) * NC + tid];
        }
        sQ[6 * GGG + gidx] = alpha_prim<MIXED>(u[H::IA0]);
      }
    }
    if (tid < 12)
      sSlot[tid] = slot_v;
    if (tid == 12)
      sNext = next_v;
    __syncthreads();
    // the next block of this CTA: its own cells and table rows into L2
    if (tid < 3 && sNext < nwalk)
    {
      const int nn = a.work ? a.work[sNext] : sNext;
      if (tid == 0)
        prefetch_l2_range(a.U + (size_t)nn * H::NV * NC, (unsigned)(H::NV * NC * sizeof(double)));
      else if (tid == 1)
        prefetch_l2_range(a.m.nbr + (size_t)nn * 27 * 8, 27 * 8 * sizeof(int32_t));
      else
        prefetch_l2_line(a.m.nbr_rel + (size_t)nn * 27);
    }
    // and its same-level or coarser face neighbours (most of its halo), from
    // the last warp (its table loads stall only that warp)
    if (tid >= NT - 6 && sNext < nwalk)
    {
      const int nn = a.work ? a.work[sNext] : sNext;
      const int fs = NT - 1 - tid; // face 0..5
      const int slot = 13 + ((fs & 1) ? 1 : -1) * ((fs >> 1) == 0 ? 1 : ((fs >> 1) == 1 ? 3 : 9));
      if (a.m.nbr_rel[(size_t)nn * 27 + slot] <= 0)
      {
        const int src = a.m.nbr[((size_t)nn * 27 + slot) * 8];
        if (src >= 0 && src < a.m.n_total)
          prefetch_l2_range(a.U + (size_t)src * H::NV * NC, (unsigned)(H::NV * NC * sizeof(double)));
      }
    }

    // ---------------- phase 2: face-neighbour cells: Hancock source
    // The 896 cells of the ring that neighbour a face (the block, then the
    // layer beyond each face; the ring's edges and corners are never a face
    // neighbour), enumerated without gaps: two rounds of 512 threads, the
    // second with 12 full warps.  r: the cell's index in the ring (S^3) layout.
    for (int h = tid; h < NC + 6 * B * B; h += NT)
    {
      int ri, rj, rk;
      if (h < NC)
      {
        ri = h & 7;
        rj = (h >> 3) & 7;
        rk = h >> 6;
      }
      else
      {
        const int i = h - NC, f = i >> 6, pa = i & 7, pb = (i >> 3) & 7;
        const int side = (f & 1) ? B : -1;
        ri = f < 2 ? side : pa;
        rj = f < 2 ? pa : (f < 4 ? side : pb);
        rk = f < 4 ? pb : side;
      }
      const int r = (ri + 1) + S * (rj + 1) + SS * (rk + 1);
      const int gi = (ri + 2) + G * (rj + 2) + GG * (rk + 2);
      if (P.integrator == 0)
      {
        R st;
        if constexpr (MIXED)
          st = P.f_slope_type;
        else
          st = P.slope_type;
        R dq[3][6], q[6];
#pragma unroll
        for (int k = 0; k < 6; ++k)
        {
          const R * Qk = sQ + k * GGG;
          q[k] = Qk[gi];
          if constexpr (MIXED)
          {
            // x and y in one packed evaluation, z alone
            const float2 d = slope_pair(make_float2(q[k], q[k]), make_float2(Qk[gi + 1], Qk[gi + G]), make_float2(Qk[gi - 1], Qk[gi - G]), st);
            dq[0][k] = d.x;
            dq[1][k] = d.y;
          }
          else
          {
            dq[0][k] = slope_at<R>(Qk, gi, 1, st);
            dq[1][k] = slope_at<R>(Qk, gi, G, st);
          }
          dq[2][k] = slope_at<R>(Qk, gi, GG, st);
        }
        const R a0 = sQ[6 * GGG + gi];
        const R r0 = q[0], r1 = q[1], p = q[2], u = q[3], v = q[4], w = q[5];
        const R rr = r0 + r1;
        R       c;
        if constexpr (MIXED)
          c = sound_speed_eos(P, eosk, rr, p, a0, r0, r1);
        else
          c = sound_speed_mix(P, rr, p, a0, 1 - a0, r0, r1);
        const R drx0 = dq[0][0], drx1 = dq[0][1], dpx = dq[0][2], dux = dq[0][3], dvx = dq[0][4], dwx = dq[0][5];
        const R dry0 = dq[1][0], dry1 = dq[1][1], dpy = dq[1][2], duy = dq[1][3], dvy = dq[1][4], dwy = dq[1][5];
        const R drz0 = dq[2][0], drz1 = dq[2][1], dpz = dq[2][2], duz = dq[2][3], dvz = dq[2][4], dwz = dq[2][5];
        const R dtdx = dtdx_r, dtdy = dtdx_r, dtdz = dtdx_r;
        // ComputeFluxesAndStoreFunctor.cpp:273-306
        const R sr0 = (-u * (drx0 + drx1) - dux * rr) * dtdx + (-v * (dry0 + dry1) - dvy * rr) * dtdy +
                      (-w * (drz0 + drz1) - dwz * rr) * dtdz;
        const R sr0_0 = sr0 * a0;
        const R sr0_1 = sr0 * (R(1) - a0);
        const R su0 = (-u * dux - dpx / rr) * dtdx + (-v * duy) * dtdy + (-w * duz) * dtdz;
        const R sv0 = (-u * dvx) * dtdx + (-v * dvy - dpy / rr) * dtdy + (-w * dvz) * dtdz;
        const R sw0 = (-u * dwx) * dtdx + (-v * dwy) * dtdy + (-w * dwz - dpz / rr) * dtdz;
        const R sp0 = (-u * dpx - dux * rr * c * c) * dtdx + (-v * dpy - dvy * rr * c * c) * dtdy +
                      (-w * dpz - dwz * rr * c * c) * dtdz;
        sHS[0 * SSS + r] = R(0.5) * sr0_0;
        sHS[1 * SSS + r] = R(0.5) * sr0_1;
        sHS[2 * SSS + r] = R(0.5) * sp0;
        sHS[3 * SSS + r] = R(0.5) * su0;
        sHS[4 * SSS + r] = R(0.5) * sv0;
        sHS[5 * SSS + r] = R(0.5) * sw0;
      }

    }
    __syncthreads();

    // deferred cells (next to a finer face) are finished by reflux3d_kernel
    const int * dsl = a.m.defer_slot ? sSlot + 6 : nullptr;
    bool        deferred = false;
    if (dsl)
    {
      const int cc[3] = { ci, cj, ck };
#pragma unroll
      for (int f = 0; f < 6; ++f)
        deferred = deferred || (dsl[f] >= 0 && cc[f >> 1] == ((f & 1) ? B - 1 : 0));
    }

    // FP64 form: volume-fraction source-term factors and the running state
    // of the owned cell
    double st0 = 1.0, st1 = 1.0;
    double u2[H::NV];
    if constexpr (!MIXED)
    {
      source_factors_fp64<3>(uin, P, st0, st1);
#pragma unroll
      for (int v = 0; v < H::NV; ++v)
        u2[v] = uin[v];
    }
    // mixed form: per-direction increments of the clamped quantities (exact
    // float pairs) and running float-float sums of energy and momentum
    float hh[3][2], ll[3][2], dA[3][2];
    float es[4] = { 0.f, 0.f, 0.f, 0.f }, et[4] = { 0.f, 0.f, 0.f, 0.f };

    // passes of face directions.  FP32-bulk: 1,728 faces in 4 rounds of 512
    // threads over two flux buffers: pass 0 computes all X faces (buffer 0)
    // and the first 448 Y faces (buffer 1) and updates X; pass 1 the other
    // 128 Y faces and all Z faces (into buffer 0) and updates Y and Z.  FP64:
    // one direction per pass.
#pragma unroll
    for (int pass = 0; pass < (MIXED ? 2 : 3); ++pass)
    {
      const int nd = MIXED ? pass + 1 : 1;
      // ---------------- phase 3: faces of this pass
      if constexpr (MIXED)
      {
        static_assert(NFF > NT && NFF - NT < NT && 3 * NFF - 2 * NT <= 2 * NT, "two rounds of faces per pass");
        constexpr int XR = NFF - NT;      // X faces of pass 0's second round (64)
        constexpr int YA = NT - XR;       // Y faces of pass 0 (448)
        constexpr int YB = NFF - YA;      // Y faces of pass 1 (128)
        R *           sF1 = sF + T::NF * NFF;
        if (pass == 0)
        {
          face_flux3<MIXED, 0, THINC, STIFF == 2>(sQ, sHS, tid, sF, dtdx_r, P);
          if (tid < XR)
            face_flux3<MIXED, 0, THINC, STIFF == 2>(sQ, sHS, tid + NT, sF, dtdx_r, P);
          else
            face_flux3<MIXED, 1, THINC, STIFF == 2>(sQ, sHS, tid - XR, sF1, dtdx_r, P);
        }
        else
        {
          if (tid < YB)
            face_flux3<MIXED, 1, THINC, STIFF == 2>(sQ, sHS, tid + YA, sF1, dtdx_r, P);
          else
            face_flux3<MIXED, 2, THINC, STIFF == 2>(sQ, sHS, tid - YB, sF, dtdx_r, P);
          if (tid < NFF - (NT - YB))
            face_flux3<MIXED, 2, THINC, STIFF == 2>(sQ, sHS, tid + NT - YB, sF, dtdx_r, P);
        }
      }
      else
      {
        for (int f = tid; f < NFF; f += NT)
        {
          if (pass == 0)
            face_flux3<MIXED, 0, THINC, STIFF == 2>(sQ, sHS, f, sF, dtdx_r, P);
          else if (pass == 1)
            face_flux3<MIXED, 1, THINC, STIFF == 2>(sQ, sHS, f, sF, dtdx_r, P);
          else
            face_flux3<MIXED, 2, THINC, STIFF == 2>(sQ, sHS, f, sF, dtdx_r, P);
        }
      }
      __syncthreads();

#pragma unroll
      for (int dsub = 0; dsub < nd; ++dsub)
      {
        const int dir = MIXED ? (pass == 0 ? 0 : 1 + dsub) : pass;
        R *       sFd = sF + (MIXED && dir == 1 ? T::NF * NFF : 0);

        // face index of the owned cell's left/right face in this direction
        const int ext0 = B + (dir == 0), ext1 = B + (dir == 1);
        const int il = ci + ext0 * (cj + ext1 * ck);
        const int step = dir == 0 ? 1 : (dir == 1 ? ext0 : ext0 * ext1);
        const int ir = il + step;

        // ---------------- publish coarse/fine records of this direction (AMR only)
        if (a.m.reflux_slot)
        {
          for (int side = 0; side < 2; ++side)
          {
            const int face = 2 * dir + side;
            const int rs = sSlot[face];
            // positions along the face: the two transverse coordinates (first, second)
            if (rs >= 0 && tid < B * B)
            {
              const int t1 = tid % B, t2 = tid / B;
              int       c3[3];
              c3[dir] = side ? B : 0;
              c3[dir == 0 ? 1 : 0] = t1;
              c3[dir == 2 ? 1 : 2] = t2;
              const int fidx = c3[0] + ext0 * (c3[1] + ext1 * c3[2]);
              double *  dst = a.reflux_buf + ((size_t)rs * B * B + tid) * 9;
#pragma unroll
              for (int k = 0; k < 9; ++k)
                dst[k] = (double)sFd[k * NFF + fidx];
            }
          }
          // own face fluxes of deferred cells, this direction (left then right)
          if (deferred)
          {
            const int cc[3] = { ci, cj, ck };
            for (int f = 0; f < 6; ++f)
            {
              if (dsl[f] < 0 || cc[f >> 1] != ((f & 1) ? B - 1 : 0))
                continue;
              const int d2 = f >> 1;
              const int t1 = cc[d2 == 0 ? 1 : 0], t2 = cc[d2 == 2 ? 1 : 2];
              double *  dst = a.defer_buf + (((size_t)dsl[f] * B * B + t1 + B * t2) * 6 + 2 * dir) * 9;
#pragma unroll
              for (int k = 0; k < 9; ++k)
              {
                dst[k] = (double)sFd[k * NFF + il];
                dst[9 + k] = (double)sFd[k * NFF + ir];
              }
            }
          }
        }

        // ---------------- phase 4: this direction's update of the owned cell
        if constexpr (!MIXED)
        {
          const double a0n = uin[H::IA0], a1n = uin[H::IA1];
          double       acc[8];
#pragma unroll
          for (int k = 0; k < 8; ++k)
            acc[k] = 0.0 + sFd[k * NFF + il];
          const double usl = sFd[H::FUS * NFF + il];
          acc[H::FA0] -= st0 * usl * a0n;
          acc[H::FA1] -= st1 * usl * a1n;
#pragma unroll
          for (int k = 0; k < 8; ++k)
            acc[k] = acc[k] - sFd[k * NFF + ir];
          const double usr = sFd[H::FUS * NFF + ir];
          acc[H::FA0] += st0 * usr * a0n;
          acc[H::FA1] += st1 * usr * a1n;
          apply_dir_fp64(u2, acc);
        }
        else
        {
          // two variables per packed FP32x2 transformation (bit-identical to
          // the scalar form): the partial densities, then (E, rho u) and
          // (rho v, rho w)
          {
            float2 h, l;
            two_diff2(make_float2(sFd[H::FR0 * NFF + il], sFd[H::FR1 * NFF + il]), make_float2(sFd[H::FR0 * NFF + ir], sFd[H::FR1 * NFF + ir]), h, l);
            hh[dir][0] = h.x;
            hh[dir][1] = h.y;
            ll[dir][0] = l.x;
            ll[dir][1] = l.y;
          }
          const int ke[4] = { H::FE, H::FU, H::FV, H::FW };
#pragma unroll
          for (int e = 0; e < 4; e += 2)
          {
            float2 h, l, s, t;
            two_diff2(make_float2(sFd[ke[e] * NFF + il], sFd[ke[e + 1] * NFF + il]), make_float2(sFd[ke[e] * NFF + ir], sFd[ke[e + 1] * NFF + ir]), h, l);
            two_sum2(make_float2(es[e], es[e + 1]), h, s, t);
            const float2 tl = __fadd2_rn(make_float2(et[e], et[e + 1]), __fadd2_rn(t, l));
            es[e] = s.x;
            es[e + 1] = s.y;
            et[e] = tl.x;
            et[e + 1] = tl.y;
          }
          const float usl = sFd[H::FUS * NFF + il], usr = sFd[H::FUS * NFF + ir];
          dA[dir][0] = ((sFd[H::FA0 * NFF + il] - usl * a0f) - sFd[H::FA0 * NFF + ir]) + usr * a0f;
          dA[dir][1] = ((sFd[H::FA1 * NFF + il] - usl * a1f) - sFd[H::FA1 * NFF + ir]) + usr * a1f;
        }
      }
      __syncthreads();
    }

    if constexpr (MIXED)
    {
      // the old state read again, then the update of the three directions
      {
        const double * base = a.U + (size_t)n * H::NV * NC + tid;
#pragma unroll
        for (int v = 0; v < H::NV; ++v)
          u2[v] = base[v * NC];
      }
      apply_mixed_3d(u2, hh, ll, dA, es, et, af0, af1);
    }
    else
    {
      // FixVolumeFractionsNormalization (.cpp:49-72)
      const double sum_alpha = u2[H::IA0] + u2[H::IA1];
      const double sum_alpha_rho = u2[H::IAD0] + u2[H::IAD1];
      const double inv = 1.0 / sum_alpha;
      u2[H::IA0] *= inv;
      u2[H::IA1] *= inv;
      u2[H::ID] = sum_alpha_rho;
    }

    DtT m_inv = DtT(0);
    if (!deferred)
    {
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
      if (a.invdt)
      {
        if constexpr (MIXED)
        {
          float       df, ux, uy, uz, a0;
          const float p = pressure_mixed<3>(u2, P, eosk, df, ux, uy, uz, a0);
          const float c = sound_speed_eos(P, eosk, df, p, fmaxf(0.0f, fminf(1.0f, a0)), d2f_fast(u2[H::IAD0]), d2f_fast(u2[H::IAD1]));
          m_inv = (((c + fabsf(ux)) + (c + fabsf(uy))) + (c + fabsf(uz))) * __frcp_rn(d2f_fast(dx));
        }
        else
        {
          double       q[7];
          const double c = prim_fp64<3>(u2, q, P);
          m_inv = (c + fabs(q[H::QU])) / dx + (c + fabs(q[H::QV])) / dx + (c + fabs(q[H::QW])) / dx;
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
    const int next = sNext; // read before the barrier: the next block's claim overwrites it
    __syncthreads();
    iw = next;
  }
}

// reflux: coarse cells next to finer faces, one thread per (record, cell of
// the face).  Replays update_U direction by direction with the fine face sums
// (2x2 fine faces, / 8) of get_flux_from_fine_neighbor.
template <bool MIXED>
__global__ void
reflux3d_kernel(StepArgs a)
{
  using H = V<3>;
  using D = DeferInfo<3>;
  constexpr int B = 8, NC = 512;
  const int     gid = blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= a.m.n_defer * B * B)
    return;
  const int rec = gid / (B * B), pos = gid % (B * B);
  // first wave: the record's DeferInfo row
  int row[D::STRIDE];
  {
    const int4 * r4 = reinterpret_cast<const int4 *>(a.m.defer_info + (size_t)rec * D::STRIDE);
#pragma unroll
    for (int q = 0; q < D::STRIDE / 4; ++q)
    {
      const int4 v = r4[q];
      row[4 * q] = v.x;
      row[4 * q + 1] = v.y;
      row[4 * q + 2] = v.z;
      row[4 * q + 3] = v.w;
    }
  }
  const int code = row[0];
  const int n = code >> 3, face = code & 7;
  if (a.inst_active && !a.inst_active[row[D::INST]])
    return;
  const int dirf = face >> 1, sidef = face & 1;
  int       cc[3];
  cc[dirf] = sidef ? B - 1 : 0;
  cc[dirf == 0 ? 1 : 0] = pos % B;
  cc[dirf == 2 ? 1 : 2] = pos / B;
  const int * dsl = row + 1;
#pragma unroll
  for (int f2 = 0; f2 < 6; ++f2)
    if (f2 < face && dsl[f2] >= 0 && cc[f2 >> 1] == ((f2 & 1) ? B - 1 : 0))
      return; // handled by the lower face index
  // second wave: the cell's old state and the face fluxes
  const double * own = a.defer_buf + ((size_t)dsl[face] * B * B + pos) * 54;
  const int      cell = cc[0] + B * (cc[1] + B * cc[2]);
  const double * ub = a.U + (size_t)n * H::NV * NC + cell;
  double         uin[H::NV], u2[H::NV];
#pragma unroll
  for (int v = 0; v < H::NV; ++v)
    u2[v] = uin[v] = ub[v * NC];
  const int    ins = row[D::INST];
  const double dx = a.p.level_dx[row[D::LEVEL]];
  if constexpr (MIXED)
  {
    // FP32-bulk form: per direction the two sides' fluxes as float pairs (a
    // fine side is the float-float sum of its 2x2 fine faces, / 8; the
    // records hold floats as doubles), their differences as exact float
    // pairs, and the step kernel's update of the increments (apply_mixed_3d)
    const int eosk = a.p.mg_any ? 2 : ((a.p.gpx[0] != 0.0 || a.p.gpx[1] != 0.0) ? 1 : 0);
    float     fst0, fst1;
    source_factors_mixed<3>(uin, a.p, eosk, fst0, fst1);
    const float af0 = d2f_fast(uin[H::IA0]), af1 = d2f_fast(uin[H::IA1]);
    const float a0f = af0 * fst0, a1f = af1 * fst1;
    float       hh[3][2], ll[3][2], dA[3][2];
    float       es[4] = { 0.f, 0.f, 0.f, 0.f }, et[4] = { 0.f, 0.f, 0.f, 0.f };
    const int   ke[4] = { H::FE, H::FU, H::FV, H::FW };
#pragma unroll
    for (int dir = 0; dir < 3; ++dir)
    {
      const int e1 = dir == 0 ? 1 : 0, e2 = dir == 2 ? 1 : 2;
      float     Fh[2][9], Fl[2][9];
#pragma unroll
      for (int side = 0; side < 2; ++side)
      {
        const int  fface = 2 * dir + side;
        const bool fine = cc[dir] == (side ? B - 1 : 0) && dsl[fface] >= 0;
        if (fine)
        {
          int ch[3], fl[3];
          ch[dir] = side ? 0 : 1;
          fl[dir] = 0;
#pragma unroll
          for (int e = 0; e < 3; ++e)
            if (e != dir)
            {
              const int f = 2 * cc[e];
              ch[e] = f / B;
              fl[e] = f - ch[e] * B;
            }
          const int rs = row[D::RS + fface * D::NCF + ch[e1] + 2 * ch[e2]];
          if (rs < 0)
          {
            raise_status(a.status, STATUS_MESH);
            return;
          }
          const double * fb = a.reflux_buf + ((size_t)rs * B * B + fl[e1] + B * fl[e2]) * 9;
#pragma unroll
          for (int k = 0; k < 9; ++k)
          {
            const float v0 = d2f_fast(fb[k]), v1 = d2f_fast(fb[9 + k]);
            const float v2 = d2f_fast(fb[B * 9 + k]), v3 = d2f_fast(fb[(B + 1) * 9 + k]);
            float       s, t1, t2, t3;
            two_sum(v0, v1, s, t1);
            two_sum(s, v2, s, t2);
            two_sum(s, v3, s, t3);
            Fh[side][k] = 0.125f * s;
            Fl[side][k] = 0.125f * ((t1 + t2) + t3);
          }
        }
        else
        {
          const double * fr = own + fface * 9;
#pragma unroll
          for (int k = 0; k < 9; ++k)
          {
            Fh[side][k] = d2f_fast(fr[k]);
            Fl[side][k] = 0.0f;
          }
        }
      }
      two_diff(Fh[0][H::FR0], Fh[1][H::FR0], hh[dir][0], ll[dir][0]);
      ll[dir][0] += Fl[0][H::FR0] - Fl[1][H::FR0];
      two_diff(Fh[0][H::FR1], Fh[1][H::FR1], hh[dir][1], ll[dir][1]);
      ll[dir][1] += Fl[0][H::FR1] - Fl[1][H::FR1];
#pragma unroll
      for (int e = 0; e < 4; ++e)
      {
        float h, l, t;
        two_diff(Fh[0][ke[e]], Fh[1][ke[e]], h, l);
        l += Fl[0][ke[e]] - Fl[1][ke[e]];
        two_sum(es[e], h, es[e], t);
        et[e] += t + l;
      }
      const float usl = Fh[0][H::FUS] + Fl[0][H::FUS], usr = Fh[1][H::FUS] + Fl[1][H::FUS];
      dA[dir][0] = (((Fh[0][H::FA0] + Fl[0][H::FA0]) - usl * a0f) - (Fh[1][H::FA0] + Fl[1][H::FA0])) + usr * a0f;
      dA[dir][1] = (((Fh[0][H::FA1] + Fl[0][H::FA1]) - usl * a1f) - (Fh[1][H::FA1] + Fl[1][H::FA1])) + usr * a1f;
    }
    apply_mixed_3d(u2, hh, ll, dA, es, et, af0, af1);
  }
  else
  {
  const double a0n = uin[H::IA0], a1n = uin[H::IA1];
  double       st0, st1;
  source_factors_fp64<3>(uin, a.p, st0, st1);
  for (int dir = 0; dir < 3; ++dir)
  {
    const int e1 = dir == 0 ? 1 : 0, e2 = dir == 2 ? 1 : 2;
    double    acc[8];
    for (int k = 0; k < 8; ++k)
      acc[k] = 0.0;
    for (int side = 0; side < 2; ++side)
    {
      const int  fface = 2 * dir + side;
      const bool fine = cc[dir] == (side ? B - 1 : 0) && dsl[fface] >= 0;
      if (fine)
      {
        int ch[3], fl[3];
        ch[dir] = side ? 0 : 1;
        fl[dir] = 0;
        for (int e = 0; e < 3; ++e)
          if (e != dir)
          {
            const int f = 2 * cc[e];
            ch[e] = f / B;
            fl[e] = f - ch[e] * B;
          }
        const int rs = row[D::RS + fface * D::NCF + ch[e1] + 2 * ch[e2]];
        if (rs < 0)
        {
          raise_status(a.status, STATUS_MESH);
          return;
        }
        double fv[9];
        for (int k = 0; k < 9; ++k)
        {
          double sum = 0.0;
          for (int o2 = 0; o2 < 2; ++o2)
            for (int o1 = 0; o1 < 2; ++o1)
              sum += a.reflux_buf[((size_t)rs * B * B + (fl[e1] + o1) + B * (fl[e2] + o2)) * 9 + k];
          fv[k] = sum;
        }
        for (int k = 0; k < 8; ++k)
          acc[k] = side == 0 ? acc[k] + fv[k] / 8.0 : acc[k] - fv[k] / 8.0;
        const double us = fv[8];
        if (side == 0)
        {
          acc[H::FA0] -= st0 * us * a0n / 8.0;
          acc[H::FA1] -= st1 * us * a1n / 8.0;
        }
        else
        {
          acc[H::FA0] += st0 * us * a0n / 8.0;
          acc[H::FA1] += st1 * us * a1n / 8.0;
        }
      }
      else
      {
        const double * fr = own + (2 * dir + side) * 9;
        for (int k = 0; k < 8; ++k)
          acc[k] = side == 0 ? acc[k] + fr[k] : acc[k] - fr[k];
        const double us = fr[8];
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
    apply_dir_fp64(u2, acc);
  }
  const double sum_alpha = u2[H::IA0] + u2[H::IA1];
  const double sum_alpha_rho = u2[H::IAD0] + u2[H::IAD1];
  const double inv = 1.0 / sum_alpha;
  u2[H::IA0] *= inv;
  u2[H::IA1] *= inv;
  u2[H::ID] = sum_alpha_rho;
  }
  double * out = a.U2 + (size_t)n * H::NV * NC + cell;
  bool     finite = true;
  for (int v = 0; v < H::NV; ++v)
  {
    out[v * NC] = u2[v];
    finite = finite && finite_bits(u2[v]);
  }
  if (!finite)
    raise_status(a.status, STATUS_NONPHYSICAL);
  if (a.invdt)
  {
    if constexpr (MIXED)
    {
      float       df, ux, uy, uz, a0;
      const int   eosk = a.p.mg_any ? 2 : ((a.p.gpx[0] != 0.0 || a.p.gpx[1] != 0.0) ? 1 : 0);
      const float p = pressure_mixed<3>(u2, a.p, eosk, df, ux, uy, uz, a0);
      const float c = sound_speed_eos(a.p, eosk, df, p, fmaxf(0.0f, fminf(1.0f, a0)), d2f_fast(u2[V<3>::IAD0]), d2f_fast(u2[V<3>::IAD1]));
      atomic_max_pos_warp(a.invdt, ins, (double)((((c + fabsf(ux)) + (c + fabsf(uy))) + (c + fabsf(uz))) * __frcp_rn(d2f_fast(dx))));
    }
    else
    {
      double       q[7];
      const double c = prim_fp64<3>(u2, q, a.p);
      atomic_max_pos_warp(a.invdt, ins, (c + fabs(q[H::QU])) / dx + (c + fabs(q[H::QV])) / dx + (c + fabs(q[H::QW])) / dx);
    }
  }
}

} // namespace g5
