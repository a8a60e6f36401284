// g5_aux.cuh — boundary fill of outside blocks, standalone CFL reduction,
// refine flags and the device-side dt update of the solver loop.
#pragma once

#include <type_traits>

#include "g5_common.cuh"

namespace g5
{

// FillOutsideCellFunctor::operator() (border_conditions/FillOutside.cpp:71-170):
// one thread per outside cell.  The reference visits the faces in order and
// every face that applies rewrites the whole cell, so the last such face
// wins: it is found first (from the outside block's row, read in one wave),
// then the cell is copied once.
template <int DIM, int B>
__global__ void
fill_outside_kernel(double * U, DevMesh m, PhysParams P)
{
  using H = V<DIM>;
  constexpr int NC = (DIM == 2) ? B * B : B * B * B;
  const long    gid = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= (long)m.n_outside * NC)
    return;
  const int o = (int)(gid / NC), c = (int)(gid % NC);
  const int nout = m.n_owned + o;
  const int nin = m.out_src[o];
  int8_t    border[6], normal[3];
#pragma unroll
  for (int f = 0; f < 2 * DIM; ++f)
    border[f] = m.out_border[o * 6 + f];
#pragma unroll
  for (int e = 0; e < DIM; ++e)
    normal[e] = m.out_normal[o * 3 + e];
  if (nin < 0 || nin >= m.n_owned)
    return;
  int last = -1;
#pragma unroll
  for (int face = 0; face < 2 * DIM; ++face)
    if (border[face] && normal[face >> 1] != 0 && (P.bc[face] == 2 || P.bc[face] == 3))
      last = face;
  if (last < 0)
    return;
  const int dir = last >> 1, bc = P.bc[last];
  int       ci[3] = { c % B, (c / B) % B, DIM == 3 ? c / (B * B) : 0 };
  ci[dir] = bc == 2 ? ((last & 1) ? B - 1 : 0) : B - 1 - ci[dir];
  const int      cin = ci[0] + B * (ci[1] + B * ci[2]);
  const double * src = U + (size_t)nin * H::NV * NC + cin;
  double *       dst = U + (size_t)nout * H::NV * NC + c;
  double         u[H::NV];
#pragma unroll
  for (int v = 0; v < H::NV; ++v)
    u[v] = src[v * NC];
  if (bc == 3)
    u[H::IU + dir] = -u[H::IU + dir];
#pragma unroll
  for (int v = 0; v < H::NV; ++v)
    dst[v * NC] = u[v];
}

// ComputeDtFiveEqFunctor (scheme/ComputeDtFiveEqFunctor.cpp:87-134): one CTA
// per block, block max, one atomic per CTA.
template <int DIM, int B>
__global__ void
inv_dt_kernel(const double * U, DevMesh m, PhysParams P, double * invdt)
{
  using H = V<DIM>;
  constexpr int NC = (DIM == 2) ? B * B : B * B * B;
  __shared__ double sred[32];
  for (int n = blockIdx.x; n < m.n_owned; n += gridDim.x)
  {
    const double dx = P.level_dx[m.level[n]];
    double       mx = 0.0;
    for (int c = threadIdx.x; c < NC; c += blockDim.x)
    {
      double u[H::NV], q[H::NQ];
      for (int v = 0; v < H::NV; ++v)
        u[v] = U[((size_t)n * H::NV + v) * NC + c];
      const double cs = prim_fp64<DIM>(u, q, P);
      const double vx = cs + fabs(q[H::QU]);
      const double vy = cs + fabs(q[H::QV]);
      if constexpr (DIM == 2)
        mx = fmax(mx, vx / dx + vy / dx);
      else
        mx = fmax(mx, vx / dx + vy / dx + (cs + fabs(q[H::QW])) / dx);
    }
    for (int o = 16; o > 0; o >>= 1)
      mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0)
      sred[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x == 0)
    {
      double mm = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w)
        mm = fmax(mm, sred[w]);
      atomic_max_pos(invdt + (m.inst ? m.inst[n] : 0), mm);
    }
    __syncthreads();
  }
}

// RK2_SSP final stage (SolverGodunovFiveEq.cpp:519-520, the external
// LinearCombination with the SSP coefficients): U2 = 0.5 U + 0.5 U2 on the
// owned blocks, fused with the CFL rate of the result (one CTA per block).
template <int DIM, int B, bool MIXED>
__global__ void
rk2_combine_kernel(const double * U, double * U2, DevMesh m, PhysParams P, double * invdt)
{
  using H = V<DIM>;
  constexpr int NC = (DIM == 2) ? B * B : B * B * B;
  using DtT = typename std::conditional<MIXED, float, double>::type;
  __shared__ DtT sred[32];
  const int      eosk = P.mg_any ? 2 : ((P.gpx[0] != 0.0 || P.gpx[1] != 0.0) ? 1 : 0);
  for (int n = blockIdx.x; n < m.n_owned; n += gridDim.x)
  {
    const double dx = P.level_dx[m.level[n]];
    DtT          mx = DtT(0);
    for (int c = threadIdx.x; c < NC; c += blockDim.x)
    {
      double u[H::NV];
      for (int v = 0; v < H::NV; ++v)
      {
        const size_t i = ((size_t)n * H::NV + v) * NC + c;
        u[v] = 0.5 * U[i] + 0.5 * U2[i];
        U2[i] = u[v];
      }
      if constexpr (MIXED)
      {
        float       d, ux, uy, uz, a0;
        const float p = pressure_mixed<DIM>(u, P, eosk, d, ux, uy, uz, a0);
        const float cs = sound_speed_eos(P, eosk, d, p, fmaxf(0.0f, fminf(1.0f, a0)), d2f_fast(u[H::IAD0]), d2f_fast(u[H::IAD1]));
        float       r = (cs + fabsf(ux)) + (cs + fabsf(uy));
        if constexpr (DIM == 3)
          r += cs + fabsf(uz);
        mx = fmaxf(mx, r * __frcp_rn(d2f_fast(dx)));
      }
      else
      {
        double       q[H::NQ];
        const double cs = prim_fp64<DIM>(u, q, P);
        const double vx = cs + fabs(q[H::QU]);
        const double vy = cs + fabs(q[H::QV]);
        if constexpr (DIM == 2)
          mx = fmax(mx, vx / dx + vy / dx);
        else
          mx = fmax(mx, vx / dx + vy / dx + (cs + fabs(q[H::QW])) / dx);
      }
    }
    if (invdt)
    {
      for (int o = 16; o > 0; o >>= 1)
        mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
      if ((threadIdx.x & 31) == 0)
        sred[threadIdx.x >> 5] = mx;
      __syncthreads();
      if (threadIdx.x == 0)
      {
        DtT mm = DtT(0);
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w)
          mm = fmax(mm, sred[w]);
        atomic_max_pos(invdt + (m.inst ? m.inst[n] : 0), (double)mm);
      }
    }
    __syncthreads();
  }
}

// dt = cfl / inv_dt per instance; inv_dt accumulator cleared for the next step
static __global__ void
dt_update_kernel(double * invdt, double * dt, double * dt_hist, int n_inst, double cfl)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_inst)
    return;
  const double d = cfl / invdt[i];
  dt[i] = d;
  if (dt_hist)
    dt_hist[i] = d;
  invdt[i] = 0.0;
}

// ComputeRefineFlags (scheme/ComputeRefineFlags.cpp:66-368): value of the
// same-level face neighbour of a cell (getNeighborDataSameLevel)
template <int DIM, int B>
__device__ double
neighbor_same_level(const double * U, const DevMesh & m, int n, const int * cell, int dir, int side, int var)
{
  using H = V<DIM>;
  constexpr int NC = (DIM == 2) ? B * B : B * B * B;
  constexpr int NS = (DIM == 2) ? 9 : 27, NCH = (DIM == 2) ? 4 : 8;
  auto          cidx = [](int x, int y, int z) { return x + B * (y + B * z); };
  int           g[3] = { cell[0], cell[1], cell[2] };
  g[dir] += side;
  if (g[dir] >= 0 && g[dir] < B)
    return U[((size_t)n * H::NV + var) * NC + cidx(g[0], g[1], g[2])];
  int d[3] = { 0, 0, 0 }, v[3] = { g[0], g[1], g[2] };
  d[dir] = side;
  v[dir] = g[dir] - side * B;
  const int s = (d[0] + 1) + 3 * (d[1] + 1) + (DIM == 3 ? 9 * (d[2] + 1) : 0);
  const int rel = m.nbr_rel[n * NS + s];
  const int * nb = m.nbr + (n * NS + s) * NCH;
  const double here = U[((size_t)n * H::NV + var) * NC + cidx(cell[0], cell[1], cell[2])];
  if (rel <= 0)
  {
    const int src = nb[0];
    if (src < 0 || src >= m.n_owned)
      return here; // outside the domain: value of the current cell
    if (rel == 0)
      return U[((size_t)src * H::NV + var) * NC + cidx(v[0], v[1], v[2])];
    int cc[3] = { 0, 0, 0 };
    for (int e = 0; e < DIM; ++e)
      cc[e] = ((m.coord[n * 3 + e] + d[e]) & 1) * (B / 2) + (v[e] >> 1);
    return U[((size_t)src * H::NV + var) * NC + cidx(cc[0], cc[1], cc[2])];
  }
  int f0[3] = { 0, 0, 0 }, ch[3] = { 0, 0, 0 };
  for (int e = 0; e < DIM; ++e)
  {
    const int f = 2 * v[e];
    ch[e] = f / B;
    f0[e] = f - ch[e] * B;
  }
  const int F = nb[ch[0] + 2 * ch[1] + 4 * ch[2]];
  if (F < 0 || F >= m.n_owned)
    return here;
  double sum = 0.0;
  for (int oz = 0; oz < (DIM == 3 ? 2 : 1); ++oz)
    for (int oy = 0; oy < 2; ++oy)
      for (int ox = 0; ox < 2; ++ox)
        sum += U[((size_t)F * H::NV + var) * NC + cidx(f0[0] + ox, f0[1] + oy, f0[2] + oz)];
  return sum / (double)(1 << DIM);
}

__device__ __forceinline__ double
normalized_gradient(double v1, double v2)
{
  double vmax = fmax(fabs(v1), fabs(v2));
  if (vmax < 0.001)
    return 0.0;
  vmax = fabs(v1 - v2) / vmax;
  return fmax(fmin(vmax, 1.0), 0.0);
}

template <int DIM, int B>
__global__ void
refine_flags_kernel(const double * U,
                    DevMesh        m,
                    int            indicator,
                    double         eps_r,
                    double         eps_c,
                    double         eps_l,
                    int            lmin,
                    int            lmax,
                    int8_t *       flags)
{
  using H = V<DIM>;
  constexpr int NC = (DIM == 2) ? B * B : B * B * B;
  __shared__ int sflag;
  for (int n = blockIdx.x; n < m.n_owned; n += gridDim.x)
  {
    if (threadIdx.x == 0)
      sflag = -1;
    __syncthreads();
    const int lev = m.level[n];
    int       bflag = -1;
    for (int c = threadIdx.x; c < NC; c += blockDim.x)
    {
      const int cell[3] = { c % B, (c / B) % B, DIM == 3 ? c / (B * B) : 0 };
      int       flag = -1;
      auto      update = [&](double ind) {
        int f;
        if (lev < lmax && ind > eps_r)
          f = 2;
        else if (lev > lmin && ind < eps_c)
          f = 0;
        else
          f = 1;
        flag = flag > f ? flag : f;
      };
      const int vars[2] = { H::IAD0, H::IAD1 };
      if (indicator == 2)
      {
        for (int t = 0; t < 2; ++t)
          for (int d = 0; d < DIM; ++d)
          {
            const double L = neighbor_same_level<DIM, B>(U, m, n, cell, d, -1, vars[t]);
            const double R = neighbor_same_level<DIM, B>(U, m, n, cell, d, +1, vars[t]);
            const double C = U[((size_t)n * H::NV + vars[t]) * NC + c];
            update(fabs(L - 2 * C + R) / (fabs(R - C) + fabs(C - L) + eps_l * (fabs(L) + 2 * fabs(C) + fabs(R))));
          }
      }
      else
      {
        for (int t = 0; t < 2; ++t)
        {
          const double C = U[((size_t)n * H::NV + vars[t]) * NC + c];
          if (indicator == 1)
          {
            double num = 0.0, den = 0.0;
            for (int d = 0; d < DIM; ++d)
            {
              const double L = neighbor_same_level<DIM, B>(U, m, n, cell, d, -1, vars[t]);
              const double R = neighbor_same_level<DIM, B>(U, m, n, cell, d, +1, vars[t]);
              const double aa = L - 2 * C + R;
              num = d == 0 ? aa * aa : num + aa * aa;
              const double tmp = fabs(R - C) + fabs(C - L) + eps_l * (fabs(L) + 2 * fabs(C) + fabs(R));
              den = d == 0 ? tmp * tmp : den + tmp * tmp;
            }
            update(sqrt(num / den));
          }
          else
          {
            double res = -1.7976931348623157e308;
            for (int d = 0; d < DIM; ++d)
            {
              const double L = neighbor_same_level<DIM, B>(U, m, n, cell, d, -1, vars[t]);
              const double R = neighbor_same_level<DIM, B>(U, m, n, cell, d, +1, vars[t]);
              res = fmax(res, normalized_gradient(C, L));
              res = fmax(res, normalized_gradient(C, R));
            }
            update(res);
          }
        }
      }
      bflag = bflag > flag ? bflag : flag;
    }
    atomicMax(&sflag, bflag);
    __syncthreads();
    if (threadIdx.x == 0)
      flags[n] = (int8_t)sflag;
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// block remap after a mesh adaptation (SolverGodunovFiveEq::
// map_userdata_after_adapt, SolverGodunovFiveEq.cpp:1137-1169): one CTA per new
// owned block.  kind 0 copies an old block, kind 1 is the SIMPLE_COPY
// prolongation of one child of an old block (every fine cell takes the parent
// cell containing its centre), kind 2 the restriction of 2^dim old children
// (get_conservative_vars_restriction, ConvertToPrimitivesVariablesFunctor.cpp:
// 208-246: mean of the fine cells for IE IU IV (IW) IAD0 IAD1 IA0, summed in
// z, y, x order, IA1 = 1 - IA0, ID = IAD0 + IAD1).  The host validated kind and
// src, so every index read here is in range.
// ---------------------------------------------------------------------------
template <int DIM, int B>
__global__ void __launch_bounds__(256)
remap_kernel(const double * __restrict__ Uold, double * __restrict__ Unew, const int8_t * __restrict__ kind,
             const int32_t * __restrict__ src, int n_new)
{
  using H = V<DIM>;
  constexpr int NC = DIM == 2 ? B * B : B * B * B;
  constexpr int NCH = 1 << DIM;
  for (int j = blockIdx.x; j < n_new; j += gridDim.x)
  {
    const int       k = kind[j];
    const int32_t * s = src + (size_t)j * NCH;
    double *        out = Unew + (size_t)j * H::NV * NC;
    if (k == 0)
    {
      const double2 * in2 = reinterpret_cast<const double2 *>(Uold + (size_t)s[0] * H::NV * NC);
      double2 *       out2 = reinterpret_cast<double2 *>(out);
      for (int t = threadIdx.x; t < H::NV * NC / 2; t += blockDim.x)
        out2[t] = in2[t];
      continue;
    }
    for (int c = threadIdx.x; c < NC; c += blockDim.x)
    {
      const int cc[3] = { c % B, (c / B) % B, DIM == 3 ? c / (B * B) : 0 };
      if (k == 1)
      {
        const int      ch = s[1];
        const int      px = (ch & 1) * (B / 2) + (cc[0] >> 1);
        const int      py = ((ch >> 1) & 1) * (B / 2) + (cc[1] >> 1);
        const int      pz = DIM == 3 ? ((ch >> 2) & 1) * (B / 2) + (cc[2] >> 1) : 0;
        const double * in = Uold + (size_t)s[0] * H::NV * NC + px + B * (py + B * pz);
#pragma unroll
        for (int v = 0; v < H::NV; ++v)
          out[v * NC + c] = in[v * NC];
      }
      else
      {
        int ch[3] = { 0, 0, 0 }, f0[3] = { 0, 0, 0 };
#pragma unroll
        for (int e = 0; e < DIM; ++e)
        {
          const int f = 2 * cc[e];
          ch[e] = f / B;
          f0[e] = f - ch[e] * B;
        }
        const double * in = Uold + (size_t)s[ch[0] + 2 * ch[1] + 4 * ch[2]] * H::NV * NC;
        const int      vars[7] = { H::IE, H::IU, H::IV, H::IW, H::IAD0, H::IAD1, H::IA0 };
#pragma unroll
        for (int t = 0; t < 7; ++t)
        {
          if (DIM == 2 && t == 3)
            continue;
          const int v = vars[t];
          double    sum = 0.0;
#pragma unroll
          for (int oz = 0; oz < (DIM == 3 ? 2 : 1); ++oz)
#pragma unroll
            for (int oy = 0; oy < 2; ++oy)
#pragma unroll
              for (int ox = 0; ox < 2; ++ox)
                sum += in[v * NC + (f0[0] + ox) + B * ((f0[1] + oy) + B * (DIM == 3 ? f0[2] + oz : 0))];
          out[v * NC + c] = sum / (double)(1 << DIM);
        }
        out[H::IA1 * NC + c] = 1.0 - out[H::IA0 * NC + c];
        out[H::ID * NC + c] = out[H::IAD0 * NC + c] + out[H::IAD1 * NC + c];
      }
    }
  }
}

// per-record rows of DeferInfo<DIM> for the records listed in `codes` (one
// thread per record): everything the reflux pass needs before its data loads
template <int DIM>
__global__ void
defer_info_kernel(DevMesh m, const int32_t * codes, int n, int32_t * info)
{
  using D = DeferInfo<DIM>;
  constexpr int NF = 2 * DIM, NS = DIM == 2 ? 9 : 27, NCH = 1 << DIM;
  const int     r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n)
    return;
  const int code = codes[r];
  const int nb = code >> 3;
  int32_t * row = info + (size_t)r * D::STRIDE;
  row[0] = code;
  for (int f = 0; f < NF; ++f)
  {
    const int ds = m.defer_slot[nb * NF + f];
    row[1 + f] = ds;
    const int dir = f >> 1, side = f & 1;
    int       d[3] = { 0, 0, 0 };
    d[dir] = side ? 1 : -1;
    const int s = (d[0] + 1) + 3 * (d[1] + 1) + (DIM == 3 ? 9 * (d[2] + 1) : 0);
    for (int c = 0; c < D::NCF; ++c)
    {
      int rs = -1;
      if (ds >= 0)
      {
        int ch[3] = { 0, 0, 0 };
        ch[dir] = side ? 0 : 1;
        const int e1 = dir == 0 ? 1 : 0, e2 = dir == 2 ? 1 : 2;
        ch[e1] = c & 1;
        if (DIM == 3)
          ch[e2] = c >> 1;
        const int F = m.nbr[((size_t)nb * NS + s) * NCH + ch[0] + 2 * ch[1] + 4 * ch[2]];
        rs = (F >= 0 && F < m.n_owned) ? m.reflux_slot[F * NF + (f ^ 1)] : -1;
      }
      row[D::RS + f * D::NCF + c] = rs;
    }
  }
  row[D::LEVEL] = m.level[nb];
  row[D::INST] = m.inst ? m.inst[nb] : 0;
  for (int k = D::INST + 1; k < D::STRIDE; ++k)
    row[k] = 0;
}

// ComputeDerivedQuantities::run (utils/ComputeDerivedQuantities.h:96-180):
// one derived quantity of a cell's conservative state, FP64 in the
// reference's operation order.  quantity: 0 RHO_MIX, 1 THERMAL_PRESSURE,
// 2 SPEED_OF_SOUND, 3 SPECIFIC_EKIN, 4 LOCAL_MACH_NUMBER, 5 VX, 6 VY, 7 VZ
// (the DERIVED_QUANTITY enum order).
template <int DIM>
__device__ __forceinline__ double
derived_value(const double * u, int quantity, const PhysParams & P)
{
  using H = V<DIM>;
  double r = 0.0;
  if (quantity == 0)
    r = u[H::ID];
  else if (quantity == 1 || quantity == 3)
  {
    // compute_mixture_ekin (models/utils.h:124-151): density from ID
    const double d = fmax(u[H::ID], P.smallr);
    const double ux = u[H::IU] / d, uy = u[H::IV] / d;
    double       ekin;
    if constexpr (DIM == 2)
      ekin = 0.5 * (ux * ux + uy * uy);
    else
    {
      const double uz = u[H::IW] / d;
      ekin = 0.5 * (ux * ux + uy * uy + uz * uz);
    }
    if (quantity == 3)
      r = ekin;
    else
    {
      // compute_mixture_pressure (models/utils.h:160-185): density from the partial densities
      const double dm = fmax(u[H::IAD0] + u[H::IAD1], P.smallr);
      const double eint = u[H::IE] / dm - ekin;
      const double a0 = u[H::IA0];
      if (!P.mg_any)
        r = (dm * eint - eosPI(P, a0, 1 - a0)) / eosS(P, a0, 1 - a0);
      else
      {
        double S, PI, C1, C0;
        mg_mixture(P, a0, 1 - a0, u[H::IAD0], u[H::IAD1], S, PI, C1, C0);
        r = (dm * eint - PI) / S;
      }
    }
  }
  else
  {
    double       q[7];
    const double cs = prim_fp64<DIM>(u, q, P);
    if (quantity == 2)
      r = cs;
    else if (quantity == 4)
    {
      double un = q[H::QU] * q[H::QU] + q[H::QV] * q[H::QV];
      if constexpr (DIM == 3)
        un += q[H::QW] * q[H::QW];
      un = sqrt(un);
      r = un / cs;
    }
    else if (quantity == 5)
      r = q[H::QU];
    else if (quantity == 6)
      r = q[H::QV];
    else if constexpr (DIM == 3)
      r = q[H::QW];
  }
  return r;
}

// one derived quantity per cell of blocks [oct_begin, oct_begin + num_octs)
// into out[oct][cell]
template <int DIM, int B>
__global__ void
derived_kernel(const double * __restrict__ U, double * __restrict__ out, int quantity, long long oct_begin, long long num_octs,
               PhysParams P)
{
  using H = V<DIM>;
  constexpr int NC = DIM == 2 ? B * B : B * B * B;
  const long long total = num_octs * NC;
  for (long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x; g < total; g += (long long)gridDim.x * blockDim.x)
  {
    const long long oct = oct_begin + g / NC;
    const int       cell = (int)(g % NC);
    double          u[H::NV];
#pragma unroll
    for (int v = 0; v < H::NV; ++v)
      u[v] = U[(oct * H::NV + v) * NC + cell];
    out[oct * NC + cell] = derived_value<DIM>(u, quantity, P);
  }
}

// The fields of one output file (SolverGodunovFiveEq::save_solution_hdf5,
// SolverGodunovFiveEq.cpp:809-886: each a per-quadrant dataset of the state's
// variables or of a derived quantity) for blocks [oct_begin, oct_begin +
// num_octs), in one pass over U: field k to out[k][oct - oct_begin][cell].
// (FieldList codes: a variable of U, or FIELD_DERIVED + a derived quantity).

template <int DIM, int B>
__global__ void
pack_fields_kernel(const double * __restrict__ U, double * __restrict__ out, FieldList fl, long long oct_begin, long long num_octs,
                   PhysParams P)
{
  using H = V<DIM>;
  constexpr int NC = DIM == 2 ? B * B : B * B * B;
  const long long total = num_octs * NC;
  for (long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x; g < total; g += (long long)gridDim.x * blockDim.x)
  {
    const long long oct = oct_begin + g / NC;
    const int       cell = (int)(g % NC);
    double          u[H::NV];
#pragma unroll
    for (int v = 0; v < H::NV; ++v)
      u[v] = U[(oct * H::NV + v) * NC + cell];
    for (int k = 0; k < fl.n; ++k)
    {
      const int c = fl.code[k];
      double    r = 0.0;
#pragma unroll
      for (int v = 0; v < H::NV; ++v)
        r = c == v ? u[v] : r;
      if (c >= FIELD_DERIVED)
        r = derived_value<DIM>(u, c - FIELD_DERIVED, P);
      out[(size_t)k * total + g] = r;
    }
  }
}

} // namespace g5
