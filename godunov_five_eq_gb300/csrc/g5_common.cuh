// g5_common.cuh — shared device types and the per-cell physics of the
// five-equation model (FP64 form and the FP32-bulk form).
//
// The FP64 functions evaluate every expression in the same order as the
// reference (and the translation unit is compiled with --fmad=false), so the
// FP64 path reproduces the reference method bit for bit on identical inputs.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace g5
{

// ---------------------------------------------------------------------------
// parameters and block table passed by value to every kernel
// ---------------------------------------------------------------------------
struct PhysParams
{
  double smallr, smallc, smallp, slope_type;
  double gamma[2], pinf[2];
  double xi[2];  // 1/(gamma_k - 1)
  double gpx[2]; // gamma_k pinf_k xi_k
  double cfl, thinc_beta, thinc_eps;
  int    integrator;  // 0 HANCOCK, 1 RK1, 2 RK2_SSP
  int    thinc;       // 0 MUSCL, 1 THINC
  int    source_term; // 0 ALLAIRE_KOKH, 1 MILLER_PUCKETT
  int    bc[6];
  double level_dx[32];
  // FP32 copies for the FP32-bulk path (converted once on the host)
  float f_smallr, f_smallc, f_smallp, f_slope_type, f_thinc_beta, f_thinc_eps;
  float f_xi[2], f_gpx[2], f_dxi; // f_dxi = xi0 - xi1
  double dgpx;                    // gpx0 - gpx1
  // Mie-Grueneisen material laws (mg_law): kind per material (0 stiffened
  // gas), parameters, reference densities, and whether any law is not the
  // stiffened gas (then every EOS evaluation takes the general path)
  int    eos_kind[2];
  int    mg_any;
  double mg[2][8];
  double mg_rho0[2];
  float  f_mg[2][8]; // FP32 copies for the FP32-bulk path
  float  f_mg_rho0[2];
  float  f_gm1[2], f_gpinf[2]; // gamma_k - 1 and gamma_k pinf_k (stiffened-gas law in the mixture rules)
  // ghost cells in a coarser neighbour: 0 SIMPLE_COPY, 1 EXTRAPOLATE_LINEAR_MINMOD,
  // 2 / 3 CONSERVATIVE_INTERPOLATION_ORDER_2 / 4
  int prolong;
};

struct DevMesh
{
  const int32_t * level;
  const int32_t * coord;       // [n_total*3]
  const int32_t * nbr;         // [n_owned * NS * NC]
  const int8_t *  nbr_rel;     // [n_owned * NS]
  const int32_t * inst;        // [n_total]
  const int32_t * reflux_slot; // [n_owned * 2*dim] slot in reflux_buf, or -1
  const int32_t * defer_slot;  // [n_owned * 2*dim] slot in defer_buf, or -1
  const int32_t * defer_list;  // [n_defer_slots] (block*8 + face) of each deferred record
  const int32_t * defer_info;  // [n_defer][DEFER_INFO<DIM>] per record: code, defer slots of the
                               // block, reflux slots of the fine faces, level, instance
  const int32_t * twin_first;  // [n_owned + 1] CSR over the outside blocks filled from each owned block
  const int32_t * twin_list;   // (outside block) * 8 + the last applicable face of FillOutside
  const int32_t * out_src;     // [n_outside]
  const int8_t *  out_normal;  // [n_outside*3]
  const int8_t *  out_border;  // [n_outside*6]
  int             n_owned, n_outside, n_total, n_inst;
  int             n_defer;
  // prolonged ghost states (prolongation other than SIMPLE_COPY; null
  // otherwise): pg_slot[n] = the owned block's slot in pg, or -1 when no
  // neighbour is coarser; pg = [slot][NV][(b+4)^dim ghosted cells]
  const int32_t * pg_slot = nullptr;
  double *        pg = nullptr;
  // reflux in the tail of the FP32-bulk 2D full-mesh step (null: the separate
  // pass).  fin_tgt[n * 5 + k]: the counters owned block n counts off once
  // its step is written (its own, when it has deferred cells, and those of
  // the coarser blocks it publishes fine-face fluxes to), -1 past the last;
  // per deferred block j: fin_cnt[j] (fin_init[j] between launches: its
  // arrivals plus one tail claim) and its records fin_rec[j * 4 + k] (rows of
  // defer_info, -1 past the last); fin_ticket: the tail claims of a launch
  // (0 between launches)
  const int32_t *      fin_tgt = nullptr;
  unsigned int *       fin_cnt = nullptr;
  const unsigned int * fin_init = nullptr;
  const int32_t *      fin_rec = nullptr;
  unsigned int *       fin_ticket = nullptr;
  int                  n_fin = 0;
};

// row of the per-record table read by the reflux pass in one wave:
// [0] block*8 + face, [1 .. 2*DIM] the block's defer slots per face,
// then per face f and fine child c along the face (2 in 2D, 4 in 3D) the
// reflux slot of that fine face (-1 if none), then level and instance
template <int DIM>
struct DeferInfo
{
  static constexpr int NCF = DIM == 2 ? 2 : 4;
  static constexpr int RS = 1 + 2 * DIM;
  static constexpr int LEVEL = RS + 2 * DIM * NCF, INST = LEVEL + 1;
  static constexpr int STRIDE = DIM == 2 ? 16 : 36;
};

// fields of one output file (pack_fields_kernel): code[k] < NV a variable of
// U (the reference's VarId numbering), FIELD_DERIVED + q derived quantity q
constexpr int FIELD_DERIVED = 64, MAX_PACK_FIELDS = 16;
struct FieldList
{
  int code[MAX_PACK_FIELDS];
  int n;
};

struct StepArgs
{
  const double * U;
  double *       U2;
  const double * dt;         // [n_inst] on the device
  double *       reflux_buf; // fine-block face fluxes at coarse/fine faces
  double *       defer_buf;  // own face fluxes of coarse cells next to finer faces
  double *       invdt;      // [n_inst] (bit-pattern max), may be null
  unsigned int * status;
  const int32_t * work = nullptr; // owned blocks to step (null: all n_owned blocks in order)
  int             n_work = 0;     // entries of work
  const uint8_t * inst_active = nullptr; // per instance: nonzero = stepped (null: all); read by the reflux pass
  int             fill_twins = 0;        // also fill U2's outside blocks (the solver loop's fill after the step)
  // Dynamic block claiming (null: CTA b steps blocks b, b + grid, ...): CTA b
  // steps block b, then claims further blocks with tickets of this counter;
  // the CTA drawing the launch's last ticket resets it to 0.
  unsigned int * ticket = nullptr;
  // layout of the FP32-bulk 2D reflux pass: 0 eight lanes per deferred cell,
  // 1 one thread per deferred cell (the FP64 form and 3D: one thread per
  // cell), 2 eight lanes per cell in the step kernel's tail when m.fin_tgt is
  // set (the full-mesh step), else as 0
  int            reflux_layout = 0;
  DevMesh        m;
  PhysParams     p;
};

// Next block of a persistent step CTA (returns >= nwalk when done).  CTA b
// steps blocks b and b + grid (the CTAs start in step, so a shared counter
// would be drawn by all of them at once), then claims the remaining
// M = nwalk - 2 grid blocks in order with tickets, so that CTAs that finish
// early take more of the tail.  Each of the K = min(grid, nwalk - grid) CTAs
// with a second block draws one ticket per block from its second on, the last
// draw failing: a launch draws M + K tickets and the drawer of the last one
// resets the counter.
__device__ __forceinline__ int
claim_next(const StepArgs & a, int iw, int nwalk)
{
  const int G = (int)gridDim.x;
  if (!a.ticket || iw < G)
    return iw + G;
  const int      M = nwalk - 2 * G > 0 ? nwalk - 2 * G : 0;
  const int      K = nwalk - G < G ? nwalk - G : G;
  const unsigned t = atomicAdd(a.ticket, 1u);
  if (t == (unsigned)(M + K - 1))
    *a.ticket = 0u;
  return t < (unsigned)M ? 2 * G + (int)t : nwalk;
}

// number of blocks a step launch walks
__host__ __device__ inline int
step_count(const StepArgs & a)
{
  return a.work ? a.n_work : a.m.n_owned;
}

constexpr unsigned STATUS_NONPHYSICAL = 1u;
constexpr unsigned STATUS_MESH = 2u;

// variable ids (models/FiveEq.h:35-50)
template <int DIM>
struct V
{
  static constexpr int ID = 0, IE = 1, IP = 1, IU = 2, IV = 3;
  static constexpr int IW = (DIM == 2) ? 3 : 4;
  static constexpr int HC = IW + 1;
  static constexpr int IA0 = HC, IAD0 = HC + 1, IA1 = HC + 2, IAD1 = HC + 3;
  static constexpr int NV = HC + 4;
  // primitive components kept in shared memory: r0 r1 p u v (w) alpha0
  static constexpr int QR0 = 0, QR1 = 1, QP = 2, QU = 3, QV = 4, QW = 5;
  static constexpr int NR = (DIM == 2) ? 5 : 6; // reconstructed components
  static constexpr int QA = NR;                 // alpha0
  static constexpr int NQ = NR + 1;
  // face record: r0 r1 a0 a1 e u v (w) ustar  (already multiplied by dt/dx)
  static constexpr int FR0 = 0, FR1 = 1, FA0 = 2, FA1 = 3, FE = 4, FU = 5, FV = 6, FW = 7;
  static constexpr int FUS = (DIM == 2) ? 7 : 8;
  static constexpr int NF = FUS + 1;
};

__device__ __forceinline__ void
raise_status(unsigned int * st, unsigned bits)
{
  atomicOr(st, bits);
}

// positive doubles order like their bit patterns: max by integer atomic
__device__ __forceinline__ void
atomic_max_pos(double * addr, double v)
{
  if (!(v > 0.0))
    return;
  atomicMax(reinterpret_cast<unsigned long long *>(addr), (unsigned long long)__double_as_longlong(v));
}

// The same for one value per thread of a warp, threads of different
// instances apart: one atomic per instance present in the converged lanes
// (the max of positive doubles is the max of their bit patterns, taken as
// high word then low word).  Thousands of per-thread atomics on one address
// would serialise.
__device__ __forceinline__ void
atomic_max_pos_warp(double * base, int ins, double v)
{
  const unsigned           active = __activemask();
  const unsigned           grp = __match_any_sync(active, ins);
  const unsigned long long b = (v > 0.0) ? (unsigned long long)__double_as_longlong(v) : 0ull;
  const unsigned           hi = __reduce_max_sync(grp, (unsigned)(b >> 32));
  const unsigned           lo = __reduce_max_sync(grp, (unsigned)(b >> 32) == hi ? (unsigned)b : 0u);
  if ((int)(threadIdx.x & 31u) == __ffs(grp) - 1 && (hi | lo) != 0u)
    atomicMax(reinterpret_cast<unsigned long long *>(base + ins), ((unsigned long long)hi << 32) | lo);
}

// ---------------------------------------------------------------------------
// Stiffened-gas mixture EOS (restated, see the oracle for the formulas)
// ---------------------------------------------------------------------------
__device__ __forceinline__ double
eosS(const PhysParams & P, double a0, double a1)
{
  return a0 * P.xi[0] + a1 * P.xi[1];
}
__device__ __forceinline__ double
eosPI(const PhysParams & P, double a0, double a1)
{
  return a0 * P.gpx[0] + a1 * P.gpx[1];
}
__device__ __forceinline__ double
sound_speed_d(const PhysParams & P, double rho, double p, double a0, double a1)
{
  const double S = eosS(P, a0, a1);
  const double c2 = (p * (S + 1.0) + eosPI(P, a0, a1)) / (rho * S);
  return sqrt(fmax(c2, 0.0));
}

__device__ __forceinline__ float
sound_speed_f(float xi0, float xi1, float gp0, float gp1, float rho, float p, float a0)
{
  const float a1 = 1.0f - a0;
  const float S = a0 * xi0 + a1 * xi1;
  const float PI = a0 * gp0 + a1 * gp1;
  const float c2 = __fdividef(p * (S + 1.0f) + PI, rho * S);
  return sqrtf(fmaxf(c2, 0.0f));
}

// ---------------------------------------------------------------------------
// exp and log without the CUDA math library, the same algorithms as the
// oracle (IEEE +, -, *, / and exact frexp/ldexp only, so the FP64 path stays
// bit-reproducible against it):
//   exp: Cody-Waite reduction x = k ln2 + r, |r| <= ln2/2, degree-16 Taylor
//        polynomial of expm1(r), then 2^k (1 + expm1(r));
//   log: x = m 2^e with m in [sqrt(1/2), sqrt(2)), log m = 2 atanh(t),
//        t = (m-1)/(m+1), odd series to t^25, plus e ln2 (split hi/lo).
// ---------------------------------------------------------------------------
__device__ __forceinline__ double
expm1_small_d(double r)
{
  const double c[17] = { 1.0,
                         1.0,
                         0.5,
                         0.16666666666666666,
                         0.041666666666666664,
                         0.008333333333333333,
                         0.001388888888888889,
                         0.0001984126984126984,
                         2.48015873015873e-05,
                         2.7557319223985893e-06,
                         2.755731922398589e-07,
                         2.505210838544172e-08,
                         2.08767569878681e-09,
                         1.6059043836821613e-10,
                         1.1470745597729725e-11,
                         7.647163731819816e-13,
                         4.779477332387385e-14 };
  double       p = c[16];
#pragma unroll
  for (int k = 15; k >= 1; --k)
    p = p * r + c[k];
  return p * r;
}

__device__ __forceinline__ double
exp_d(double x)
{
  if (x != x)
    return x;
  if (x < -745.5)
    return 0.0;
  if (x > 709.7)
    return __longlong_as_double(0x7ff0000000000000LL);
  const double k = floor(x * 1.4426950408889634 + 0.5);
  const double r = (x - k * 0.6931471824645996) - k * -1.904654299957768e-09;
  return ldexp(expm1_small_d(r) + 1.0, (int)k);
}

__device__ __forceinline__ double
log_d(double x)
{
  int    e;
  double m = frexp(x, &e);
  if (m < 0.7071067811865476)
  {
    m = m * 2.0;
    e = e - 1;
  }
  const double t = (m - 1.0) / (m + 1.0);
  const double t2 = t * t;
  const double c[13] = { 1.0 / 1.0,  1.0 / 3.0,  1.0 / 5.0,  1.0 / 7.0,  1.0 / 9.0,  1.0 / 11.0, 1.0 / 13.0,
                         1.0 / 15.0, 1.0 / 17.0, 1.0 / 19.0, 1.0 / 21.0, 1.0 / 23.0, 1.0 / 25.0 };
  double       sr = c[12];
#pragma unroll
  for (int j = 11; j >= 0; --j)
    sr = sr * t2 + c[j];
  const double de = (double)e;
  return (2.0 * t * sr + de * 0.6931471824645996) + de * -1.904654299957768e-09;
}

// ---------------------------------------------------------------------------
// Mie-Grueneisen material laws (restated from their published forms; the
// reference's core::eos::MieGruneisenMixture is external).  Each law is
// written p = G(rho) rho e + f(rho) and gives G, dG/drho, f and df/drho:
//   stiffened gas  G = gamma - 1, f = -gamma pinf
//   JWL (Lee, Hornig & Kury 1968), x_i = R_i rho0 / rho:
//       G = Gamma0, f = sum_i A_i (1 - Gamma0/x_i) exp(-x_i) - Gamma0 rho e0
//   SHOCKWAVE (Grueneisen form with a cubic Us-up Hugoniot fit, Steinberg),
//   mu = rho/rho0 - 1:  G rho = (Gamma0 + b mu) rho0,
//       f = pc - (Gamma0 + b mu) rho0 e0,
//       pc = rho0 c0^2 mu N / D^2 (mu > 0), rho0 c0^2 mu (mu <= 0),
//       N = 1 + (1 - Gamma0/2) mu - b mu^2/2,
//       D = 1 - (s1-1) mu - s2 mu^2/(mu+1) - s3 mu^3/(mu+1)^2
//   SHOCKWAVE2 (linear Us-up Hugoniot as the reference curve), eta = 1 - rho0/rho:
//       pH = p0 + rho0 c0^2 eta / (1 - s eta)^2, eH = e0 + (pH + p0) eta / (2 rho0),
//       G = Gamma0 (rho0/rho)^alpha, f = pH - G rho eH
// Mixture under pressure equilibrium (Allaire, Clerc & Kokh 2002), material
// densities rho_k = (alpha rho)_k / alpha_k (rho0_k when alpha_k = 0), xi_k = 1/G_k:
//   S = sum a_k xi_k, PI = -sum a_k xi_k f_k:  p = (rho e - PI)/S, rho e = p S + PI
//   rho c^2 S = sum a_k xi_k rho_k c_k^2 = p C1 + C0 with
//   rho_k c_k^2 = (1 + rho_k G'_k xi_k)(p - f_k) + rho_k f'_k + G_k p,
//   C1 = sum a_k (xi_k (1 + rho_k G'_k xi_k) + 1),
//   C0 = sum a_k (xi_k rho_k f'_k - xi_k (1 + rho_k G'_k xi_k) f_k).
// With stiffened gases only these reduce to the forms above (S, PI and
// c^2 = (p (S+1) + PI)/(rho S)), which the code keeps for that case.
// ---------------------------------------------------------------------------
constexpr int EOS_STIFFENED = 0, EOS_JWL = 1, EOS_SHOCKWAVE = 2, EOS_SHOCKWAVE2 = 3;

__device__ __forceinline__ void
mg_law(const PhysParams & P, int k, double rho, double & G, double & dG, double & f, double & df)
{
  const double * c = P.mg[k];
  const int      kind = P.eos_kind[k];
  if (kind == EOS_JWL)
  {
    const double rho0 = c[0], w = c[1], A1 = c[2], A2 = c[3], R1 = c[4], R2 = c[5], e0 = c[6];
    const double x1 = R1 * rho0 / rho, x2 = R2 * rho0 / rho;
    const double E1 = exp_d(-x1), E2 = exp_d(-x2);
    G = w;
    dG = 0.0;
    f = A1 * (1.0 - w / x1) * E1 + A2 * (1.0 - w / x2) * E2 - w * rho * e0;
    df = (A1 * E1 * (x1 - w - w / x1) + A2 * E2 * (x2 - w - w / x2)) / rho - w * e0;
  }
  else if (kind == EOS_SHOCKWAVE)
  {
    const double rho0 = c[0], g0 = c[1], c0 = c[2], s1 = c[3], s2 = c[4], s3 = c[5], b = c[6], e0 = c[7];
    const double mu = rho / rho0 - 1.0;
    const double K = rho0 * c0 * c0;
    double       pc, dpc;
    if (mu > 0.0)
    {
      const double m1 = mu + 1.0;
      const double N = 1.0 + (1.0 - 0.5 * g0) * mu - 0.5 * b * mu * mu;
      const double Np = (1.0 - 0.5 * g0) - b * mu;
      const double D = 1.0 - (s1 - 1.0) * mu - s2 * mu * mu / m1 - s3 * mu * mu * mu / (m1 * m1);
      const double Dp = -(s1 - 1.0) - s2 * (mu * mu + 2.0 * mu) / (m1 * m1) - s3 * (mu * mu * mu + 3.0 * mu * mu) / (m1 * m1 * m1);
      pc = K * mu * N / (D * D);
      dpc = K * ((N + mu * Np) / (D * D) - 2.0 * mu * N * Dp / (D * D * D));
    }
    else
    {
      pc = K * mu;
      dpc = K;
    }
    const double gr = (g0 + b * mu) * rho0;
    G = gr / rho;
    dG = b / rho - G / rho;
    f = pc - gr * e0;
    df = dpc / rho0 - b * e0;
  }
  else if (kind == EOS_SHOCKWAVE2)
  {
    const double rho0 = c[0], g0 = c[1], c0 = c[2], s = c[3], al = c[4], e0 = c[5], p0 = c[6];
    const double eta = 1.0 - rho0 / rho;
    const double w = 1.0 - s * eta;
    const double K = rho0 * c0 * c0;
    const double pH = p0 + K * eta / (w * w);
    const double eH = e0 + (pH + p0) * eta / (2.0 * rho0);
    const double v = rho0 / rho;
    double       gp;
    if (al == 1.0)
      gp = v;
    else if (al == 0.0)
      gp = 1.0;
    else
      gp = exp_d(al * log_d(v));
    G = g0 * gp;
    dG = -al * G / rho;
    const double dpH = K * (1.0 + s * eta) / (w * w * w);
    const double deH = (dpH * eta + pH + p0) / (2.0 * rho0);
    const double deta = rho0 / (rho * rho);
    f = pH - G * rho * eH;
    df = dpH * deta - (dG * rho + G) * eH - G * rho * deH * deta;
  }
  else
  {
    G = P.gamma[k] - 1.0;
    dG = 0.0;
    f = -P.gamma[k] * P.pinf[k];
    df = 0.0;
  }
}

// material density of the mixture rules (the law's reference density when
// the material is absent)
__device__ __forceinline__ double
mg_material_density(const PhysParams & P, int k, double a, double ar)
{
  return a > 0.0 ? fmax(ar / a, P.smallr) : P.mg_rho0[k];
}

// S, PI, C1, C0 of the mixture rules above for volume fractions a0, a1 and
// partial densities ar0, ar1
__device__ __forceinline__ void
mg_mixture(const PhysParams & P, double a0, double a1, double ar0, double ar1, double & S, double & PI, double & C1, double & C0)
{
  S = 0.0;
  PI = 0.0;
  C1 = 0.0;
  C0 = 0.0;
#pragma unroll
  for (int k = 0; k < 2; ++k)
  {
    const double a = k == 0 ? a0 : a1;
    const double rho = mg_material_density(P, k, a, k == 0 ? ar0 : ar1);
    double       G, dG, f, df;
    mg_law(P, k, rho, G, dG, f, df);
    const double xi = 1.0 / G;
    const double h = xi * (1.0 + rho * dG * xi);
    S = S + a * xi;
    PI = PI - a * xi * f;
    C1 = C1 + a * (h + 1.0);
    C0 = C0 + a * (xi * rho * df - h * f);
  }
}

// bulk modulus rho_k c_k^2 of material k at pressure p (Miller-Puckett)
__device__ __forceinline__ double
mg_bulk_modulus(const PhysParams & P, int k, double a, double ar, double p)
{
  const double rho = mg_material_density(P, k, a, ar);
  double       G, dG, f, df;
  mg_law(P, k, rho, G, dG, f, df);
  return (1.0 + rho * dG / G) * (p - f) + rho * df + G * p;
}

// mixture sound speed for either path: the stiffened-gas form, or the
// general one from the partial densities
__device__ __forceinline__ double
sound_speed_mix(const PhysParams & P, double rho, double p, double a0, double a1, double ar0, double ar1)
{
  if (!P.mg_any)
    return sound_speed_d(P, rho, p, a0, a1);
  double S, PI, C1, C0;
  mg_mixture(P, a0, a1, ar0, ar1, S, PI, C1, C0);
  const double c2 = (p * C1 + C0) / (rho * S);
  return sqrt(fmax(c2, 0.0));
}

// ---------------------------------------------------------------------------
// conservative (FP64) -> primitive, models/utils.h:200-250 (computePrimitives)
// q[] receives the shared-memory components (r0 r1 p u v (w) alpha0).
// Returns the mixture sound speed c; ux/uy/uz are the velocities.
// ---------------------------------------------------------------------------
template <int DIM>
__device__ __forceinline__ double
prim_fp64(const double * u, double * q, const PhysParams & P)
{
  using H = V<DIM>;
  const double d = fmax(u[H::ID], P.smallr);
  const double ux = u[H::IU] / d;
  const double uy = u[H::IV] / d;
  double       ekin;
  double       uz = 0.0;
  if constexpr (DIM == 2)
    ekin = 0.5 * (ux * ux + uy * uy);
  else
  {
    uz = u[H::IW] / d;
    ekin = 0.5 * (ux * ux + uy * uy + uz * uz);
  }
  const double eint = u[H::IE] / d - ekin;
  const double a0u = u[H::IA0];
  double       p;
  if (!P.mg_any)
    p = (d * eint - eosPI(P, a0u, 1.0 - a0u)) / eosS(P, a0u, 1.0 - a0u);
  else
  {
    double S, PI, C1, C0;
    mg_mixture(P, a0u, 1.0 - a0u, u[H::IAD0], u[H::IAD1], S, PI, C1, C0);
    p = (d * eint - PI) / S;
  }
  double       a0 = fmax(0.0, fmin(1.0, a0u));
  double       r0 = u[H::IAD0], r1 = u[H::IAD1];
  const double eps = 1e-12;
  if (r0 < eps)
    r0 = 0.0;
  if (r1 < eps)
    r1 = 0.0;
  if (a0 < eps)
    a0 = 0.0;
  if (a0 > 1.0 - eps)
    a0 = 1.0;
  q[H::QR0] = r0;
  q[H::QR1] = r1;
  q[H::QP] = p;
  q[H::QU] = ux;
  q[H::QV] = uy;
  if constexpr (DIM == 3)
    q[H::QW] = uz;
  q[H::QA] = a0;
  return sound_speed_mix(P, d, p, a0, 1.0 - a0, r0, r1);
}

// Volume-fraction source-term factors st_k of get_source_term_factor
// (ReadFluxesAndConservativeUpdateFunctor.h:412-443): 1 for ALLAIRE_KOKH;
// MILLER_PUCKETT: 1 - Kbar / K_k with K_k = gamma_k (p + pinf_k) and
// 1/Kbar = a0/K0 + a1/K1 (stiffened gas, restated), p from
// compute_mixture_pressure (models/utils.h:160-185).  FP64, reference order.
template <int DIM>
__device__ __forceinline__ void
source_factors_fp64(const double * u, const PhysParams & P, double & st0, double & st1)
{
  using H = V<DIM>;
  if (P.source_term != 1)
  {
    st0 = st1 = 1.0;
    return;
  }
  const double d = fmax(u[H::IAD0] + u[H::IAD1], P.smallr);
  const double dd = fmax(u[H::ID], P.smallr);
  const double ux = u[H::IU] / dd, uy = u[H::IV] / dd;
  double       ekin;
  if constexpr (DIM == 2)
    ekin = 0.5 * (ux * ux + uy * uy);
  else
  {
    const double uz = u[H::IW] / dd;
    ekin = 0.5 * (ux * ux + uy * uy + uz * uz);
  }
  const double eint = u[H::IE] / d - ekin;
  const double a0 = u[H::IA0];
  double       p, K0, K1;
  if (!P.mg_any)
  {
    p = (d * eint - eosPI(P, a0, 1 - a0)) / eosS(P, a0, 1 - a0);
    K0 = P.gamma[0] * (p + P.pinf[0]);
    K1 = P.gamma[1] * (p + P.pinf[1]);
  }
  else
  {
    double S, PI, C1, C0;
    mg_mixture(P, a0, 1 - a0, u[H::IAD0], u[H::IAD1], S, PI, C1, C0);
    p = (d * eint - PI) / S;
    K0 = mg_bulk_modulus(P, 0, u[H::IA0], u[H::IAD0], p);
    K1 = mg_bulk_modulus(P, 1, u[H::IA1], u[H::IAD1], p);
  }
  const double kbar = 1.0 / (u[H::IA0] / K0 + u[H::IA1] / K1);
  st0 = 1.0 - kbar / K0;
  st1 = 1.0 - kbar / K1;
}

// scheme/ComputeLimitedSlopesFunctor.cpp:116-137
template <typename R>
__device__ __forceinline__ R
slope_scalar(R q, R qPlus, R qMinus, R slope_type)
{
  R dq = R(0);
  if (slope_type == R(1) || slope_type == R(2))
  {
    const R dlft = slope_type * (q - qMinus);
    const R drgt = slope_type * (qPlus - q);
    const R dcen = R(0.5) * (qPlus - qMinus);
    const R dsgn = (dcen >= R(0)) ? R(1) : R(-1);
    const R slop = fmin(fabs(dlft), fabs(drgt));
    const R dlim = (dlft * drgt) <= R(0) ? R(0) : slop;
    dq = dsgn * fmin(dlim, fabs(dcen));
  }
  return dq;
}

// slope_scalar of two independent (q, qPlus, qMinus) triples at once (FP32):
// its differences and products on the packed FP32x2 pipe of sm_100+, each
// lane rounded as the scalar operation is; |.|, min and the selects per lane
__device__ __forceinline__ float2
slope_pair(float2 q, float2 qPlus, float2 qMinus, float slope_type)
{
  if (!(slope_type == 1.0f || slope_type == 2.0f))
    return make_float2(0.0f, 0.0f);
  const float2 st = make_float2(slope_type, slope_type);
  const float2 dlft = __fmul2_rn(st, __ffma2_rn(qMinus, make_float2(-1.0f, -1.0f), q));
  const float2 drgt = __fmul2_rn(st, __ffma2_rn(q, make_float2(-1.0f, -1.0f), qPlus));
  const float2 dcen = __fmul2_rn(make_float2(0.5f, 0.5f), __ffma2_rn(qMinus, make_float2(-1.0f, -1.0f), qPlus));
  const float2 pr = __fmul2_rn(dlft, drgt);
  const float2 sg = make_float2(dcen.x >= 0.0f ? 1.0f : -1.0f, dcen.y >= 0.0f ? 1.0f : -1.0f);
  const float2 m = make_float2(fminf(pr.x <= 0.0f ? 0.0f : fminf(fabsf(dlft.x), fabsf(drgt.x)), fabsf(dcen.x)),
                               fminf(pr.y <= 0.0f ? 0.0f : fminf(fabsf(dlft.y), fabsf(drgt.y)), fabsf(dcen.y)));
  return __fmul2_rn(sg, m);
}

// ---------------------------------------------------------------------------
// tanh: same algorithm as the oracle (Cody-Waite reduced Taylor expm1),
// FP64, bit-reproducible on IEEE hardware without contraction.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double
tanh_d(double x)
{
  if (x != x)
    return x;
  const double ax = fabs(x);
  double       t;
  if (ax > 22.0)
    t = 1.0;
  else
  {
    const double y = 2.0 * ax;
    double       em;
    if (y < 0.34657359027997264)
      em = expm1_small_d(y);
    else
    {
      const double k = floor(y * 1.4426950408889634 + 0.5);
      const double r = (y - k * 0.6931471824645996) - k * -1.904654299957768e-09;
      em = ldexp(expm1_small_d(r) + 1.0, (int)k) - 1.0;
    }
    t = em / (em + 2.0);
  }
  return x < 0.0 ? -t : t;
}

// ---------------------------------------------------------------------------
// HLLC, models/RiemannSolvers.h:57-262, FP64 (reference order).
// ql/qr: components r0 r1 p u v (w) alpha0 (normal velocity in u).
// out: FR0 FR1 FA0 FA1 FE FU FV (FW) FUS, NOT yet scaled by dt/dx.
// ---------------------------------------------------------------------------
template <int DIM>
__device__ __forceinline__ void
hllc_fp64(const double * ql, const double * qr, const PhysParams & P, double * f)
{
  using H = V<DIM>;
  const double smallr = P.smallr, smallp = P.smallp, smallc = P.smallc;
  const double al = ql[H::QA], ar = qr[H::QA];
  double       Sl, PIl, Sr, PIr, C1l, C0l, C1r, C0r;
  if (!P.mg_any)
  {
    Sl = eosS(P, al, 1 - al);
    PIl = eosPI(P, al, 1 - al);
    Sr = eosS(P, ar, 1 - ar);
    PIr = eosPI(P, ar, 1 - ar);
    C1l = Sl + 1.0;
    C0l = PIl;
    C1r = Sr + 1.0;
    C0r = PIr;
  }
  else
  {
    mg_mixture(P, al, 1 - al, ql[H::QR0], ql[H::QR1], Sl, PIl, C1l, C0l);
    mg_mixture(P, ar, 1 - ar, qr[H::QR0], qr[H::QR1], Sr, PIr, C1r, C0r);
  }

  const double rl = fmax(ql[H::QR0] + ql[H::QR1], smallr);
  double       pl = fmax(ql[H::QP], rl * smallp);
  const double ul = ql[H::QU];
  const double eintl = (pl * Sl + PIl) / rl;
  pl = (rl * eintl - PIl) / Sl;
  double ecinl = 0.5 * rl * ul * ul;
  ecinl += 0.5 * rl * ql[H::QV] * ql[H::QV];
  if constexpr (DIM == 3)
    ecinl += 0.5 * rl * ql[H::QW] * ql[H::QW];
  const double cl2 = (pl * C1l + C0l) / (rl * Sl);
  const double cl = sqrt(fmax(cl2, 0.0));
  const double etotl = rl * eintl + ecinl;
  const double ptotl = pl;

  const double rr = fmax(qr[H::QR0] + qr[H::QR1], smallr);
  double       pr = fmax(qr[H::QP], rr * smallp);
  const double ur = qr[H::QU];
  const double eintr = (pr * Sr + PIr) / rr;
  pr = (rr * eintr - PIr) / Sr;
  double ecinr = 0.5 * rr * ur * ur;
  ecinr += 0.5 * rr * qr[H::QV] * qr[H::QV];
  if constexpr (DIM == 3)
    ecinr += 0.5 * rr * qr[H::QW] * qr[H::QW];
  const double cr2 = (pr * C1r + C0r) / (rr * Sr);
  const double cr = sqrt(fmax(cr2, 0.0));
  const double etotr = rr * eintr + ecinr;
  const double ptotr = pr;

  const double cfastl = sqrt(fmax(cl * cl, smallc * smallc));
  const double cfastr = sqrt(fmax(cr * cr, smallc * smallc));
  const double SL = fmin(ul, ur) - fmax(cfastl, cfastr);
  const double SR = fmax(ul, ur) + fmax(cfastl, cfastr);

  const double rcl = rl * (ul - SL);
  const double rcr = rr * (SR - ur);
  const double us = (rcr * ur + rcl * ul + (ptotl - ptotr)) / (rcr + rcl);
  const double ptotstar = (rcr * ptotl + rcl * ptotr + rcl * rcr * (ul - ur)) / (rcr + rcl);

  double ro, ro_0, ro_1, uo, ptoto, etoto;
  if (SL > 0.0)
  {
    ro_0 = ql[H::QR0];
    ro_1 = ql[H::QR1];
    ro = rl;
    uo = ul;
    ptoto = ptotl;
    etoto = etotl;
  }
  else if (us > 0.0)
  {
    const double factorL = (SL - ul) / (SL - us);
    ro_0 = ql[H::QR0] * factorL;
    ro_1 = ql[H::QR1] * factorL;
    ro = rl * factorL;
    uo = us;
    ptoto = ptotstar;
    etoto = ((SL - ul) * etotl - ptotl * ul + ptotstar * us) / (SL - us);
  }
  else if (SR > 0.0)
  {
    const double factorR = (SR - ur) / (SR - us);
    ro_0 = qr[H::QR0] * factorR;
    ro_1 = qr[H::QR1] * factorR;
    ro = rr * factorR;
    uo = us;
    ptoto = ptotstar;
    etoto = ((SR - ur) * etotr - ptotr * ur + ptotstar * us) / (SR - us);
  }
  else
  {
    ro_0 = qr[H::QR0];
    ro_1 = qr[H::QR1];
    ro = rr;
    uo = ur;
    ptoto = ptotr;
    etoto = etotr;
  }
  const double fid = (ro_0 + ro_1) * uo;
  f[H::FR0] = ro_0 * uo;
  f[H::FR1] = ro_1 * uo;
  f[H::FU] = ro * uo * uo + ptoto;
  f[H::FE] = (etoto + ptoto) * uo;
  f[H::FV] = (fid > 0.0) ? fid * ql[H::QV] : fid * qr[H::QV];
  if constexpr (DIM == 3)
    f[H::FW] = (fid > 0.0) ? fid * ql[H::QW] : fid * qr[H::QW];
  const double phi0 = (fid > 0.0) ? al : ar;
  const double phi1 = 1.0 - phi0;
  f[H::FA0] = uo * phi0;
  f[H::FA1] = uo * phi1;
  f[H::FUS] = uo;
}

// HLLC in FP32.  The p -> e -> p round trip of the reference is an identity
// in exact arithmetic and is dropped here (in FP32 it would cancel the
// stiffened-gas constant against p S).
// ---------------------------------------------------------------------------
// FP32 forms of the Mie-Grueneisen laws and mixture rules above (the
// FP32-bulk path: fast-math exp and log), same formulas and order
// ---------------------------------------------------------------------------
__device__ __forceinline__ void
mg_law_f(const PhysParams & P, int k, float rho, float & G, float & dG, float & f, float & df)
{
  const float * c = P.f_mg[k];
  const int     kind = P.eos_kind[k];
  if (kind == EOS_JWL)
  {
    const float rho0 = c[0], w = c[1], A1 = c[2], A2 = c[3], R1 = c[4], R2 = c[5], e0 = c[6];
    const float irho = __frcp_rn(rho);
    const float x1 = R1 * rho0 * irho, x2 = R2 * rho0 * irho;
    const float E1 = __expf(-x1), E2 = __expf(-x2);
    G = w;
    dG = 0.0f;
    f = A1 * (1.0f - __fdividef(w, x1)) * E1 + A2 * (1.0f - __fdividef(w, x2)) * E2 - w * rho * e0;
    df = (A1 * E1 * (x1 - w - __fdividef(w, x1)) + A2 * E2 * (x2 - w - __fdividef(w, x2))) * irho - w * e0;
  }
  else if (kind == EOS_SHOCKWAVE)
  {
    const float rho0 = c[0], g0 = c[1], c0 = c[2], s1 = c[3], s2 = c[4], s3 = c[5], b = c[6], e0 = c[7];
    const float mu = __fdividef(rho, rho0) - 1.0f;
    const float K = rho0 * c0 * c0;
    float       pc, dpc;
    if (mu > 0.0f)
    {
      const float m1 = mu + 1.0f;
      const float im1 = __frcp_rn(m1);
      const float N = 1.0f + (1.0f - 0.5f * g0) * mu - 0.5f * b * mu * mu;
      const float Np = (1.0f - 0.5f * g0) - b * mu;
      const float D = 1.0f - (s1 - 1.0f) * mu - s2 * mu * mu * im1 - s3 * mu * mu * mu * im1 * im1;
      const float Dp = -(s1 - 1.0f) - s2 * (mu * mu + 2.0f * mu) * im1 * im1 - s3 * (mu * mu * mu + 3.0f * mu * mu) * im1 * im1 * im1;
      const float iD = __frcp_rn(D);
      pc = K * mu * N * iD * iD;
      dpc = K * ((N + mu * Np) * iD * iD - 2.0f * mu * N * Dp * iD * iD * iD);
    }
    else
    {
      pc = K * mu;
      dpc = K;
    }
    const float gr = (g0 + b * mu) * rho0;
    const float irho = __frcp_rn(rho);
    G = gr * irho;
    dG = (b - G) * irho;
    f = pc - gr * e0;
    df = __fdividef(dpc, rho0) - b * e0;
  }
  else if (kind == EOS_SHOCKWAVE2)
  {
    const float rho0 = c[0], g0 = c[1], c0 = c[2], sl = c[3], al = c[4], e0 = c[5], p0 = c[6];
    const float irho = __frcp_rn(rho);
    const float v = rho0 * irho;
    const float eta = 1.0f - v;
    const float w = 1.0f - sl * eta;
    const float iw = __frcp_rn(w);
    const float K = rho0 * c0 * c0;
    const float pH = p0 + K * eta * iw * iw;
    const float eH = e0 + __fdividef((pH + p0) * eta, 2.0f * rho0);
    const float gp = al == 1.0f ? v : (al == 0.0f ? 1.0f : __expf(al * __logf(v)));
    G = g0 * gp;
    dG = -al * G * irho;
    const float dpH = K * (1.0f + sl * eta) * iw * iw * iw;
    const float deH = __fdividef(dpH * eta + pH + p0, 2.0f * rho0);
    const float deta = v * irho;
    f = pH - G * rho * eH;
    df = dpH * deta - (dG * rho + G) * eH - G * rho * deH * deta;
  }
  else
  {
    G = P.f_gm1[k];
    dG = 0.0f;
    f = -P.f_gpinf[k];
    df = 0.0f;
  }
}

__device__ __forceinline__ float
mg_material_density_f(const PhysParams & P, int k, float a, float ar)
{
  return a > 0.0f ? fmaxf(__fdividef(ar, a), P.f_smallr) : P.f_mg_rho0[k];
}

__device__ __forceinline__ void
mg_mixture_f(const PhysParams & P, float a0, float a1, float ar0, float ar1, float & S, float & PI, float & C1, float & C0)
{
  S = 0.0f;
  PI = 0.0f;
  C1 = 0.0f;
  C0 = 0.0f;
#pragma unroll
  for (int k = 0; k < 2; ++k)
  {
    const float a = k == 0 ? a0 : a1;
    const float rho = mg_material_density_f(P, k, a, k == 0 ? ar0 : ar1);
    float       G, dG, f, df;
    mg_law_f(P, k, rho, G, dG, f, df);
    const float xi = __frcp_rn(G);
    const float h = xi * (1.0f + rho * dG * xi);
    S = S + a * xi;
    PI = PI - a * xi * f;
    C1 = C1 + a * (h + 1.0f);
    C0 = C0 + a * (xi * rho * df - h * f);
  }
}

__device__ __forceinline__ float
mg_bulk_modulus_f(const PhysParams & P, int k, float a, float ar, float p)
{
  const float rho = mg_material_density_f(P, k, a, ar);
  float       G, dG, f, df;
  mg_law_f(P, k, rho, G, dG, f, df);
  return (1.0f + __fdividef(rho * dG, G)) * (p - f) + rho * df + G * p;
}

// FP32 mixture sound speed: eosk 2 takes the Mie-Grueneisen mixture rules
// from the partial densities, otherwise the stiffened-gas form
__device__ __forceinline__ float
sound_speed_eos(const PhysParams & P, int eosk, float rho, float p, float a0, float r0, float r1)
{
  if (eosk == 2)
  {
    float S, PI, C1, C0;
    mg_mixture_f(P, a0, 1.0f - a0, r0, r1, S, PI, C1, C0);
    return sqrtf(fmaxf(__fdividef(p * C1 + C0, rho * S), 0.0f));
  }
  return sound_speed_f(P.f_xi[0], P.f_xi[1], P.f_gpx[0], P.f_gpx[1], rho, p, a0);
}

template <int DIM>
__device__ __forceinline__ void
hllc_fp32(const float * ql, const float * qr, float xi0, float xi1, float gp0, float gp1, float smallr, float smallp, float smallc, float * f,
          const PhysParams * Pmg = nullptr)
{
  using H = V<DIM>;
  const float al = ql[H::QA], ar = qr[H::QA];
  // mixture rules of each side: S, PI and the sound-speed coefficients C1, C0
  // (rho c^2 S = p C1 + C0; stiffened gases: C1 = S + 1, C0 = PI)
  float Sl, PIl, C1l, C0l, Sr, PIr, C1r, C0r;
  if (Pmg)
  {
    mg_mixture_f(*Pmg, al, 1.0f - al, ql[H::QR0], ql[H::QR1], Sl, PIl, C1l, C0l);
    mg_mixture_f(*Pmg, ar, 1.0f - ar, qr[H::QR0], qr[H::QR1], Sr, PIr, C1r, C0r);
  }
  else
  {
    Sl = al * xi0 + (1.0f - al) * xi1;
    PIl = al * gp0 + (1.0f - al) * gp1;
    Sr = ar * xi0 + (1.0f - ar) * xi1;
    PIr = ar * gp0 + (1.0f - ar) * gp1;
    C1l = Sl + 1.0f;
    C0l = PIl;
    C1r = Sr + 1.0f;
    C0r = PIr;
  }

  const float rl = fmaxf(ql[H::QR0] + ql[H::QR1], smallr);
  const float pl = fmaxf(ql[H::QP], rl * smallp);
  const float ul = ql[H::QU];
  float       k2l = ul * ul + ql[H::QV] * ql[H::QV];
  if constexpr (DIM == 3)
    k2l += ql[H::QW] * ql[H::QW];
  const float rel = pl * Sl + PIl; // rho e
  const float cl = sqrtf(fmaxf(__fdividef(pl * C1l + C0l, rl * Sl), 0.0f));
  const float etotl = rel + 0.5f * rl * k2l;

  const float rr = fmaxf(qr[H::QR0] + qr[H::QR1], smallr);
  const float pr = fmaxf(qr[H::QP], rr * smallp);
  const float ur = qr[H::QU];
  float       k2r = ur * ur + qr[H::QV] * qr[H::QV];
  if constexpr (DIM == 3)
    k2r += qr[H::QW] * qr[H::QW];
  const float rer = pr * Sr + PIr;
  const float cr = sqrtf(fmaxf(__fdividef(pr * C1r + C0r, rr * Sr), 0.0f));
  const float etotr = rer + 0.5f * rr * k2r;

  const float cf = fmaxf(fmaxf(cl, smallc), fmaxf(cr, smallc));
  const float SL = fminf(ul, ur) - cf;
  const float SR = fmaxf(ul, ur) + cf;
  const float rcl = rl * (ul - SL);
  const float rcr = rr * (SR - ur);
  const float inv = __frcp_rn(rcr + rcl);
  const float us = (rcr * ur + rcl * ul + (pl - pr)) * inv;
  const float ps = (rcr * pl + rcl * pr + rcl * rcr * (ul - ur)) * inv;

  float ro_0, ro_1, ro, uo, po, eo;
  if (SL > 0.0f)
  {
    ro_0 = ql[H::QR0];
    ro_1 = ql[H::QR1];
    ro = rl;
    uo = ul;
    po = pl;
    eo = etotl;
  }
  else if (us > 0.0f)
  {
    const float ifl = __frcp_rn(SL - us);
    const float fl = (SL - ul) * ifl;
    ro_0 = ql[H::QR0] * fl;
    ro_1 = ql[H::QR1] * fl;
    ro = rl * fl;
    uo = us;
    po = ps;
    eo = ((SL - ul) * etotl - pl * ul + ps * us) * ifl;
  }
  else if (SR > 0.0f)
  {
    const float ifr = __frcp_rn(SR - us);
    const float fr = (SR - ur) * ifr;
    ro_0 = qr[H::QR0] * fr;
    ro_1 = qr[H::QR1] * fr;
    ro = rr * fr;
    uo = us;
    po = ps;
    eo = ((SR - ur) * etotr - pr * ur + ps * us) * ifr;
  }
  else
  {
    ro_0 = qr[H::QR0];
    ro_1 = qr[H::QR1];
    ro = rr;
    uo = ur;
    po = pr;
    eo = etotr;
  }
  const float fid = (ro_0 + ro_1) * uo;
  f[H::FR0] = ro_0 * uo;
  f[H::FR1] = ro_1 * uo;
  f[H::FU] = ro * uo * uo + po;
  f[H::FE] = (eo + po) * uo;
  f[H::FV] = (fid > 0.0f) ? fid * ql[H::QV] : fid * qr[H::QV];
  if constexpr (DIM == 3)
    f[H::FW] = (fid > 0.0f) ? fid * ql[H::QW] : fid * qr[H::QW];
  const float phi0 = (fid > 0.0f) ? al : ar;
  f[H::FA0] = uo * phi0;
  f[H::FA1] = uo * (1.0f - phi0);
  f[H::FUS] = uo;
}


// ---------------------------------------------------------------------------
// helpers of the FP32-bulk path.  On GB300 the FP64 pipe issues 1.6
// instructions/clk/SM against 115 for FP32, and float -> double conversion
// runs on the FP64 pipe, so the mixed path keeps FP64 to the adds into the
// stored state, the renormalisation and the stiffened-gas pressure
// numerator, and does everything else on the FP32 and integer pipes.
// ---------------------------------------------------------------------------

// double -> float on the integer pipe (the hardware conversion issues on the
// FP64 pipe, 1.9 per clock per SM on GB300): the exponent and the top 23
// mantissa bits move into float position with one funnel shift, the exponent
// is rebiased by flipping its top bit (e - 896 mod 256), the mantissa is
// truncated; magnitudes below FLT_MIN (zeros included) give a signed zero.
// Only for finite values of the state (far below FLT_MAX): a NaN or an
// infinity gives a finite float.  It converts the cell's own values, whose
// non-finiteness the FP64 adds into the new state carry to the status word.
__device__ __forceinline__ float
d2f_fast(double x)
{
  const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
  const unsigned m = __funnelshift_l(lo, hi, 3); // e[8:0] m[51:29]
  const unsigned f = (((m & 0x7FFFFFFFu) ^ 0x40000000u)) | (hi & 0x80000000u);
  return __uint_as_float(((hi & 0x7FFFFFFFu) < (897u << 20)) ? (hi & 0x80000000u) : f);
}

// The same conversion keeping non-finite values non-finite, for states that
// enter the fluxes (the primitive conversion of the block and its halo): a
// double of magnitude 2^128 or more, an infinity or a NaN gives a float with
// an all-ones exponent and the top 23 mantissa bits, i.e. infinity stays
// infinity and a NaN whose top mantissa bits are not all zero (every NaN that
// arithmetic produces) stays NaN.  Two integer instructions more than
// d2f_fast (a compare and a select).
__device__ __forceinline__ float
d2f_nan(double x)
{
  const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
  const unsigned ah = hi & 0x7FFFFFFFu, sgn = hi & 0x80000000u;
  const unsigned m = __funnelshift_l(lo, hi, 3); // e[8:0] m[51:29]
  unsigned       f = (((m & 0x7FFFFFFFu) ^ 0x40000000u)) | sgn;
  f = ah < (897u << 20) ? sgn : f;
  f = ah >= (1151u << 20) ? ((m & 0x007FFFFFu) | 0x7F800000u | sgn) : f;
  return __uint_as_float(f);
}

// exact float -> double on the integer pipe (float denormals read as zero,
// as the fast-math build flushes them anyway)
__device__ __forceinline__ double
f2d_exact(float f)
{
  const unsigned b = __float_as_uint(f);
  const unsigned e = (b >> 23) & 0xFFu;
  const unsigned sgn = b & 0x80000000u;
  const unsigned m = b & 0x7FFFFFu;
  unsigned       hi = sgn | ((e + 896u) << 20) | (m >> 3);
  unsigned       lo = m << 29;
  if (e == 0u)
  {
    hi = sgn;
    lo = 0u;
  }
  if (e == 0xFFu)
    hi = sgn | 0x7FF00000u | (m >> 3);
  return __hiloint2double((int)hi, (int)lo);
}

// L2 prefetch of a contiguous range (cp.async.bulk.prefetch: 16-byte aligned
// address, size a multiple of 16; anything else is skipped) and of one line
__device__ __forceinline__ void
prefetch_l2_range(const void * p, unsigned bytes)
{
  if ((((unsigned long long)p | bytes) & 15u) == 0)
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(__cvta_generic_to_global(p)), "r"(bytes) : "memory");
}

__device__ __forceinline__ void
prefetch_l2_line(const void * p)
{
  asm volatile("prefetch.global.L2 [%0];" ::"l"(__cvta_generic_to_global(p)));
}

// The double nearest below (in magnitude) s + t for a renormalised float pair
// (|t| <= ulp(s)), built on the integer pipe: the 24-bit mantissa of t is added
// into the 53-bit mantissa of s; bits of t below that window are dropped (an
// error under 2^-53 |s|).  Pairs that are not renormalised, zero, subnormal or
// non-finite parts take the FP64 path.
__device__ __forceinline__ double
ff_to_d(float s, float t)
{
  const unsigned sb = __float_as_uint(s), tb = __float_as_uint(t);
  const int      es = (int)((sb >> 23) & 0xFFu), et = (int)((tb >> 23) & 0xFFu);
  if (et == 0)
    return f2d_exact(s);
  const int sh = 29 + et - es; // position of t's mantissa within s's 53-bit window
  if (es == 0 || es == 0xFF || et == 0xFF || sh > 5)
    return f2d_exact(s) + f2d_exact(t);
  unsigned long long M = (unsigned long long)((sb & 0x7FFFFFu) | 0x800000u) << 29;
  const unsigned     mt = (tb & 0x7FFFFFu) | 0x800000u;
  const unsigned     T = sh >= 0 ? (mt << sh) : (sh > -24 ? (mt >> -sh) : 0u);
  M = ((sb ^ tb) & 0x80000000u) ? M - T : M + T;
  unsigned long long e = (unsigned long long)(es + 896); // 1023 - 127
  if (M >> 53)
  {
    M >>= 1;
    ++e;
  }
  else if (!(M >> 52))
  {
    M <<= 1;
    --e;
  }
  return __longlong_as_double((long long)(((unsigned long long)(sb & 0x80000000u) << 32) | (e << 52) | (M & 0xFFFFFFFFFFFFFull)));
}

// error-free difference of two floats: a - b == hi + lo exactly (Knuth's TwoSum)
__device__ __forceinline__ void
two_diff(float a, float b, float & hi, float & lo)
{
  hi = __fsub_rn(a, b);
  const float bb = __fsub_rn(a, hi);
  lo = __fadd_rn(__fsub_rn(a, __fadd_rn(hi, bb)), __fsub_rn(bb, b));
}

// error-free sum of two floats: a + b == hi + lo exactly
__device__ __forceinline__ void
two_sum(float a, float b, float & hi, float & lo)
{
  hi = __fadd_rn(a, b);
  const float bb = __fsub_rn(hi, a);
  lo = __fadd_rn(__fsub_rn(a, __fsub_rn(hi, bb)), __fsub_rn(b, bb));
}

// The same two transformations on two independent pairs at once, with the
// packed FP32x2 arithmetic of sm_100+ (one issue slot for both lanes; each
// lane rounds to nearest like the scalar form, so the results are the scalar
// ones bit for bit).  x - y is formed as fma(y, -1, x), exact in its product.
__device__ __forceinline__ float2
fsub2_rn(float2 x, float2 y)
{
  return __ffma2_rn(y, make_float2(-1.0f, -1.0f), x);
}

__device__ __forceinline__ void
two_diff2(float2 a, float2 b, float2 & hi, float2 & lo)
{
  hi = fsub2_rn(a, b);
  const float2 bb = fsub2_rn(a, hi);
  lo = __fadd2_rn(fsub2_rn(a, __fadd2_rn(hi, bb)), fsub2_rn(bb, b));
}

__device__ __forceinline__ void
two_sum2(float2 a, float2 b, float2 & hi, float2 & lo)
{
  hi = __fadd2_rn(a, b);
  const float2 bb = fsub2_rn(hi, a);
  lo = __fadd2_rn(fsub2_rn(a, fsub2_rn(hi, bb)), fsub2_rn(b, bb));
}

// ordered comparisons of doubles against positive constants on the integer
// pipe (IEEE doubles order like sign-magnitude integers; NaN never clamps to 0)
__device__ __forceinline__ bool
dlt_pos(double x, double c)
{
  return __double_as_longlong(x) < __double_as_longlong(c);
}
__device__ __forceinline__ bool
dgt_pos(double x, double c)
{
  const long long b = __double_as_longlong(x);
  return b > __double_as_longlong(c) && b < 0x7FF0000000000001LL;
}
__device__ __forceinline__ bool
finite_bits(double x)
{
  return (__double2hiint(x) & 0x7FF00000) != 0x7FF00000;
}

// mixture pressure from a conservative state: FP32 except the numerator
// rho e - PI when it can cancel (FP64 then): eosk 0 ideal gases, 1 a
// stiffened-gas constant, 2 Mie-Grueneisen laws (S and PI from the partial
// densities).  Returns p; also the FP32 density and velocities.
template <int DIM>
__device__ __forceinline__ float
pressure_mixed(const double * u, const PhysParams & P, int eosk, float & d, float & ux, float & uy, float & uz, float & a0f)
{
  using H = V<DIM>;
  d = fmaxf(d2f_nan(u[H::ID]), P.f_smallr);
  const float inv = __frcp_rn(d);
  ux = d2f_nan(u[H::IU]) * inv;
  uy = d2f_nan(u[H::IV]) * inv;
  float k2 = ux * ux + uy * uy;
  uz = 0.0f;
  if constexpr (DIM == 3)
  {
    uz = d2f_nan(u[H::IW]) * inv;
    k2 += uz * uz;
  }
  const double a0u = u[H::IA0];
  a0f = d2f_nan(a0u);
  const float K = 0.5f * d * k2;
  float       num;
  if (eosk == 2)
  {
    float S, PI, C1, C0;
    mg_mixture_f(P, a0f, 1.0f - a0f, d2f_nan(u[H::IAD0]), d2f_nan(u[H::IAD1]), S, PI, C1, C0);
    num = d2f_nan((u[H::IE] - f2d_exact(PI)) - f2d_exact(K));
    return __fdividef(num, S);
  }
  if (eosk == 1)
  {
    const double PI = fma(a0u, P.dgpx, P.gpx[1]);
    num = d2f_nan((u[H::IE] - PI) - f2d_exact(K));
  }
  else
    num = d2f_nan(u[H::IE]) - K;
  const float S = fmaf(a0f, P.f_dxi, P.f_xi[1]);
  return __fdividef(num, S);
}
// FP32 form of the source-term factors (see source_factors_fp64)
template <int DIM>
__device__ __forceinline__ void
source_factors_mixed(const double * u, const PhysParams & P, int eosk, float & st0, float & st1)
{
  using H = V<DIM>;
  if (P.source_term != 1)
  {
    st0 = st1 = 1.0f;
    return;
  }
  float       d, ux, uy, uz, a0f;
  const float p = pressure_mixed<DIM>(u, P, eosk, d, ux, uy, uz, a0f);
  float       K0, K1;
  if (eosk == 2)
  {
    K0 = mg_bulk_modulus_f(P, 0, a0f, d2f_nan(u[H::IAD0]), p);
    K1 = mg_bulk_modulus_f(P, 1, d2f_nan(u[H::IA1]), d2f_nan(u[H::IAD1]), p);
  }
  else
  {
    K0 = (float)P.gamma[0] * (p + (float)P.pinf[0]);
    K1 = (float)P.gamma[1] * (p + (float)P.pinf[1]);
  }
  const float kbar = __frcp_rn(a0f * __frcp_rn(K0) + d2f_nan(u[H::IA1]) * __frcp_rn(K1));
  st0 = 1.0f - kbar * __frcp_rn(K0);
  st1 = 1.0f - kbar * __frcp_rn(K1);
}

// FP32-bulk conservative -> primitive (computePrimitives, models/utils.h:200-250)
template <int DIM>
__device__ __forceinline__ void
prim_mixed(const double * u, float * q, const PhysParams & P, int eosk)
{
  using H = V<DIM>;
  float       d, ux, uy, uz, a0f;
  const float p = pressure_mixed<DIM>(u, P, eosk, d, ux, uy, uz, a0f);
  float       a0 = fmaxf(0.0f, fminf(1.0f, a0f));
  float       r0 = d2f_nan(u[H::IAD0]), r1 = d2f_nan(u[H::IAD1]);
  const float eps = 1e-12f;
  if (r0 < eps)
    r0 = 0.0f;
  if (r1 < eps)
    r1 = 0.0f;
  if (a0 < eps)
    a0 = 0.0f;
  if (a0 > 1.0f - eps)
    a0 = 1.0f;
  q[H::QR0] = r0;
  q[H::QR1] = r1;
  q[H::QP] = p;
  q[H::QU] = ux;
  q[H::QV] = uy;
  if constexpr (DIM == 3)
    q[H::QW] = uz;
  q[H::QA] = a0;
}

} // namespace g5
