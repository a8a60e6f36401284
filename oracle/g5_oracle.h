/*
 * g5_oracle.h — CPU restatement of the godunov_five_eq per-block timestep.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity checker of the GPU
 * path: only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
 * may load it.  The product (godunov_five_eq_gb300) never links or calls it.
 *
 * Parity status: the scheme is pinned to the reference's own code, compiled
 * from the reference tree with shim headers (oracle/refpin/), through golden
 * vectors committed under tests/golden/: the HLLC solver and the
 * conservative->primitive conversion per state (models/RiemannSolvers.h,
 * models/utils.h), and one whole do_time_step of periodic tiles of
 * same-level blocks through the reference's scheme functors (limited slopes,
 * MUSCL-Hancock and THINC reconstruction, flux store, read-back update with
 * the ALLAIRE_KOKH and MILLER_PUCKETT source terms, volume-fraction
 * renormalisation, CFL reduction), 2D and 3D, bit for bit, and the
 * refinement flags of ComputeRefineFlags over threshold sweeps.  The mixture EOS,
 * the Youngs normal, the AMR stencil semantics (restriction / prolongation /
 * face sibling sums), the cell length and tree ordering live in the external
 * kalypsso core, which is not available; they are restated from published
 * mathematics and are "parity unpinned" (the pin uses the same restatements
 * for them).
 *
 * Layout of every conservative array U: [n_blocks][nv][b^dim] (cells x
 * fastest), owned blocks first, then "outside" blocks (the reference's
 * outside quadrants that carry the boundary conditions).
 */
#ifndef G5_ORACLE_H_
#define G5_ORACLE_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct G5OParams
{
  int32_t dim;          /* 2 or 3 */
  int32_t b;            /* cells per block edge (bx = by = bz) */
  int32_t integrator;   /* 0 HANCOCK, 1 RK1 */
  int32_t thinc;        /* 0 MUSCL, 1 THINC */
  int32_t source_term;  /* 0 ALLAIRE_KOKH, 1 MILLER_PUCKETT */
  int32_t prolongation; /* 0 SIMPLE_COPY, 1 EXTRAPOLATE_LINEAR_MINMOD, 2/3 CONSERVATIVE_INTERPOLATION_ORDER_2/4 */
  int32_t bc[6];        /* per face (xmin,xmax,ymin,ymax,zmin,zmax): 0 NONE 1 PERIODIC 2 ZERO_GRADIENT 3 WALL */
  double  gamma[2];
  double  pinf[2];
  double  smallr;
  double  smallc;
  double  slope_type;
  double  cfl;
  double  thinc_beta;
  double  thinc_eps;
  double  level_dx[32]; /* cell length per AMR level (already scaled) */
  int32_t eos[2];       /* material law per material: 0 stiffened gas, 1 JWL, 2 SHOCKWAVE, 3 SHOCKWAVE2 */
  double  mg[2][8];     /* law parameters (see g5_oracle.cpp, mg_law) */
} G5OParams;

typedef struct G5OMesh
{
  int32_t         n_owned;
  int32_t         n_outside;
  int32_t         n_inst;     /* number of independent instances (>= 1) */
  int32_t         pad;
  const int32_t * level;      /* [n_total] */
  const int32_t * coord;      /* [n_total*3] block coords at own level */
  const int32_t * nbr;        /* [n_owned * 3^dim * 2^dim] */
  const int8_t *  nbr_rel;    /* [n_owned * 3^dim] : -1 coarser, 0 same, +1 finer */
  const int32_t * out_src;    /* [n_outside] inside block mirrored by each outside block */
  const int8_t *  out_normal; /* [n_outside*3] outside direction per dim */
  const int8_t *  out_border; /* [n_outside*6] inside block touches domain face f */
  const int32_t * inst;       /* [n_total] instance id, NULL => 0 */
} G5OMesh;

/* whole-step API (one context per mesh) */
void * g5o_create(const G5OMesh * mesh, const G5OParams * prm, int nthreads);
void   g5o_destroy(void * ctx);
/* U2 owned blocks <- one step of U; dt[inst] per instance.  returns 0 */
int    g5o_step(void * ctx, const double * U, double * U2, const double * dt);
/* conservative state the ghost fill of owned block n gives its ghosted cell
 * g (g[e] in -2 .. b+1; g[2] = 0 in 2D), before the primitive conversion */
int    g5o_ghost_state(void * ctx, const double * U, int n, const int * g, double * u);
/* max over owned cells of sum_d (c+|u_d|)/dx, per instance */
int    g5o_inv_dt(void * ctx, const double * U, double * inv_dt);
/* fill outside blocks of U from inside blocks (boundary conditions) */
int    g5o_fill_outside(void * ctx, double * U);
/* refine flags per owned block (int8: -1 init, 0 coarsen, 1 nothing, 2 refine) */
int    g5o_refine_flags(void * ctx,
                        const double * U,
                        int            indicator, /* 0 SIMPLE_GRADIENT 1 LOHNER_UNSPLIT 2 LOHNER_SPLIT */
                        double         eps_refine,
                        double         eps_coarsen,
                        double         eps_lohner,
                        int            level_min,
                        int            level_max,
                        int8_t *       flags);

/* block remap after a mesh adaptation: new owned block j from the old owned
 * blocks (kind 0 copy of src[j*2^dim]; 1 SIMPLE_COPY prolongation of child
 * src[j*2^dim+1] of old block src[j*2^dim]; 2 restriction of the old children
 * src[j*2^dim .. +2^dim-1]).  returns 0 */
int    g5o_remap(const G5OParams * prm, int n_new, const int8_t * kind, const int32_t * src, const double * Uold, double * Unew);
/* as g5o_remap, then the refined blocks prolonged with the context's
 * prolongation (if not SIMPLE_COPY) over the context's mesh, which must be
 * the old mesh (src[j*2^dim] its owned blocks) */
int g5o_remap_mesh(void * ctx, int n_new, const int8_t * kind, const int32_t * src, const double * Uold, double * Unew);

/* ComputeDerivedQuantities: quantity (0 RHO_MIX .. 7 VZ) per cell of blocks
 * [begin, begin + count) into out[n_blocks][ncell].  returns 0 */
int    g5o_derived(const G5OParams * prm, const double * U, int quantity, long long begin, long long count, double * out);

/* point functions (used by the golden-vector pins) */
double g5o_compute_primitives(const G5OParams * prm, const double * u, double * q);
void   g5o_riemann_hllc(const G5OParams * prm, const double * qL, const double * qR, double * out);
double g5o_slope(const G5OParams * prm, double q, double qp, double qm);
double g5o_tanh(double x);
double g5o_mixture_pressure(const G5OParams * prm, double rho, double eint, double a0, double ar0, double ar1);
double g5o_mixture_sound_speed(const G5OParams * prm, double rho, double p, double a0, double ar0, double ar1);

#ifdef __cplusplus
}
#endif

#endif
