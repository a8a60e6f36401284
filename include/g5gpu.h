/*
 * g5gpu.h — C ABI of the GB300 (sm_103a) five-equation block timestep.
 *
 * This is the drop-in boundary for the reference's GodunovImplemBase
 * (scheme/GodunovImplemBase.h:59-198): a solver that owns U and U2 on the
 * device calls g5_step where it called GodunovImplemBase::do_time_step, and
 * g5_compute_inv_dt where it called ComputeDtFiveEqFunctor::apply.  Plain
 * pointers and sizes only; all device pointers are caller-owned except the
 * scratch the context allocates in g5_set_mesh and frees in g5_destroy.
 *
 * Data layout (identical to the reference's DataArrayBlock, cell index
 * fastest, then variable, then block):
 *   U[n_blocks][nv][bsize^dim], FP64, nv = 8 (2D) or 9 (3D),
 *   variable ids ID=0 IE=1 IU=2 IV=3 (IW=4) IA0 IAD0 IA1 IAD1
 *   (models/FiveEq.h:35-50); owned blocks first, then outside blocks.
 *
 * Every call returns 0 on success or a negative G5_ERR_* code.  Nothing
 * traps or asserts on the device: device-side problems raise bits in a
 * status word read by g5_status.  Calls are asynchronous on the stream
 * given; g5_step_dev, g5_fill_outside, g5_compute_inv_dt and g5_advance
 * neither allocate nor synchronise, so they may be captured in a CUDA graph
 * (g5_step copies dt from host memory first: capture g5_step_dev instead).
 */
#ifndef G5GPU_H_
#define G5GPU_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* error codes */
#define G5_OK 0
#define G5_ERR_ARG (-1)         /* invalid argument */
#define G5_ERR_CUDA (-2)        /* a CUDA runtime call failed */
#define G5_ERR_NONPHYSICAL (-3) /* device flag: non-finite state or empty volume fractions */
#define G5_ERR_TIMEOUT (-4)     /* device flag: a bounded device wait gave up */
#define G5_ERR_MESH (-5)        /* invalid block table (or device flag: index out of range) */
#define G5_ERR_UNSUPPORTED (-6) /* (dim, bsize, option) combination not compiled */

/* status bits returned by g5_status */
#define G5_STATUS_NONPHYSICAL 1u
#define G5_STATUS_MESH 2u
#define G5_STATUS_TIMEOUT 4u

/* precision modes of g5_step (arithmetic of the flux computation) */
#define G5_MODE_FP64 0  /* the reference's method, all FP64 */
#define G5_MODE_MIXED 1 /* FP32 bulk (slopes, predictor, HLLC), FP64 pressure recovery, accumulation, renormalisation, dt */

/* boundary condition codes (border_conditions/FillOutside.h:51-55) */
#define G5_BC_NONE 0
#define G5_BC_PERIODIC 1
#define G5_BC_ZERO_GRADIENT 2
#define G5_BC_WALL 3

/*
 * Scheme parameters: HydroSettings (models/HydroSettings.h:30-54), the EOS of
 * the two materials (stiffened gas; gamma, pinf), THINCParams, the time
 * integrator, the volume-fraction source term type, border conditions and the
 * cell length of every AMR level (compute_cell_length(level, bx) *
 * scaling_factor, scheme/ComputeFluxesAndStoreFunctor.cpp:359).
 */
typedef struct G5Params
{
  int32_t dim;          /* 2 or 3 */
  int32_t bsize;        /* cells per block edge: 2D 8 or 16, 3D 8 */
  int32_t integrator;   /* 0 HANCOCK, 1 RK1, 2 RK2_SSP (two stages in g5_advance / g5_run) */
  int32_t thinc;        /* 0 MUSCL, 1 THINC interface reconstruction */
  int32_t source_term;  /* 0 ALLAIRE_KOKH, 1 MILLER_PUCKETT */
  int32_t prolongation; /* ghost cells in a coarser neighbour: G5_PROLONG_* below */
  int32_t bc[6];        /* xmin xmax ymin ymax zmin zmax */
  double  gamma[2];
  double  pinf[2];
  double  smallr;
  double  smallc;
  double  slope_type; /* 1 minmod, 2 MC */
  double  cfl;
  double  thinc_beta;
  double  thinc_eps;
  double  level_dx[32];
  /* Material laws (Mie-Grueneisen family), per material k.  G5_EOS_STIFFENED
   * uses gamma[k] and pinf[k] (ideal gas: pinf 0); the other laws read mg[k]:
   *   G5_EOS_JWL         {rho0, Gamma0, A1, A2, R1, R2, e0}
   *   G5_EOS_SHOCKWAVE   {rho0, Gamma0, c0, s1, s2, s3, b, e0}
   *   G5_EOS_SHOCKWAVE2  {rho0, Gamma0, c0, s, alpha, e0, p0}
   * (the [material<k>_mie_gruneisen_jwl/_sw/_sw2] sections of the decks).
   * Both precision modes step every law (G5_MODE_MIXED evaluates the laws and
   * the mixture rules in FP32 and the pressure numerator rho e - PI in FP64);
   * gamma[k] must still be > 1 (unused by those laws). */
  int32_t eos[2];
  double  mg[2][8];
} G5Params;

#define G5_EOS_STIFFENED 0
#define G5_EOS_JWL 1
#define G5_EOS_SHOCKWAVE 2
#define G5_EOS_SHOCKWAVE2 3

/* CellCenteredProlongationType of the ghost fill
 * (scheme/ConvertToPrimitivesVariablesFunctor.cpp:893-917).  SIMPLE_COPY
 * copies the coarse cell; the others are computed by a pass before each step
 * kernel launch (g5_step, g5_step_batched, g5_step_host, g5_advance, g5_run)
 * from the coarse cells around the block.  CONSERVATIVE_O4 on 8-cell blocks
 * also reads children of a finer neighbour that do not touch the block; where
 * such a child is refined further or lies beyond a domain face the device
 * raises G5_ERR_MESH (g5_status).  g5_step_static supports SIMPLE_COPY only. */
#define G5_PROLONG_SIMPLE_COPY 0
#define G5_PROLONG_EXTRAPOLATE_LINEAR_MINMOD 1
#define G5_PROLONG_CONSERVATIVE_O2 2
#define G5_PROLONG_CONSERVATIVE_O4 3

/*
 * Block table (host pointers; copied to the device by g5_set_mesh).  It
 * replaces the reference's orchard keys + hashmap + StencilHelper +
 * conformal status for one step (resize_auxiliary_data,
 * scheme/GodunovImplemV0.cpp:37-61).  Slot s of a block is the same-level
 * neighbour at offset (dx,dy,dz) in {-1,0,1}^dim, s = (dx+1) + 3(dy+1) + 9(dz+1).
 */
typedef struct G5Mesh
{
  int32_t         n_owned;    /* owned leaf blocks */
  int32_t         n_outside;  /* outside blocks (boundary conditions), stored after the owned ones */
  int32_t         n_inst;     /* independent instances batched in the table (>= 1) */
  int32_t         reserved;
  const int32_t * level;      /* [n_owned + n_outside] AMR level */
  const int32_t * coord;      /* [(n_owned + n_outside) * 3] block coordinates at its level */
  const int32_t * nbr;        /* [n_owned * 3^dim * 2^dim] neighbour blocks per slot (children for finer slots) */
  const int8_t *  nbr_rel;    /* [n_owned * 3^dim] -1 coarser, 0 same level, +1 finer */
  const int32_t * out_src;    /* [n_outside] inside block copied by each outside block */
  const int8_t *  out_normal; /* [n_outside * 3] outside normal of each outside block */
  const int8_t *  out_border; /* [n_outside * 6] inside block touches domain face f */
  const int32_t * inst;       /* [n_owned + n_outside] instance of each block, NULL = all 0 */
} G5Mesh;

typedef struct G5Context G5Context;

/* version string of the library */
const char * g5_version(void);

/* Create a context on the current CUDA device.  Mirrors the
 * GodunovImplemBase constructor (scheme/GodunovImplemBase.h:71-89). */
int g5_create(const G5Params * params, G5Context ** out_ctx);

/* Destroy a context and free its device memory. */
int g5_destroy(G5Context * ctx);

/* Upload a block table and size the scratch memory: mirrors
 * GodunovImplemV0::resize_auxiliary_data (scheme/GodunovImplemV0.cpp:37-61).
 * Synchronous (allocates); call it outside stream capture.  A table without
 * blocks (a rank that owns none) is accepted, its arrays may be NULL; the
 * calls on it launch nothing (their device pointers must still be non-NULL). */
int g5_set_mesh(G5Context * ctx, const G5Mesh * mesh);

/* Device bytes held by the context: GodunovImplemBase::total_mem_size_in_bytes
 * (scheme/GodunovImplemBase.h:98-99). */
int64_t g5_mem_bytes(const G5Context * ctx);

/* One time step U -> U2 of every owned block, with dt per instance given on
 * the host (dt_host[n_inst]).  GodunovImplemBase::do_time_step(U, U2, dt)
 * (scheme/GodunovImplemBase.h:102-103, scheme/GodunovImplemV0.cpp:85-151).
 * U's outside blocks must hold the boundary values (g5_fill_outside).
 * The owned blocks of U2 are written (U2's outside blocks are untouched);
 * U2 need not be initialised.  mode = G5_MODE_FP64 or G5_MODE_MIXED.
 * inv_dt_out (device, [n_inst], may be NULL) receives, fused in the same
 * kernels, max over owned cells of sum_d (c+|u_d|)/dx of the NEW state U2,
 * i.e. the input of the next step's dt (ComputeDtFiveEqFunctor::compute_cfl,
 * scheme/ComputeDtFiveEqFunctor.cpp:87-134); it must be zeroed by the caller
 * (or use g5_step_dev, which manages it). */
int g5_step(G5Context * ctx, const double * d_U, double * d_U2, const double * dt_host, int mode, double * d_inv_dt_out, void * stream);

/* Same as g5_step with dt read from device memory (d_dt[n_inst]). */
int g5_step_dev(G5Context * ctx, const double * d_U, double * d_U2, const double * d_dt, int mode, double * d_inv_dt_out, void * stream);

/* Batched form of g5_step_dev over a work list of instances: one step of the
 * owned blocks of the instances listed in instances[n_list] (host array), each
 * with its own dt (d_dt[instance]); the blocks of the other instances are not
 * written in U2 and their CFL accumulators in d_inv_dt_out are left as they
 * are.  Instances are independent meshes batched in one table (G5Mesh.inst),
 * e.g. runs that reached their end time drop out of the list. */
int g5_step_batched(G5Context * ctx,
                    const double * d_U,
                    double *       d_U2,
                    const double * d_dt,
                    int            mode,
                    const int32_t * instances,
                    int            n_list,
                    double *       d_inv_dt_out,
                    void *         stream);

/* GodunovImplemBase::do_time_step for a caller whose U and U2 live in host
 * memory (pinned, for the copies to overlap): h_U[n_owned + n_outside blocks]
 * (outside blocks filled) is copied to a device staging array and h_U2's
 * owned blocks are copied back, in chunks of consecutive blocks on two
 * internal streams, overlapped with the step: a chunk of blocks is stepped as
 * soon as its own and its neighbours' data are on the device, and copied back
 * as soon as its blocks are final (coarse/fine refluxing included).  Same
 * results as g5_step.  h_inv_dt_out (host, [n_inst], may be NULL) receives the
 * CFL rate of the new state.  Asynchronous on `stream`: synchronise it before
 * reading h_U2.  The first call allocates the staging arrays (2 x the state);
 * g5_set_mesh frees them. */
int g5_step_host(G5Context * ctx, const double * h_U, double * h_U2, const double * dt_host, int mode, double * h_inv_dt_out, void * stream);

/* derived quantities of ComputeDerivedQuantities (utils/ComputeDerivedQuantities.h:
 * 42-51, the DERIVED_QUANTITY order) */
#define G5_DQ_RHO_MIX 0
#define G5_DQ_THERMAL_PRESSURE 1
#define G5_DQ_SPEED_OF_SOUND 2
#define G5_DQ_SPECIFIC_EKIN 3
#define G5_DQ_LOCAL_MACH_NUMBER 4
#define G5_DQ_VX 5
#define G5_DQ_VY 6
#define G5_DQ_VZ 7

/* ComputeDerivedQuantities::run (utils/ComputeDerivedQuantities.h:96-180): one
 * quantity per cell of blocks [oct_begin, oct_begin + num_octs) of d_U into
 * d_out[n_blocks][1][bsize^dim] (other blocks of d_out untouched), FP64 in the
 * reference's order.  The range must lie within the context's block table
 * (owned + outside blocks), as check_args_validity requires. */
int g5_derived_quantity(G5Context * ctx, const double * d_U, int quantity, int64_t oct_begin, int64_t num_octs, double * d_out, void * stream);

/* The datasets of one output file of SolverGodunovFiveEq::save_solution_hdf5
 * (SolverGodunovFiveEq.cpp:809-886: a per-quadrant array per state variable
 * and per derived quantity), packed on the device in one pass over d_U so that
 * a single device-to-host copy carries them: fields[k] (host, 1 <= nfields <=
 * G5_MAX_PACK_FIELDS) is a variable of the state (0 .. nv - 1, the reference's
 * VarId numbering: rho_mix, e_tot, rho_vx, rho_vy[, rho_vz], alpha_0,
 * alpha_rho_0, alpha_1, alpha_rho_1) or G5_FIELD_DERIVED + a G5_DQ_*
 * quantity (the values of g5_derived_quantity).  Blocks [oct_begin, oct_begin
 * + num_octs) of the table go to d_out[k][num_octs][bsize^dim].  No
 * counterpart of the packing in the reference, which copies the whole state
 * to the host and writes each dataset from there. */
#define G5_FIELD_DERIVED 64
#define G5_MAX_PACK_FIELDS 16
int g5_pack_fields(G5Context * ctx, const double * d_U, const int32_t * fields, int nfields, int64_t oct_begin, int64_t num_octs,
                   double * d_out, void * stream);

/* ComputeDtFiveEqFunctor::apply (scheme/ComputeDtFiveEqFunctor.h:113-121):
 * d_inv_dt[n_inst] <- max over owned cells of sum_d (c+|u_d|)/dx. */
int g5_compute_inv_dt(G5Context * ctx, const double * d_U, double * d_inv_dt, void * stream);

/* FillOutsideCellFunctor::apply (border_conditions/FillOutside.cpp:44-65):
 * fill the outside blocks of U from the inside blocks. */
int g5_fill_outside(G5Context * ctx, double * d_U, void * stream);

/* Solver loop of SolverGodunovFiveEq::next_iteration_impl for HANCOCK/RK1
 * (SolverGodunovFiveEq.cpp:394-526), split in two calls so that a caller can
 * interleave its own work between steps:
 *   g5_begin(U):        fill the outside blocks of U and set the context's
 *                       CFL accumulator to inv_dt(U) (compute_dt_local);
 *   g5_advance(U, U2):  dt = cfl / inv_dt (kept on the device), U2 = step(U),
 *                       fill the outside blocks of U2, inv_dt(U2) fused in
 *                       the step.  The caller then swaps U and U2.
 * g5_advance replays a CUDA graph cached per (U, U2, mode).  d_dt_out
 * (device, [n_inst], may be NULL) receives the dt used. */
int g5_begin(G5Context * ctx, double * d_U, void * stream);
int g5_advance(G5Context * ctx, const double * d_U, double * d_U2, int mode, double * d_dt_out, void * stream);

/* nsteps of the loop above (g5_begin then g5_advance with U/U2 swapped each
 * step); on exit the final state is in d_U (d_U2 is scratch of the same
 * size).  d_dt_hist (device, [nsteps * n_inst], may be NULL) receives every dt. */
int g5_run(G5Context * ctx, double * d_U, double * d_U2, int nsteps, int mode, double * d_dt_hist, void * stream);

/* ComputeRefineFlags::run (scheme/ComputeRefineFlags.cpp:18-65): per owned
 * block, max over cells of the indicator flag (-1 init, 0 coarsen, 1 nothing,
 * 2 refine).  indicator: 0 SIMPLE_GRADIENT, 1 LOHNER_UNSPLIT, 2 LOHNER_SPLIT. */
int g5_refine_flags(G5Context * ctx,
                    const double * d_U,
                    int            indicator,
                    double         eps_refine,
                    double         eps_coarsen,
                    double         eps_lohner,
                    int            level_min,
                    int            level_max,
                    int8_t *       d_flags,
                    void *         stream);

/* Block map of one mesh adaptation (host arrays), for g5_remap.  New owned
 * block j (order of the new mesh's U) comes from the old owned blocks:
 *   kind[j] = G5_REMAP_COPY:      old block src[j*2^dim];
 *   kind[j] = G5_REMAP_REFINED:   child src[j*2^dim + 1] (x + 2y + 4z) of old
 *                                 block src[j*2^dim];
 *   kind[j] = G5_REMAP_COARSENED: parent of old blocks src[j*2^dim + c],
 *                                 c = x + 2y + 4z the child position. */
#define G5_REMAP_COPY 0
#define G5_REMAP_REFINED 1
#define G5_REMAP_COARSENED 2
typedef struct G5Remap
{
  int32_t         n_old; /* owned blocks of the old mesh */
  int32_t         n_new; /* owned blocks of the new mesh */
  const int8_t *  kind;  /* [n_new] */
  const int32_t * src;   /* [n_new * 2^dim] */
} G5Remap;

/* UserDataRemapper::remap_block_data as called by
 * SolverGodunovFiveEq::map_userdata_after_adapt (SolverGodunovFiveEq.cpp:
 * 1137-1169): the owned blocks of d_Unew from those of d_Uold.  Refined blocks
 * take the SIMPLE_COPY prolongation of their parent, coarsened blocks the
 * restriction of get_conservative_vars_restriction (mean of the 2^dim fine
 * cells; IA1 = 1 - IA0, ID = IAD0 + IAD1).  Under another G5Params.prolongation
 * the refined blocks are prolonged with it from the parent cell and its
 * neighbours at the old level: the context must still hold the old mesh
 * (call g5_remap before g5_set_mesh of the adapted mesh; G5_ERR_ARG
 * otherwise) and d_Uold's outside blocks must be filled.  Outside blocks of d_Unew are not
 * written (g5_set_mesh with the new table, then g5_fill_outside).  The map is
 * validated on the host (G5_ERR_MESH) and copied to stream-ordered device
 * memory (cudaMallocAsync/cudaFreeAsync on `stream`): not capturable. */
int g5_remap(G5Context * ctx, const G5Remap * remap, const double * d_Uold, double * d_Unew, void * stream);

/* Read and clear the device status word (synchronises the stream).
 * Returns the G5_STATUS_* bits (>= 0) or a negative error. */
int g5_status(G5Context * ctx, void * stream);

/* Autotune the launch shape of the step for the current mesh and one
 * precision mode (no counterpart in the reference, whose Kokkos policies are
 * fixed).  Candidates: CTAs per SM of the persistent step kernel (1 up to the
 * occupancy maximum), dynamic block claiming on or off, the block walk order
 * (blocks with coarse/fine neighbours first, or table order) and, for the
 * FP32-bulk 2D pass over coarse/fine records, its layout (a separate pass
 * with 8 lanes or one thread per deferred cell, or 8 lanes per cell in the
 * step kernel's tail, by the CTAs out of blocks).  Every candidate computes the
 * same values bit for bit.  Each is timed twice on d_U -> d_U2 (3 steps after a warm-up, CUDA
 * events on `stream`), and g5_tune_pick chooses with a 2 % margin in favour of
 * the default shape.  The choice is kept by the context for that mode
 * (across g5_set_mesh) until the next g5_tune or g5_set_shape.  Synchronises
 * the stream; d_U2 is overwritten.  Returns the packed shape
 * (ctas_per_sm + 16 claim + 32 walk + 64 reflux layout, > 0) or a negative
 * error. */
int g5_tune(G5Context * ctx, const double * d_U, double * d_U2, int mode, void * stream);

/* The tuner's selection rule, host only: the index of the smallest positive
 * time of ms[n], except that the default index stays chosen while its time is
 * within (1 + margin) of the smallest.  Negative on bad arguments. */
int g5_tune_pick(const float * ms, int n, int default_index, float margin);

/* The launch shape a mode uses: out4 = {CTAs per SM, claim, walk order,
 * reflux layout (0: a separate pass, 8 lanes per deferred cell; 1: a separate
 * pass, one thread per cell; 2 (the FP32-bulk form's default): 8 lanes per
 * cell in the step kernel's tail, by the CTAs out of blocks, where the
 * FP32-bulk 2D full-mesh step has coarse/fine records, otherwise as 0; the
 * FP64 form (default 0) and 3D take a separate pass with one thread per
 * cell whatever the layout)}. */
int g5_tune_choice(const G5Context * ctx, int mode, int32_t * out4);

/* The candidates and their times (ms per step) of the last g5_tune of a mode:
 * up to cap entries (packed shapes as g5_tune returns them); returns the
 * number of candidates. */
int g5_tune_report(const G5Context * ctx, int mode, int32_t * shapes, float * ms, int cap);

/* Set the launch shape of a mode by hand (shape4 as g5_tune_choice gives it;
 * CTAs per SM 0 = the occupancy maximum). */
int g5_set_shape(G5Context * ctx, int mode, const int32_t * shape4);

/* Number of kernel launches issued by the last g5_step / g5_advance / g5_run call. */
int g5_last_launch_count(const G5Context * ctx);

/* Size of the fixed device scratch array used by g5_step_static (16 MiB). */
#define G5_STATIC_SCRATCH_BYTES (16u << 20)

/* No counterpart in the reference: an allocation-free variant of g5_step.
 *
 * For callers that must not allocate device memory while they advance the
 * solution, e.g. a solver whose device memory belongs to its framework's
 * pool allocator, or a plugin whose host process accounts for every device
 * allocation.  It needs no context: the block table is taken from host memory
 * (the G5Mesh pointers are HOST pointers, as for g5_set_mesh), and dt, the
 * block table, the coarse/fine face records and the status word are staged
 * in one file-scope device array of G5_STATIC_SCRATCH_BYTES that every GPU
 * loading the library keeps until the process exits.  No cudaMalloc, cudaFree
 * or other allocating routine is called.
 *
 * Same step and arguments meaning as g5_step; the block table is checked as
 * g5_set_mesh checks it (G5_ERR_MESH).  d_status_out (device, may be NULL)
 * receives the G5_STATUS_* bits raised by the kernels (the caller zeroes it);
 * with NULL the bits go to a word inside the scratch array that no call
 * reads, so non-physical states are not reported.  Returns G5_ERR_ARG when
 * the mesh needs more than G5_STATIC_SCRATCH_BYTES of scratch, and
 * G5_ERR_UNSUPPORTED when `stream` is in capture mode (the host arrays are
 * staged at call time).
 *
 * dt_host and the G5Mesh arrays are copied to the scratch array with
 * cudaMemcpyAsync on `stream`.  From pageable memory the copy is staged
 * before the call returns, so the arrays may be reused at once; from
 * page-locked memory (cudaHostAlloc, registered or pinned buffers) it runs
 * when the stream reaches it, so the caller must leave those arrays unchanged
 * until the stream has passed this call.
 *
 * The first call on a device looks up the array's device address with that
 * device current (cudaGetSymbolAddress); make that first call before any
 * stream capture.  All calls share the one array and the last call's contents
 * stay in it: calls whose work overlaps on the GPU (several streams, or
 * several host threads on one device) race and must be serialised by the
 * caller. */
int g5_step_static(const G5Params * params,
                   const G5Mesh *   mesh,
                   const double *   d_U,
                   double *         d_U2,
                   const double *   dt_host,
                   int              mode,
                   double *         d_inv_dt_out,
                   unsigned int *   d_status_out,
                   void *           stream);

/*
 * Block forest of the dynamic AMR cycle (host only; no device call).  It
 * stands where the reference adapts its p4est forest
 * (AMRManager::rebuild_from_context, SolverGodunovFiveEq.cpp:258-314) and
 * rebuilds the neighbour hashmap the stencils read: refinement, 2:1 balance
 * across faces, edges and corners, adaptation from ComputeRefineFlags codes
 * with the old -> new block map of g5_remap, and the G5Mesh block table.
 * Leaves are rows (level, x, y, z) in block units of their level (z = 0 in
 * 2D) on a brick of nbrick level-0 trees; leaf order (and owned-block order
 * of the table): brick tree, then the Morton index of the leaf's origin at the
 * finest level present.
 */
typedef struct G5Forest G5Forest;
typedef struct G5ForestSpec
{
  int32_t dim;
  int32_t bsize;
  int32_t nbrick[3];
  int32_t periodic[3];
  int32_t level_min;
  int32_t level_max;
} G5ForestSpec;

/* n_leaves == 0: uniform at level_min.  G5_ERR_MESH for a leaf outside the
 * brick or the level range. */
int g5_forest_create(const G5ForestSpec * spec, const int32_t * leaves, int64_t n_leaves, G5Forest ** out);
int g5_forest_destroy(G5Forest * forest);
int64_t g5_forest_num_leaves(const G5Forest * forest);
/* the leaves in table order, 4 int32 each */
int g5_forest_leaves(const G5Forest * forest, int32_t * out);
/* refine the given leaves below level_max; returns how many */
int g5_forest_refine(G5Forest * forest, const int32_t * keys, int64_t n);
/* refine until 2:1 balanced; returns how many refinements */
int g5_forest_balance(G5Forest * forest);
/* one adaptation: flags[i] for the i-th leaf in table order (2 refine, 0
 * coarsen, else keep).  Refines flagged leaves below level_max, restores the
 * balance by refining, coarsens complete families flagged 0 above level_min
 * that were not refined unless the coarse block would touch a leaf two levels
 * finer.  Writes kind[j] / src[j * 2^dim ..] of every new leaf (G5Remap's
 * arrays, capacity cap >= n_flags * 2^dim) and returns the new leaf count. */
int64_t g5_forest_adapt(G5Forest * forest, const int8_t * flags, int64_t n_flags, int8_t * kind, int32_t * src, int64_t cap);
/* block table of the leaves (G5Mesh arrays: level and coord for owned then
 * outside blocks, nbr / nbr_rel per owned block, the outside twins'
 * out_src / out_normal / out_border); sizes first */
int g5_forest_table_sizes(G5Forest * forest, int32_t * n_owned, int32_t * n_outside);
int g5_forest_table(G5Forest * forest,
                    int32_t *  level,
                    int32_t *  coord,
                    int32_t *  nbr,
                    int8_t *   nbr_rel,
                    int32_t *  out_src,
                    int8_t *   out_normal,
                    int8_t *   out_border);

#ifdef __cplusplus
}
#endif

#endif /* G5GPU_H_ */
