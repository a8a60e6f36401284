// g5_launch.h — launchers exported by the kernel translation units to the
// C-ABI layer (internal to libg5gpu.so).
#pragma once

#include <cuda_runtime.h>

#include "g5_common.cuh"

namespace g5
{

// fused step (FP64 TU: mixed == false, mixed TU: mixed == true).
// ctas_per_sm <= 0 selects the occupancy maximum.  Returns the launch error.
cudaError_t launch_step_fp64(int dim, int b, const StepArgs & a, int ctas_per_sm, cudaStream_t s, int * launches);
cudaError_t launch_step_mixed(int dim, int b, const StepArgs & a, int ctas_per_sm, cudaStream_t s, int * launches);
// ghost cells in coarser neighbours prolonged into a.m.pg (nothing when
// a.m.pg is null, i.e. SIMPLE_COPY); launched by both step launchers first
cudaError_t launch_prolong(int dim, int b, const StepArgs & a, cudaStream_t s, int * launches);
// whether the (dim, b) pair is compiled
bool step_supported(int dim, int b);
// occupancy (CTAs per SM) of the fused step kernel
int step_max_ctas_per_sm_fp64(int dim, int b);
int step_max_ctas_per_sm_mixed(int dim, int b);

cudaError_t launch_fill_outside(int dim, int b, double * U, const DevMesh & m, const PhysParams & p, cudaStream_t s);
cudaError_t launch_inv_dt(int dim, int b, const double * U, const DevMesh & m, const PhysParams & p, double * invdt, cudaStream_t s);
cudaError_t launch_rk2_combine(int dim, int b, bool mixed, const double * U, double * U2, const DevMesh & m, const PhysParams & p,
                               double * invdt, cudaStream_t s);
cudaError_t launch_rk2_combine_mixed(int dim, int b, const double * U, double * U2, const DevMesh & m, const PhysParams & p,
                                     double * invdt, cudaStream_t s);
cudaError_t launch_dt_update(double * invdt, double * dt, double * dt_hist, int n_inst, double cfl, cudaStream_t s);
cudaError_t launch_refine_flags(int dim, int b, const double * U, const DevMesh & m, int indicator, double er, double ec,
                                double el, int lmin, int lmax, int8_t * flags, cudaStream_t s);
// block remap after a mesh adaptation (kind/src validated by the caller)
cudaError_t launch_remap(int dim, int b, const double * Uold, double * Unew, const int8_t * kind, const int32_t * src, int n_new,
                         cudaStream_t s);
// refined blocks of a remap prolonged over the old mesh m (prolongation mode
// 1-3); list rows: old block, then the new block of each child
cudaError_t launch_remap_prolong(int dim, int b, int mode, const double * Uold, double * Unew, const DevMesh & m, const int32_t * list,
                                 int n_ref, unsigned int * status, cudaStream_t s);
// per-record rows of the reflux pass (DeferInfo) for `n` record codes
cudaError_t launch_defer_info(int dim, const DevMesh & m, const int32_t * codes, int n, int32_t * info, cudaStream_t s);
// derived quantity per cell (ComputeDerivedQuantities)
cudaError_t launch_derived(int dim, int b, const double * U, double * out, int quantity, long long oct_begin, long long num_octs,
                           const PhysParams & p, cudaStream_t s);
// the fields of one output file in one pass (pack_fields_kernel): codes[k] a
// variable of U or FIELD_DERIVED + a derived quantity, 1 <= n <= 16
cudaError_t launch_pack_fields(int dim, int b, const double * U, double * out, const int * codes, int n, long long oct_begin,
                               long long num_octs, const PhysParams & p, cudaStream_t s);

// the FP32-bulk 3D step of case v = 3 THINC + equation-of-state kind
// (g5_mixed3d.cu) and the occupancy maximum of its kernels
cudaError_t launch_step3d_mixed_case(int v, const StepArgs & a, int ctas_per_sm, cudaStream_t s, int * launches);
int         step_max_ctas_per_sm_mixed3d();

} // namespace g5
