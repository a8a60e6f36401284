// g5_fp64.cu — FP64 instantiations.  Built with --fmad=false so that every
// product and sum is rounded separately, as in the reference's arithmetic.
#include "g5_aux.cuh"
#include "g5_launch.h"
#include "g5_prolong.cuh"
#include "g5_step2d.cuh"
#include "g5_step3d.cuh"

namespace g5
{

static int g_num_sms = 0;

static int
num_sms()
{
  if (g_num_sms == 0)
  {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
    if (g_num_sms <= 0)
      g_num_sms = 1;
  }
  return g_num_sms;
}

template <int B, bool MIXED>
static cudaError_t
launch_step2d(const StepArgs & a, int ctas_per_sm, cudaStream_t s, int * launches)
{
  using T = Step2DTraits<B, MIXED>;
  static bool configured = false;
  static int  occ = 1;
  if (!configured)
  {
    cudaError_t e = cudaFuncSetAttribute(step2d_kernel<B, MIXED>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)T::smem_bytes);
    if (e != cudaSuccess)
      return e;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, step2d_kernel<B, MIXED>, T::NT, T::smem_bytes);
    if (occ < 1)
      occ = 1;
    configured = true;
  }
  const int per_sm = (ctas_per_sm > 0 && ctas_per_sm < occ) ? ctas_per_sm : occ;
  int       grid = num_sms() * per_sm;
  if (grid > step_count(a))
    grid = step_count(a);
  cudaError_t e = cudaSuccess;
  if (grid >= 1)
  {
    step2d_kernel<B, MIXED><<<grid, T::NT, T::smem_bytes, s>>>(a);
    ++*launches;
    e = cudaGetLastError();
    if (e != cudaSuccess)
      return e;
  }
  if (a.m.n_defer > 0)
  {
    const int n = a.m.n_defer * B;
    reflux2d_kernel<B, false><<<(n + 31) / 32, 32, 0, s>>>(a);
    ++*launches;
    e = cudaGetLastError();
  }
  return e;
}

template <int B, bool MIXED>
static int
occupancy2d()
{
  using T = Step2DTraits<B, MIXED>;
  cudaFuncSetAttribute(step2d_kernel<B, MIXED>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)T::smem_bytes);
  int occ = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, step2d_kernel<B, MIXED>, T::NT, T::smem_bytes);
  return occ;
}

template <bool MIXED>
static cudaError_t
launch_step3d(const StepArgs & a, int ctas_per_sm, cudaStream_t s, int * launches)
{
  using T = Step3DTraits<MIXED>;
  static bool configured = false;
  static int  occ = 1;
  if (!configured)
  {
    cudaError_t e = cudaFuncSetAttribute(step3d_kernel<MIXED>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)T::smem_bytes);
    if (e != cudaSuccess)
      return e;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, step3d_kernel<MIXED>, T::NT, T::smem_bytes);
    if (occ < 1)
      occ = 1;
    configured = true;
  }
  const int per_sm = (ctas_per_sm > 0 && ctas_per_sm < occ) ? ctas_per_sm : occ;
  int       grid = num_sms() * per_sm;
  if (grid > step_count(a))
    grid = step_count(a);
  cudaError_t e = cudaSuccess;
  if (grid >= 1)
  {
    step3d_kernel<MIXED><<<grid, T::NT, T::smem_bytes, s>>>(a);
    ++*launches;
    e = cudaGetLastError();
    if (e != cudaSuccess)
      return e;
  }
  if (a.m.n_defer > 0)
  {
    const int n = a.m.n_defer * 64;
    reflux3d_kernel<MIXED><<<(n + 31) / 32, 32, 0, s>>>(a);
    ++*launches;
    e = cudaGetLastError();
  }
  return e;
}

template <bool MIXED>
static int
occupancy3d()
{
  using T = Step3DTraits<MIXED>;
  cudaFuncSetAttribute(step3d_kernel<MIXED>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)T::smem_bytes);
  int occ = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, step3d_kernel<MIXED>, T::NT, T::smem_bytes);
  return occ;
}

bool
step_supported(int dim, int b)
{
  return (dim == 2 && (b == 8 || b == 16)) || (dim == 3 && b == 8);
}

template <int DIM, int B, int MODE>
static cudaError_t
prolong_t(const StepArgs & a, cudaStream_t s, int * launches)
{
  using T = ProlongTraits<DIM, B, MODE>;
  static bool configured = false;
  if (!configured)
  {
    const cudaError_t e = cudaFuncSetAttribute(prolong_kernel<DIM, B, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)T::smem_bytes);
    if (e != cudaSuccess)
      return e;
    configured = true;
  }
  int grid = num_sms() * 8;
  if (grid > step_count(a))
    grid = step_count(a);
  if (grid < 1)
    return cudaSuccess;
  prolong_kernel<DIM, B, MODE><<<grid, T::NT, T::smem_bytes, s>>>(a);
  ++*launches;
  return cudaGetLastError();
}

cudaError_t
launch_prolong(int dim, int b, const StepArgs & a, cudaStream_t s, int * launches)
{
  if (!a.m.pg)
    return cudaSuccess;
  const int mode = a.p.prolong;
  if (dim == 2 && b == 16)
    return mode == 1 ? prolong_t<2, 16, 1>(a, s, launches)
         : mode == 2 ? prolong_t<2, 16, 2>(a, s, launches)
         : mode == 3 ? prolong_t<2, 16, 3>(a, s, launches)
                     : cudaErrorInvalidValue;
  if (dim == 2 && b == 8)
    return mode == 1 ? prolong_t<2, 8, 1>(a, s, launches)
         : mode == 2 ? prolong_t<2, 8, 2>(a, s, launches)
         : mode == 3 ? prolong_t<2, 8, 3>(a, s, launches)
                     : cudaErrorInvalidValue;
  if (dim == 3 && b == 8)
    return mode == 1 ? prolong_t<3, 8, 1>(a, s, launches)
         : mode == 2 ? prolong_t<3, 8, 2>(a, s, launches)
         : mode == 3 ? prolong_t<3, 8, 3>(a, s, launches)
                     : cudaErrorInvalidValue;
  return cudaErrorInvalidValue;
}

template <int DIM, int B, int MODE>
static cudaError_t
refine_t(const double * Uold, double * Unew, const DevMesh & m, const int32_t * list, int n_ref, unsigned int * status, cudaStream_t s)
{
  using T = RefineTraits<DIM, B, MODE>;
  static bool configured = false;
  if (!configured)
  {
    const cudaError_t e = cudaFuncSetAttribute(prolong_refine_kernel<DIM, B, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)T::smem_bytes);
    if (e != cudaSuccess)
      return e;
    configured = true;
  }
  int grid = num_sms() * 4;
  if (grid > n_ref)
    grid = n_ref;
  if (grid < 1)
    return cudaSuccess;
  prolong_refine_kernel<DIM, B, MODE><<<grid, T::NT, T::smem_bytes, s>>>(Uold, Unew, m, list, n_ref, status);
  return cudaGetLastError();
}

cudaError_t
launch_remap_prolong(int dim, int b, int mode, const double * Uold, double * Unew, const DevMesh & m, const int32_t * list, int n_ref,
                     unsigned int * status, cudaStream_t s)
{
  if (dim == 2 && b == 16)
    return mode == 1 ? refine_t<2, 16, 1>(Uold, Unew, m, list, n_ref, status, s)
         : mode == 2 ? refine_t<2, 16, 2>(Uold, Unew, m, list, n_ref, status, s)
         : mode == 3 ? refine_t<2, 16, 3>(Uold, Unew, m, list, n_ref, status, s)
                     : cudaErrorInvalidValue;
  if (dim == 2 && b == 8)
    return mode == 1 ? refine_t<2, 8, 1>(Uold, Unew, m, list, n_ref, status, s)
         : mode == 2 ? refine_t<2, 8, 2>(Uold, Unew, m, list, n_ref, status, s)
         : mode == 3 ? refine_t<2, 8, 3>(Uold, Unew, m, list, n_ref, status, s)
                     : cudaErrorInvalidValue;
  if (dim == 3 && b == 8)
    return mode == 1 ? refine_t<3, 8, 1>(Uold, Unew, m, list, n_ref, status, s)
         : mode == 2 ? refine_t<3, 8, 2>(Uold, Unew, m, list, n_ref, status, s)
         : mode == 3 ? refine_t<3, 8, 3>(Uold, Unew, m, list, n_ref, status, s)
                     : cudaErrorInvalidValue;
  return cudaErrorInvalidValue;
}

cudaError_t
launch_step_fp64(int dim, int b, const StepArgs & a, int ctas_per_sm, cudaStream_t s, int * launches)
{
  const cudaError_t e = launch_prolong(dim, b, a, s, launches);
  if (e != cudaSuccess)
    return e;
  if (dim == 2 && b == 16)
    return launch_step2d<16, false>(a, ctas_per_sm, s, launches);
  if (dim == 2 && b == 8)
    return launch_step2d<8, false>(a, ctas_per_sm, s, launches);
  if (dim == 3 && b == 8)
    return launch_step3d<false>(a, ctas_per_sm, s, launches);
  return cudaErrorInvalidValue;
}

int
step_max_ctas_per_sm_fp64(int dim, int b)
{
  if (dim == 2 && b == 16)
    return occupancy2d<16, false>();
  if (dim == 2 && b == 8)
    return occupancy2d<8, false>();
  if (dim == 3 && b == 8)
    return occupancy3d<false>();
  return 0;
}

template <int DIM, int B>
static cudaError_t
fill_outside_t(double * U, const DevMesh & m, const PhysParams & p, cudaStream_t s)
{
  constexpr int NC = (DIM == 2) ? B * B : B * B * B;
  const long    n = (long)m.n_outside * NC;
  if (n == 0)
    return cudaSuccess;
  fill_outside_kernel<DIM, B><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(U, m, p);
  return cudaGetLastError();
}

cudaError_t
launch_fill_outside(int dim, int b, double * U, const DevMesh & m, const PhysParams & p, cudaStream_t s)
{
  if (dim == 2 && b == 16)
    return fill_outside_t<2, 16>(U, m, p, s);
  if (dim == 2 && b == 8)
    return fill_outside_t<2, 8>(U, m, p, s);
  if (dim == 3 && b == 8)
    return fill_outside_t<3, 8>(U, m, p, s);
  return cudaErrorInvalidValue;
}

template <int DIM, int B>
static cudaError_t
inv_dt_t(const double * U, const DevMesh & m, const PhysParams & p, double * invdt, cudaStream_t s)
{
  if (m.n_owned == 0)
    return cudaSuccess;
  int grid = num_sms() * 8;
  if (grid > m.n_owned)
    grid = m.n_owned;
  inv_dt_kernel<DIM, B><<<grid, 256, 0, s>>>(U, m, p, invdt);
  return cudaGetLastError();
}

cudaError_t
launch_inv_dt(int dim, int b, const double * U, const DevMesh & m, const PhysParams & p, double * invdt, cudaStream_t s)
{
  if (dim == 2 && b == 16)
    return inv_dt_t<2, 16>(U, m, p, invdt, s);
  if (dim == 2 && b == 8)
    return inv_dt_t<2, 8>(U, m, p, invdt, s);
  if (dim == 3 && b == 8)
    return inv_dt_t<3, 8>(U, m, p, invdt, s);
  return cudaErrorInvalidValue;
}

template <int DIM, int B>
static cudaError_t
rk2_t(const double * U, double * U2, const DevMesh & m, const PhysParams & p, double * invdt, cudaStream_t s)
{
  if (m.n_owned == 0)
    return cudaSuccess;
  int grid = num_sms() * 8;
  if (grid > m.n_owned)
    grid = m.n_owned;
  rk2_combine_kernel<DIM, B, false><<<grid, 256, 0, s>>>(U, U2, m, p, invdt);
  return cudaGetLastError();
}

cudaError_t
launch_rk2_combine(int dim, int b, bool mixed, const double * U, double * U2, const DevMesh & m, const PhysParams & p, double * invdt,
                   cudaStream_t s)
{
  if (mixed)
    return launch_rk2_combine_mixed(dim, b, U, U2, m, p, invdt, s);
  if (dim == 2 && b == 16)
    return rk2_t<2, 16>(U, U2, m, p, invdt, s);
  if (dim == 2 && b == 8)
    return rk2_t<2, 8>(U, U2, m, p, invdt, s);
  if (dim == 3 && b == 8)
    return rk2_t<3, 8>(U, U2, m, p, invdt, s);
  return cudaErrorInvalidValue;
}

cudaError_t
launch_dt_update(double * invdt, double * dt, double * dt_hist, int n_inst, double cfl, cudaStream_t s)
{
  dt_update_kernel<<<(n_inst + 127) / 128, 128, 0, s>>>(invdt, dt, dt_hist, n_inst, cfl);
  return cudaGetLastError();
}

template <int DIM, int B>
static cudaError_t
flags_t(const double * U, const DevMesh & m, int ind, double er, double ec, double el, int lmin, int lmax, int8_t * flags, cudaStream_t s)
{
  if (m.n_owned == 0)
    return cudaSuccess;
  int grid = num_sms() * 8;
  if (grid > m.n_owned)
    grid = m.n_owned;
  refine_flags_kernel<DIM, B><<<grid, 256, 0, s>>>(U, m, ind, er, ec, el, lmin, lmax, flags);
  return cudaGetLastError();
}

cudaError_t
launch_refine_flags(int dim, int b, const double * U, const DevMesh & m, int indicator, double er, double ec, double el,
                    int lmin, int lmax, int8_t * flags, cudaStream_t s)
{
  if (dim == 2 && b == 16)
    return flags_t<2, 16>(U, m, indicator, er, ec, el, lmin, lmax, flags, s);
  if (dim == 2 && b == 8)
    return flags_t<2, 8>(U, m, indicator, er, ec, el, lmin, lmax, flags, s);
  if (dim == 3 && b == 8)
    return flags_t<3, 8>(U, m, indicator, er, ec, el, lmin, lmax, flags, s);
  return cudaErrorInvalidValue;
}

template <int DIM, int B>
static cudaError_t
remap_t(const double * Uold, double * Unew, const int8_t * kind, const int32_t * src, int n_new, cudaStream_t s)
{
  if (n_new == 0)
    return cudaSuccess;
  int grid = num_sms() * 8;
  if (grid > n_new)
    grid = n_new;
  remap_kernel<DIM, B><<<grid, 256, 0, s>>>(Uold, Unew, kind, src, n_new);
  return cudaGetLastError();
}

cudaError_t
launch_remap(int dim, int b, const double * Uold, double * Unew, const int8_t * kind, const int32_t * src, int n_new, cudaStream_t s)
{
  if (dim == 2 && b == 16)
    return remap_t<2, 16>(Uold, Unew, kind, src, n_new, s);
  if (dim == 2 && b == 8)
    return remap_t<2, 8>(Uold, Unew, kind, src, n_new, s);
  if (dim == 3 && b == 8)
    return remap_t<3, 8>(Uold, Unew, kind, src, n_new, s);
  return cudaErrorInvalidValue;
}

cudaError_t
launch_defer_info(int dim, const DevMesh & m, const int32_t * codes, int n, int32_t * info, cudaStream_t s)
{
  if (n <= 0)
    return cudaSuccess;
  if (dim == 2)
    defer_info_kernel<2><<<(n + 127) / 128, 128, 0, s>>>(m, codes, n, info);
  else
    defer_info_kernel<3><<<(n + 127) / 128, 128, 0, s>>>(m, codes, n, info);
  return cudaGetLastError();
}

template <int DIM, int B>
static cudaError_t
derived_t(const double * U, double * out, int quantity, long long oct_begin, long long num_octs, const PhysParams & p, cudaStream_t s)
{
  constexpr int   NC = DIM == 2 ? B * B : B * B * B;
  const long long total = num_octs * NC;
  if (total <= 0)
    return cudaSuccess;
  long long grid = (total + 255) / 256;
  if (grid > (long long)num_sms() * 16)
    grid = (long long)num_sms() * 16;
  derived_kernel<DIM, B><<<(unsigned)grid, 256, 0, s>>>(U, out, quantity, oct_begin, num_octs, p);
  return cudaGetLastError();
}

cudaError_t
launch_derived(int dim, int b, const double * U, double * out, int quantity, long long oct_begin, long long num_octs, const PhysParams & p,
               cudaStream_t s)
{
  if (dim == 2 && b == 16)
    return derived_t<2, 16>(U, out, quantity, oct_begin, num_octs, p, s);
  if (dim == 2 && b == 8)
    return derived_t<2, 8>(U, out, quantity, oct_begin, num_octs, p, s);
  if (dim == 3 && b == 8)
    return derived_t<3, 8>(U, out, quantity, oct_begin, num_octs, p, s);
  return cudaErrorInvalidValue;
}

template <int DIM, int B>
static cudaError_t
pack_fields_t(const double * U, double * out, const FieldList & fl, long long oct_begin, long long num_octs, const PhysParams & p,
              cudaStream_t s)
{
  constexpr int   NC = DIM == 2 ? B * B : B * B * B;
  const long long total = num_octs * NC;
  if (total <= 0)
    return cudaSuccess;
  long long grid = (total + 255) / 256;
  if (grid > (long long)num_sms() * 16)
    grid = (long long)num_sms() * 16;
  pack_fields_kernel<DIM, B><<<(unsigned)grid, 256, 0, s>>>(U, out, fl, oct_begin, num_octs, p);
  return cudaGetLastError();
}

cudaError_t
launch_pack_fields(int dim, int b, const double * U, double * out, const int * codes, int n, long long oct_begin, long long num_octs,
                   const PhysParams & p, cudaStream_t s)
{
  if (n < 1 || n > MAX_PACK_FIELDS)
    return cudaErrorInvalidValue;
  FieldList fl;
  fl.n = n;
  for (int k = 0; k < MAX_PACK_FIELDS; ++k)
    fl.code[k] = k < n ? codes[k] : 0;
  if (dim == 2 && b == 16)
    return pack_fields_t<2, 16>(U, out, fl, oct_begin, num_octs, p, s);
  if (dim == 2 && b == 8)
    return pack_fields_t<2, 8>(U, out, fl, oct_begin, num_octs, p, s);
  if (dim == 3 && b == 8)
    return pack_fields_t<3, 8>(U, out, fl, oct_begin, num_octs, p, s);
  return cudaErrorInvalidValue;
}

} // namespace g5
