// g5_mixed.cu — FP32-bulk instantiations of the 2D step (fast FP32 math; FP64
// kept for the pressure numerator, the accumulation into U2, the
// renormalisation and dt) and the dispatch of every FP32-bulk step; the 3D
// kernels are in g5_mixed3d.cu.
#include "g5_aux.cuh"
#include "g5_launch.h"
#include "g5_step2d.cuh"

namespace g5
{

static int
num_sms_m()
{
  static int n = 0;
  if (n == 0)
  {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (n <= 0)
      n = 1;
  }
  return n;
}

// the persistent step kernel of one case (FUSED: the coarse/fine records
// finished in its tail, m.fin_tgt set)
template <int B, bool THINC, int STIFF, bool FUSED>
static cudaError_t
launch_step2d_kernel_m(const StepArgs & a, int ctas_per_sm, cudaStream_t s, int * launches)
{
  using T = Step2DTraits<B, true>;
  static bool configured = false;
  static int  occ = 1;
  if (!configured)
  {
    cudaError_t e =
      cudaFuncSetAttribute(step2d_kernel<B, true, THINC, STIFF, FUSED>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)T::smem_bytes);
    if (e != cudaSuccess)
      return e;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, step2d_kernel<B, true, THINC, STIFF, FUSED>, T::NT, T::smem_bytes);
    if (occ < 1)
      occ = 1;
    configured = true;
  }
  const int per_sm = (ctas_per_sm > 0 && ctas_per_sm < occ) ? ctas_per_sm : occ;
  int       grid = num_sms_m() * per_sm;
  if (grid > step_count(a))
    grid = step_count(a);
  if (grid < 1)
    return cudaSuccess;
  step2d_kernel<B, true, THINC, STIFF, FUSED><<<grid, T::NT, T::smem_bytes, s>>>(a);
  ++*launches;
  return cudaGetLastError();
}

template <int B, bool THINC, int STIFF>
static cudaError_t
launch_step2d_m(const StepArgs & a, int ctas_per_sm, cudaStream_t s, int * launches)
{
  cudaError_t e = a.m.fin_tgt ? launch_step2d_kernel_m<B, THINC, STIFF, true>(a, ctas_per_sm, s, launches)
                              : launch_step2d_kernel_m<B, THINC, STIFF, false>(a, ctas_per_sm, s, launches);
  if (e != cudaSuccess)
    return e;
  if (a.m.fin_tgt)
    return e; // the step kernel's tail finished the deferred cells
  if (a.m.n_defer > 0 && a.reflux_layout == 1)
  {
    const int n = a.m.n_defer * B;
    reflux2d_kernel<B, true><<<(n + 31) / 32, 32, 0, s>>>(a);
    ++*launches;
    e = cudaGetLastError();
  }
  else if (a.m.n_defer > 0)
  {
    // 8 lanes per deferred cell
    const int n = a.m.n_defer * B * 8;
    reflux2d_mixed_lanes_kernel<B><<<(n + 127) / 128, 128, 0, s>>>(a);
    ++*launches;
    e = cudaGetLastError();
  }
  return e;
}

template <int B>
static int
occupancy2d_m()
{
  using T = Step2DTraits<B, true>;
  int occ = 1 << 20;
  auto one = [&](const void * k) {
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)T::smem_bytes);
    int o = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, k, T::NT, T::smem_bytes);
    occ = o < occ ? o : occ;
  };
  one((const void *)step2d_kernel<B, true, false, 0>);
  one((const void *)step2d_kernel<B, true, false, 1>);
  one((const void *)step2d_kernel<B, true, true, 0>);
  one((const void *)step2d_kernel<B, true, true, 1>);
  one((const void *)step2d_kernel<B, true, false, 2>);
  one((const void *)step2d_kernel<B, true, true, 2>);
  one((const void *)step2d_kernel<B, true, false, 0, true>);
  one((const void *)step2d_kernel<B, true, false, 1, true>);
  one((const void *)step2d_kernel<B, true, true, 0, true>);
  one((const void *)step2d_kernel<B, true, true, 1, true>);
  one((const void *)step2d_kernel<B, true, false, 2, true>);
  one((const void *)step2d_kernel<B, true, true, 2, true>);
  return occ;
}

template <int DIM, int B>
static cudaError_t
rk2_m(const double * U, double * U2, const DevMesh & m, const PhysParams & p, double * invdt, cudaStream_t s)
{
  if (m.n_owned == 0)
    return cudaSuccess;
  int grid = num_sms_m() * 8;
  if (grid > m.n_owned)
    grid = m.n_owned;
  rk2_combine_kernel<DIM, B, true><<<grid, 256, 0, s>>>(U, U2, m, p, invdt);
  return cudaGetLastError();
}

cudaError_t
launch_rk2_combine_mixed(int dim, int b, const double * U, double * U2, const DevMesh & m, const PhysParams & p, double * invdt,
                         cudaStream_t s)
{
  if (dim == 2 && b == 16)
    return rk2_m<2, 16>(U, U2, m, p, invdt, s);
  if (dim == 2 && b == 8)
    return rk2_m<2, 8>(U, U2, m, p, invdt, s);
  if (dim == 3 && b == 8)
    return rk2_m<3, 8>(U, U2, m, p, invdt, s);
  return cudaErrorInvalidValue;
}

cudaError_t
launch_step_mixed(int dim, int b, const StepArgs & a, int ctas_per_sm, cudaStream_t s, int * launches)
{
  const cudaError_t e = launch_prolong(dim, b, a, s, launches);
  if (e != cudaSuccess)
    return e;
  // one kernel per case: THINC on or off, and the equation of state (0 ideal
  // gases, 1 a stiffened-gas constant, 2 Mie-Grueneisen laws)
  const int eosk = a.p.mg_any ? 2 : ((a.p.gpx[0] != 0.0 || a.p.gpx[1] != 0.0) ? 1 : 0);
  const int v = (a.p.thinc ? 3 : 0) + eosk;
  if (dim == 3 && b == 8)
    return launch_step3d_mixed_case(v, a, ctas_per_sm, s, launches);
  if (dim == 2 && b == 16)
  {
    switch (v)
    {
      case 0: return launch_step2d_m<16, false, 0>(a, ctas_per_sm, s, launches);
      case 1: return launch_step2d_m<16, false, 1>(a, ctas_per_sm, s, launches);
      case 2: return launch_step2d_m<16, false, 2>(a, ctas_per_sm, s, launches);
      case 3: return launch_step2d_m<16, true, 0>(a, ctas_per_sm, s, launches);
      case 4: return launch_step2d_m<16, true, 1>(a, ctas_per_sm, s, launches);
      default: return launch_step2d_m<16, true, 2>(a, ctas_per_sm, s, launches);
    }
  }
  if (dim == 2 && b == 8)
  {
    switch (v)
    {
      case 0: return launch_step2d_m<8, false, 0>(a, ctas_per_sm, s, launches);
      case 1: return launch_step2d_m<8, false, 1>(a, ctas_per_sm, s, launches);
      case 2: return launch_step2d_m<8, false, 2>(a, ctas_per_sm, s, launches);
      case 3: return launch_step2d_m<8, true, 0>(a, ctas_per_sm, s, launches);
      case 4: return launch_step2d_m<8, true, 1>(a, ctas_per_sm, s, launches);
      default: return launch_step2d_m<8, true, 2>(a, ctas_per_sm, s, launches);
    }
  }
  return cudaErrorInvalidValue;
}

int
step_max_ctas_per_sm_mixed(int dim, int b)
{
  if (dim == 2 && b == 16)
    return occupancy2d_m<16>();
  if (dim == 2 && b == 8)
    return occupancy2d_m<8>();
  if (dim == 3 && b == 8)
    return step_max_ctas_per_sm_mixed3d();
  return 0;
}

} // namespace g5
