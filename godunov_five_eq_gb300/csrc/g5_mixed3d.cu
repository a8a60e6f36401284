// g5_mixed3d.cu — FP32-bulk instantiations of the 3D step (8^3 blocks) and
// its coarse/fine reflux pass (a translation unit of its own so that the
// library's units compile side by side).
#include "g5_aux.cuh"
#include "g5_launch.h"
#include "g5_step3d.cuh"

namespace g5
{

static int
num_sms_m3()
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

template <int THINC, int STIFF>
static cudaError_t
launch_step3d_m(const StepArgs & a, int ctas_per_sm, cudaStream_t s, int * launches)
{
  using T = Step3DTraits<true>;
  static bool configured = false;
  static int  occ = 1;
  if (!configured)
  {
    cudaError_t e = cudaFuncSetAttribute(step3d_kernel<true, THINC, STIFF>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)T::smem_bytes);
    if (e != cudaSuccess)
      return e;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, step3d_kernel<true, THINC, STIFF>, T::NT, T::smem_bytes);
    if (occ < 1)
      occ = 1;
    configured = true;
  }
  const int per_sm = (ctas_per_sm > 0 && ctas_per_sm < occ) ? ctas_per_sm : occ;
  int       grid = num_sms_m3() * per_sm;
  if (grid > step_count(a))
    grid = step_count(a);
  cudaError_t e = cudaSuccess;
  if (grid >= 1)
  {
    step3d_kernel<true, THINC, STIFF><<<grid, T::NT, T::smem_bytes, s>>>(a);
    ++*launches;
    e = cudaGetLastError();
    if (e != cudaSuccess)
      return e;
  }
  if (a.m.n_defer > 0)
  {
    const int n = a.m.n_defer * 64;
    reflux3d_kernel<true><<<(n + 31) / 32, 32, 0, s>>>(a);
    ++*launches;
    e = cudaGetLastError();
  }
  return e;
}

cudaError_t
launch_step3d_mixed_case(int v, const StepArgs & a, int ctas_per_sm, cudaStream_t s, int * launches)
{
  switch (v)
  {
    case 0: return launch_step3d_m<0, 0>(a, ctas_per_sm, s, launches);
    case 1: return launch_step3d_m<0, 1>(a, ctas_per_sm, s, launches);
    case 2: return launch_step3d_m<0, 2>(a, ctas_per_sm, s, launches);
    case 3: return launch_step3d_m<1, 0>(a, ctas_per_sm, s, launches);
    case 4: return launch_step3d_m<1, 1>(a, ctas_per_sm, s, launches);
    default: return launch_step3d_m<1, 2>(a, ctas_per_sm, s, launches);
  }
}

int
step_max_ctas_per_sm_mixed3d()
{
  using T = Step3DTraits<true>;
  int  occ = 1 << 20;
  auto one = [&](const void * k) {
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)T::smem_bytes);
    int o = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, k, T::NT, T::smem_bytes);
    occ = o < occ ? o : occ;
  };
  one((const void *)step3d_kernel<true, 0, 0>);
  one((const void *)step3d_kernel<true, 0, 1>);
  one((const void *)step3d_kernel<true, 1, 0>);
  one((const void *)step3d_kernel<true, 1, 1>);
  one((const void *)step3d_kernel<true, 0, 2>);
  one((const void *)step3d_kernel<true, 1, 2>);
  return occ;
}

} // namespace g5
