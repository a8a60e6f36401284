// g5_static.cu — g5_step_static: the timestep for callers that cannot
// allocate device memory.
//
// Some host codes cannot call cudaMalloc on the path that advances the
// solution: a solver whose device memory is owned by a pool allocator of its
// own framework (cudaMalloc there would fragment or bypass the pool, or is
// forbidden), code that runs between a framework's capture-safe allocation
// phases, or a plugin loaded into a process that budgets every device
// allocation.  g5_step_static gives them the same step as g5_step without a
// context: everything the step needs besides the caller's inputs and outputs
// (the dt copy, the block table, the coarse/fine face records and the status
// word) lives in one file-scope device array of fixed size,
// G5_STATIC_SCRATCH_BYTES, which every GPU that loads the library holds until
// the process exits.
#include <cstddef>
#include <cstring>
#include <mutex>

#include <cuda_runtime.h>

#include "../../include/g5gpu.h"
#include "g5_launch.h"
#include "g5_phys.h"

namespace
{

// The scratch of g5_step_static.  In host code this name is only a host-side
// stand-in for the symbol; its device address comes from
// cudaGetSymbolAddress (see static_scratch_address).
static __device__ __align__(256) unsigned char g5_static_scratch[G5_STATIC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex    g_mutex;
void *        g_addr[kMaxDevices] = {};

// Device address of the scratch array on the current device, looked up once
// per device with that device current.
int
static_scratch_address(unsigned char ** out)
{
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return G5_ERR_CUDA;
  std::lock_guard<std::mutex> lock(g_mutex);
  if (!g_addr[dev])
  {
    void * p = nullptr;
    if (cudaGetSymbolAddress(&p, g5_static_scratch) != cudaSuccess || !p)
      return G5_ERR_CUDA;
    g_addr[dev] = p;
  }
  *out = static_cast<unsigned char *>(g_addr[dev]);
  return G5_OK;
}

size_t
align256(size_t x)
{
  return (x + 255) & ~(size_t)255;
}

// host -> scratch copy of a caller array.  From pageable memory (the stack
// buffers of the face records, and most callers' tables) cudaMemcpyAsync
// returns once the bytes are staged, so the source may be reused at once; a
// page-locked source is read later, when the stream reaches the copy, so the
// caller must leave it unchanged until then.
int
put(unsigned char * base, size_t off, const void * src, size_t bytes, cudaStream_t s)
{
  if (bytes == 0)
    return G5_OK;
  return cudaMemcpyAsync(base + off, src, bytes, cudaMemcpyHostToDevice, s) == cudaSuccess ? G5_OK : G5_ERR_CUDA;
}

} // namespace

extern "C" int
g5_step_static(const G5Params * params,
               const G5Mesh *   mesh,
               const double *   d_U,
               double *         d_U2,
               const double *   dt_host,
               int              mode,
               double *         d_inv_dt_out,
               unsigned int *   d_status_out,
               void *           stream)
{
  if (!params || !mesh || !d_U || !d_U2 || !dt_host || d_U == d_U2)
    return G5_ERR_ARG;
  if (mode != G5_MODE_FP64 && mode != G5_MODE_MIXED)
    return G5_ERR_ARG;
  const int dim = params->dim, b = params->bsize;
  if ((dim != 2 && dim != 3) || b < 4 || (b & 1))
    return G5_ERR_ARG;
  if (!g5::step_supported(dim, b))
    return G5_ERR_UNSUPPORTED;
  if ((params->integrator != 0 && params->integrator != 1) || params->source_term != 0 || params->prolongation != 0)
    return G5_ERR_UNSUPPORTED;
  if (!(params->gamma[0] > 1.0) || !(params->gamma[1] > 1.0) || !g5::eos_params_valid(params))
    return G5_ERR_ARG;
  const int n_owned = mesh->n_owned, n_outside = mesh->n_outside;
  const int n_total = n_owned + n_outside, n_inst = mesh->n_inst > 0 ? mesh->n_inst : 1;
  if (n_owned <= 0 || n_outside < 0 || !mesh->level || !mesh->coord || !mesh->nbr || !mesh->nbr_rel)
    return G5_ERR_ARG;
  const int ns = dim == 2 ? 9 : 27, nch = dim == 2 ? 4 : 8, nfaces = 2 * dim;
  for (int i = 0; i < n_inst; ++i)
    if (!(dt_host[i] > 0.0))
      return G5_ERR_ARG;
  // the host arrays are staged at call time (copies from host memory, some
  // from this function's stack): refuse a stream in capture mode rather than
  // record copies whose sources are gone when the graph runs
  {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing((cudaStream_t)stream, &cs) != cudaSuccess)
      return G5_ERR_CUDA;
    if (cs != cudaStreamCaptureStatusNone)
      return G5_ERR_UNSUPPORTED;
  }

  // ---- validate the table (the same check as g5_set_mesh) and count the
  // coarse/fine face records
  if (n_outside > 0 && !mesh->out_src)
    return G5_ERR_ARG;
  if (g5::validate_table(dim, mesh) != G5_OK)
    return G5_ERR_MESH;
  int n_reflux = 0, n_defer = 0;
  for (int n = 0; n < n_owned; ++n)
    for (int f = 0; f < nfaces; ++f)
    {
      int d[3] = { 0, 0, 0 };
      d[f >> 1] = (f & 1) ? 1 : -1;
      const int   s = (d[0] + 1) + 3 * (d[1] + 1) + (dim == 3 ? 9 * (d[2] + 1) : 0);
      const int   rel = mesh->nbr_rel[(size_t)n * ns + s];
      const int * nb = mesh->nbr + ((size_t)n * ns + s) * nch;
      if (rel < 0 && nb[0] < n_owned)
        ++n_reflux;
      if (rel > 0)
      {
        bool owned = true;
        for (int ch = 0; ch < nch; ++ch)
          if (nb[ch] >= n_owned)
            owned = false;
        n_defer += owned ? 1 : 0;
      }
    }

  // ---- scratch layout; refuse meshes that do not fit
  const size_t face_cells = dim == 2 ? (size_t)b : (size_t)b * b;
  const size_t nf = dim == 2 ? 8 : 9;
  size_t       off = 0;
  const size_t o_status = off;
  off = align256(off + sizeof(unsigned int));
  const size_t o_dt = off;
  off = align256(off + sizeof(double) * n_inst);
  const size_t o_level = off;
  off = align256(off + sizeof(int32_t) * n_total);
  const size_t o_coord = off;
  off = align256(off + sizeof(int32_t) * 3 * n_total);
  const size_t o_nbr = off;
  off = align256(off + sizeof(int32_t) * (size_t)n_owned * ns * nch);
  const size_t o_rel = off;
  off = align256(off + (size_t)n_owned * ns);
  const size_t o_inst = off;
  off = align256(off + (mesh->inst ? sizeof(int32_t) * n_total : 0));
  const size_t o_rslot = off;
  off = align256(off + (n_defer > 0 ? sizeof(int32_t) * (size_t)n_owned * nfaces : 0));
  const size_t o_dslot = off;
  off = align256(off + (n_defer > 0 ? sizeof(int32_t) * (size_t)n_owned * nfaces : 0));
  const size_t o_dlist = off;
  off = align256(off + sizeof(int32_t) * (size_t)n_defer);
  const size_t o_dinfo = off; // DeferInfo rows of the reflux pass, built on the device
  off = align256(off + sizeof(int32_t) * (size_t)n_defer * (dim == 2 ? g5::DeferInfo<2>::STRIDE : g5::DeferInfo<3>::STRIDE));
  const size_t o_rbuf = off;
  off = align256(off + sizeof(double) * (size_t)n_reflux * face_cells * nf);
  const size_t o_dbuf = off;
  off = align256(off + sizeof(double) * (size_t)n_defer * face_cells * nfaces * nf);
  if (off > (size_t)G5_STATIC_SCRATCH_BYTES)
    return G5_ERR_ARG; // the mesh needs more scratch than the fixed array holds

  unsigned char * base = nullptr;
  int             rc = static_scratch_address(&base);
  if (rc)
    return rc;
  cudaStream_t s = (cudaStream_t)stream;

  // ---- stage dt and the block table in the scratch
  rc |= put(base, o_dt, dt_host, sizeof(double) * n_inst, s);
  rc |= put(base, o_level, mesh->level, sizeof(int32_t) * n_total, s);
  rc |= put(base, o_coord, mesh->coord, sizeof(int32_t) * 3 * n_total, s);
  rc |= put(base, o_nbr, mesh->nbr, sizeof(int32_t) * (size_t)n_owned * ns * nch, s);
  rc |= put(base, o_rel, mesh->nbr_rel, (size_t)n_owned * ns, s);
  if (mesh->inst)
    rc |= put(base, o_inst, mesh->inst, sizeof(int32_t) * n_total, s);
  if (rc)
    return G5_ERR_CUDA;
  if (n_defer > 0)
  {
    // face record slots, streamed through a small stack buffer
    constexpr int kChunk = 1024;
    int32_t       rs[kChunk], ds[kChunk], dl[kChunk];
    int           nr = 0, nd = 0, fill = 0, lfill = 0;
    size_t        slot_off = 0, list_off = 0;
    for (int n = 0; n < n_owned; ++n)
      for (int f = 0; f < nfaces; ++f)
      {
        int d[3] = { 0, 0, 0 };
        d[f >> 1] = (f & 1) ? 1 : -1;
        const int   sl = (d[0] + 1) + 3 * (d[1] + 1) + (dim == 3 ? 9 * (d[2] + 1) : 0);
        const int   rel = mesh->nbr_rel[(size_t)n * ns + sl];
        const int * nb = mesh->nbr + ((size_t)n * ns + sl) * nch;
        rs[fill] = (rel < 0 && nb[0] < n_owned) ? nr++ : -1;
        ds[fill] = -1;
        if (rel > 0)
        {
          bool owned = true;
          for (int ch = 0; ch < nch; ++ch)
            if (nb[ch] >= n_owned)
              owned = false;
          if (owned)
          {
            ds[fill] = nd++;
            dl[lfill++] = n * 8 + f;
          }
        }
        if (++fill == kChunk)
        {
          rc |= put(base, o_rslot + slot_off, rs, sizeof(int32_t) * fill, s);
          rc |= put(base, o_dslot + slot_off, ds, sizeof(int32_t) * fill, s);
          slot_off += sizeof(int32_t) * fill;
          fill = 0;
        }
        if (lfill == kChunk)
        {
          rc |= put(base, o_dlist + list_off, dl, sizeof(int32_t) * lfill, s);
          list_off += sizeof(int32_t) * lfill;
          lfill = 0;
        }
      }
    rc |= put(base, o_rslot + slot_off, rs, sizeof(int32_t) * fill, s);
    rc |= put(base, o_dslot + slot_off, ds, sizeof(int32_t) * fill, s);
    rc |= put(base, o_dlist + list_off, dl, sizeof(int32_t) * lfill, s);
    if (rc)
      return G5_ERR_CUDA;
  }
  unsigned int * status = d_status_out ? d_status_out : reinterpret_cast<unsigned int *>(base + o_status);
  if (!d_status_out && cudaMemsetAsync(status, 0, sizeof(unsigned int), s) != cudaSuccess)
    return G5_ERR_CUDA;

  // ---- the step, with every scratch pointer inside the static array
  const g5::PhysParams p = g5::make_phys(params);

  g5::StepArgs a;
  std::memset(&a, 0, sizeof(a));
  a.U = d_U;
  a.U2 = d_U2;
  a.dt = reinterpret_cast<const double *>(base + o_dt);
  a.reflux_buf = n_defer > 0 ? reinterpret_cast<double *>(base + o_rbuf) : nullptr;
  a.defer_buf = n_defer > 0 ? reinterpret_cast<double *>(base + o_dbuf) : nullptr;
  a.invdt = d_inv_dt_out;
  a.status = status;
  a.p = p;
  a.m.level = reinterpret_cast<const int32_t *>(base + o_level);
  a.m.coord = reinterpret_cast<const int32_t *>(base + o_coord);
  a.m.nbr = reinterpret_cast<const int32_t *>(base + o_nbr);
  a.m.nbr_rel = reinterpret_cast<const int8_t *>(base + o_rel);
  a.m.inst = mesh->inst ? reinterpret_cast<const int32_t *>(base + o_inst) : nullptr;
  a.m.reflux_slot = n_defer > 0 ? reinterpret_cast<const int32_t *>(base + o_rslot) : nullptr;
  a.m.defer_slot = n_defer > 0 ? reinterpret_cast<const int32_t *>(base + o_dslot) : nullptr;
  a.m.defer_list = n_defer > 0 ? reinterpret_cast<const int32_t *>(base + o_dlist) : nullptr;
  a.m.defer_info = n_defer > 0 ? reinterpret_cast<const int32_t *>(base + o_dinfo) : nullptr;
  a.m.n_owned = n_owned;
  a.m.n_outside = n_outside;
  a.m.n_total = n_total;
  a.m.n_inst = n_inst;
  a.m.n_defer = n_defer;
  if (n_defer > 0 &&
      g5::launch_defer_info(dim, a.m, a.m.defer_list, n_defer, reinterpret_cast<int32_t *>(base + o_dinfo), s) != cudaSuccess)
    return G5_ERR_CUDA;
  int         launches = 0;
  cudaError_t e = mode == G5_MODE_FP64 ? g5::launch_step_fp64(dim, b, a, 0, s, &launches)
                                       : g5::launch_step_mixed(dim, b, a, 0, s, &launches);
  return e == cudaSuccess ? G5_OK : G5_ERR_CUDA;
}
