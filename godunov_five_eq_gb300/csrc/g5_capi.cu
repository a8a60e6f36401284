// g5_capi.cu — the C ABI (include/g5gpu.h): context, block-table upload,
// scratch sizing, launches, the graph-replayed solver loop and the autotuner.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/g5gpu.h"
#include "g5_launch.h"
#include "g5_phys.h"

struct G5Context
{
  G5Params       prm;
  g5::PhysParams phys;
  int            dim = 2, b = 16, nv = 8, ns = 9, nch = 4;
  int            device = 0;
  bool           has_mesh = false;
  int            n_owned = 0, n_outside = 0, n_total = 0, n_inst = 1;
  int            n_defer = 0, n_reflux = 0;
  // device block table
  int32_t *d_level = nullptr, *d_coord = nullptr, *d_nbr = nullptr, *d_inst = nullptr;
  int32_t *d_reflux_slot = nullptr, *d_defer_slot = nullptr, *d_defer_list = nullptr, *d_out_src = nullptr;
  int32_t * d_defer_info = nullptr; // DeferInfo rows, in the order of d_defer_list
  int32_t * d_twin_first = nullptr, *d_twin_list = nullptr; // outside blocks per owned source block
  int32_t * d_walk = nullptr;                                // block order of the full-mesh step
  int32_t * d_pg_slot = nullptr;                             // prolonged-ghost slot per owned block (DevMesh::pg_slot)
  double *  d_pg = nullptr;                                  // prolonged ghost states (DevMesh::pg)
  bool      fused_fill = false;                              // the 2D solver loop fills them in the step
  int8_t * d_nbr_rel = nullptr, *d_out_normal = nullptr, *d_out_border = nullptr;
  // scratch
  double *       d_reflux_buf = nullptr, *d_defer_buf = nullptr;
  double *       d_dt = nullptr, *d_invdt = nullptr;
  double *       d_urk = nullptr; // RK2_SSP intermediate stage (SolverGodunovFiveEq.h:349-358 m_U_RK)
  unsigned int * d_ticket = nullptr; // block claiming counter of the step kernels (zero between launches)
  // reflux in the tail of the FP32-bulk 2D full-mesh step (DevMesh::fin_*)
  int32_t *      d_fin_tgt = nullptr, *d_fin_rec = nullptr;
  unsigned int * d_fin_cnt = nullptr, *d_fin_init = nullptr, *d_fin_ticket = nullptr;
  int            n_fin = 0;
  // g5_step_batched: owned blocks grouped by instance (host), the call's work
  // list and instance mask (device)
  std::vector<int32_t> inst_blocks, inst_off;
  int32_t *            d_batch_work = nullptr;
  uint8_t *            d_inst_active = nullptr;
  unsigned int * d_status = nullptr;
  int64_t        bytes = 0;
  struct PoolEntry
  {
    void * p = nullptr;
    size_t cap = 0;
  };
  std::unordered_map<const void *, PoolEntry> pool; // device buffers by field (dev_alloc)
  // launch shape of the step per precision mode (g5_tune): CTAs per SM (0:
  // occupancy maximum), dynamic block claiming, walk order (1: blocks with
  // coarse/fine neighbours first, 0: table order), reflux layout (2: the
  // step kernel's tail where the FP32-bulk 2D full-mesh step has records,
  // otherwise the separate pass with 8 lanes per cell)
  struct Shape
  {
    int ctas_per_sm = 0;
    int claim = 1;
    int walk = 1;
    int reflux = 2;
  };
  Shape          shape[2];
  std::vector<std::pair<int, float>> tune_log[2]; // (packed shape, ms per step) of the last g5_tune
  int            last_launches = 0;
  // cached one-step graphs of g5_advance
  struct GraphSlot
  {
    cudaGraphExec_t exec = nullptr;
    const void *    U = nullptr;
    const void *    U2 = nullptr;
    const void *    dt_out = nullptr;
    int             mode = -1;
    int             launches = 0;
  };
  static constexpr int kGraphs = 4;
  GraphSlot            graphs[kGraphs];
  int                  next_graph = 0;
  // g5_step_host: U and U2 in host memory, copies pipelined with the step.
  // The owned blocks are cut into K copy chunks; launch k steps the blocks
  // whose own and neighbour data have arrived once chunk k is in, then the
  // coarse/fine records whose blocks are all stepped; U2 chunks are copied
  // back as soon as their last block is final.
  struct HostPipe
  {
    int                  K = 0;
    std::vector<int>     lo;       // [K+1] owned-block bounds of the copy chunks
    std::vector<int>     work_off; // [K+1] launch k steps d_work[work_off[k] .. work_off[k+1])
    std::vector<int>     rec_off;  // [K+1] launch k refluxes records rec_off[k] .. rec_off[k+1] of d_defer_info
    std::vector<int>     out_off;  // [K+1] after launch k copy back chunks out_list[out_off[k] .. out_off[k+1])
    std::vector<int>     out_list;
    int32_t *            d_work = nullptr;
    std::vector<int32_t> recs; // record codes in launch order (the order of d_defer_list)
    double *             d_U = nullptr;  // staging of U, n_total blocks (first g5_step_host call)
    double *             d_U2 = nullptr; // staging of U2, n_owned blocks
    static constexpr int kComputeStreams = 8;
    cudaStream_t         s_in = nullptr, s_out = nullptr, s_c[kComputeStreams] = {};
    cudaEvent_t          ev_start = nullptr, ev_out = nullptr, ev_dt_read = nullptr;
    std::vector<cudaEvent_t> ev_in, ev_step, ev_comp;
    double *             h_dt_stage = nullptr;  // pinned copy of dt_host read by the (captured) step
    double *             h_inv_stage = nullptr; // pinned landing of the CFL rate
    int                  n_stage = 0;
    bool                 dt_pending = false; // a launched step may still read h_dt_stage
    struct InvCopy
    {
      double *       dst = nullptr;
      const double * src = nullptr;
      size_t         bytes = 0;
    };
    struct Graph
    {
      cudaGraphExec_t exec = nullptr;
      const void *    hU = nullptr;
      const void *    hU2 = nullptr;
      const void *    inv = nullptr;
      int             mode = -1;
      int             launches = 0;
      InvCopy         inv_copy;
    };
    static constexpr int kGraphs = 4;
    Graph                graphs[kGraphs];
    int                  next_graph = 0;
  } pipe;
};

namespace
{

// Device buffers of the context, one per field (keyed by the field's
// address): a new mesh reuses a buffer that is large enough, so that an AMR
// cycle's table upload costs copies, not frees (each a device-wide
// synchronisation) and allocations.  The pool is released by g5_destroy.
template <typename T>
int
dev_alloc(G5Context * c, T ** p, size_t count)
{
  *p = nullptr;
  if (count == 0)
    return G5_OK;
  const size_t           bytes = count * sizeof(T);
  G5Context::PoolEntry & e = c->pool[(const void *)p];
  if (e.p && e.cap >= bytes)
  {
    *p = static_cast<T *>(e.p);
    return G5_OK;
  }
  if (e.p)
  {
    cudaFree(e.p);
    c->bytes -= (int64_t)e.cap;
    e = G5Context::PoolEntry();
  }
  void * np = nullptr;
  if (cudaMalloc(&np, bytes) != cudaSuccess)
    return G5_ERR_CUDA;
  e.p = np;
  e.cap = bytes;
  c->bytes += (int64_t)bytes;
  *p = static_cast<T *>(np);
  return G5_OK;
}

void
free_pool(G5Context * c)
{
  for (auto & kv : c->pool)
    if (kv.second.p)
      cudaFree(kv.second.p);
  c->pool.clear();
  c->bytes = c->d_status ? (int64_t)sizeof(unsigned int) : 0;
}

template <typename T>
int
dev_upload(G5Context * c, T ** p, const T * host, size_t count)
{
  int rc = dev_alloc(c, p, count);
  if (rc || count == 0)
    return rc;
  if (cudaMemcpy(*p, host, count * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess)
    return G5_ERR_CUDA;
  return G5_OK;
}

void
drop_graphs(G5Context * c)
{
  for (auto & g : c->graphs)
  {
    if (g.exec)
      cudaGraphExecDestroy(g.exec);
    g = G5Context::GraphSlot();
  }
}

// the context forgets its mesh; the buffers stay in the pool for the next one
void
free_mesh(G5Context * c)
{
  c->d_level = c->d_coord = c->d_nbr = c->d_inst = nullptr;
  c->d_reflux_slot = c->d_defer_slot = c->d_defer_list = c->d_out_src = nullptr;
  c->d_nbr_rel = c->d_out_normal = c->d_out_border = nullptr;
  c->d_reflux_buf = c->d_defer_buf = c->d_dt = c->d_invdt = nullptr;
  c->d_ticket = nullptr;
  c->d_fin_tgt = c->d_fin_rec = nullptr;
  c->d_fin_cnt = c->d_fin_init = c->d_fin_ticket = nullptr;
  c->n_fin = 0;
  c->d_batch_work = nullptr;
  c->d_inst_active = nullptr;
  c->inst_blocks.clear();
  c->inst_off.clear();
  c->d_urk = nullptr;
  c->d_defer_info = nullptr;
  c->d_twin_first = c->d_twin_list = c->d_walk = c->d_pg_slot = nullptr;
  c->d_pg = nullptr;
  c->fused_fill = false;
  c->pipe.d_work = nullptr;
  c->pipe.d_U = c->pipe.d_U2 = nullptr;
  c->pipe.K = 0;
  for (auto & g : c->pipe.graphs)
  {
    if (g.exec)
      cudaGraphExecDestroy(g.exec);
    g = G5Context::HostPipe::Graph();
  }
  drop_graphs(c);
  c->has_mesh = false;
}

g5::DevMesh
dev_mesh(const G5Context * c)
{
  g5::DevMesh m;
  m.level = c->d_level;
  m.coord = c->d_coord;
  m.nbr = c->d_nbr;
  m.nbr_rel = c->d_nbr_rel;
  m.inst = c->d_inst;
  m.reflux_slot = (c->n_defer > 0) ? c->d_reflux_slot : nullptr;
  m.defer_slot = (c->n_defer > 0) ? c->d_defer_slot : nullptr;
  m.defer_list = c->d_defer_list;
  m.defer_info = c->d_defer_info;
  m.twin_first = c->d_twin_first;
  m.twin_list = c->d_twin_list;
  m.out_src = c->d_out_src;
  m.out_normal = c->d_out_normal;
  m.out_border = c->d_out_border;
  m.n_owned = c->n_owned;
  m.n_outside = c->n_outside;
  m.n_total = c->n_total;
  m.n_inst = c->n_inst;
  m.n_defer = c->n_defer;
  m.pg_slot = c->d_pg_slot;
  m.pg = c->d_pg;
  return m;
}

int
do_step(G5Context * c, const double * U, double * U2, const double * d_dt, int mode, double * invdt, cudaStream_t s, bool fill_twins = false)
{
  if (!c || !c->has_mesh || !U || !U2 || !d_dt)
    return G5_ERR_ARG;
  if (mode != G5_MODE_FP64 && mode != G5_MODE_MIXED)
    return G5_ERR_ARG;
  if (!g5::step_supported(c->dim, c->b))
    return G5_ERR_UNSUPPORTED;
  g5::StepArgs a;
  a.U = U;
  a.U2 = U2;
  a.dt = d_dt;
  a.reflux_buf = c->d_reflux_buf;
  a.defer_buf = c->d_defer_buf;
  a.invdt = invdt;
  a.status = c->d_status;
  a.m = dev_mesh(c);
  a.p = c->phys;
  a.fill_twins = fill_twins ? 1 : 0;
  const G5Context::Shape & sh = c->shape[mode];
  a.ticket = sh.claim ? c->d_ticket : nullptr;
  a.work = sh.walk ? c->d_walk : nullptr;
  a.n_work = sh.walk ? c->n_owned : 0;
  a.reflux_layout = sh.reflux;
  if (mode == G5_MODE_MIXED && sh.reflux == 2 && c->n_fin > 0)
  {
    a.m.fin_tgt = c->d_fin_tgt;
    a.m.fin_cnt = c->d_fin_cnt;
    a.m.fin_init = c->d_fin_init;
    a.m.fin_rec = c->d_fin_rec;
    a.m.fin_ticket = c->d_fin_ticket;
    a.m.n_fin = c->n_fin;
  }
  int         launches = 0;
  cudaError_t e = mode == G5_MODE_FP64 ? g5::launch_step_fp64(c->dim, c->b, a, sh.ctas_per_sm, s, &launches)
                                       : g5::launch_step_mixed(c->dim, c->b, a, sh.ctas_per_sm, s, &launches);
  c->last_launches = launches;
  return e == cudaSuccess ? G5_OK : G5_ERR_CUDA;
}

// Plan of g5_step_host for the table being uploaded (host arrays of g5_set_mesh).
int
plan_host_pipe(G5Context * c, const G5Mesh * m, const std::vector<int32_t> & defer_slot, const std::vector<int32_t> & defer_list)
{
  G5Context::HostPipe & hp = c->pipe;
  const int             n_owned = m->n_owned, ns = c->ns, nch = c->nch, nfaces = 2 * c->dim;
  const int             center = c->dim == 2 ? 4 : 13;
  // 8 chunks of at least 64 blocks, or in 2D more (up to 16) when the chunks
  // would exceed about 3.5 MB (the copy of chunk 0 is the pipeline's start-up
  // latency, each chunk's step launch has a fixed cost; 3D chunks of that size
  // hold too few blocks whose 26 neighbours have all arrived)
  const double          mbytes = (double)(n_owned + m->n_outside) * c->nv * (c->dim == 2 ? c->b * c->b : c->b * c->b * c->b) * 8.0 / (1 << 20);
  int                   K = n_owned / 64;
  K = K > 8 ? 8 : K;
  const int             Kb = (int)(mbytes / 3.5 + 0.5);
  K = c->dim == 2 && Kb > K && Kb <= n_owned / 64 ? Kb : K;
  K = K < 1 ? 1 : (K > 16 ? 16 : K);
  hp.K = K;
  hp.lo.assign(K + 1, 0);
  for (int k = 0; k <= K; ++k)
    hp.lo[k] = (int)((int64_t)n_owned * k / K);
  std::vector<int> chunk(n_owned);
  for (int k = 0; k < K; ++k)
    for (int n = hp.lo[k]; n < hp.lo[k + 1]; ++n)
      chunk[n] = k;
  // outside blocks travel with chunk 0
  auto arrival = [&](int b) { return b >= n_owned ? 0 : chunk[b]; };
  std::vector<int> ready(n_owned);
  for (int n = 0; n < n_owned; ++n)
  {
    int r = chunk[n];
    for (int s = 0; s < ns; ++s)
    {
      if (s == center)
        continue;
      const int32_t * nb = m->nbr + ((size_t)n * ns + s) * nch;
      // only a finer slot lists more than one block
      const int       nread = m->nbr_rel[(size_t)n * ns + s] > 0 ? nch : 1;
      for (int ch = 0; ch < nread; ++ch)
        if (nb[ch] >= 0)
          r = r > arrival(nb[ch]) ? r : arrival(nb[ch]);
    }
    ready[n] = r;
  }
  // a block with coarse/fine records is final once its finer face neighbours are stepped
  std::vector<int> final_(ready);
  for (int n = 0; n < n_owned; ++n)
    for (int f = 0; f < nfaces; ++f)
    {
      if (defer_slot.empty() || defer_slot[(size_t)n * nfaces + f] < 0)
        continue;
      int d[3] = { 0, 0, 0 };
      d[f >> 1] = (f & 1) ? 1 : -1;
      const int       s = (d[0] + 1) + 3 * (d[1] + 1) + (c->dim == 3 ? 9 * (d[2] + 1) : 0);
      const int32_t * nb = m->nbr + ((size_t)n * ns + s) * nch;
      for (int ch = 0; ch < nch; ++ch)
        if (nb[ch] >= 0 && nb[ch] < n_owned)
          final_[n] = final_[n] > ready[nb[ch]] ? final_[n] : ready[nb[ch]];
    }
  std::vector<int32_t>   work;
  std::vector<int32_t> & recs = hp.recs;
  recs.clear();
  hp.work_off.assign(K + 1, 0);
  hp.rec_off.assign(K + 1, 0);
  for (int k = 0; k < K; ++k)
  {
    hp.work_off[k] = (int)work.size();
    for (int n = 0; n < n_owned; ++n)
      if (ready[n] == k)
        work.push_back(n);
    hp.rec_off[k] = (int)recs.size();
    for (int32_t code : defer_list)
      if (final_[code >> 3] == k)
        recs.push_back(code);
  }
  hp.work_off[K] = (int)work.size();
  hp.rec_off[K] = (int)recs.size();
  hp.out_off.assign(K + 1, 0);
  hp.out_list.clear();
  std::vector<int> out_ready(K, 0);
  for (int n = 0; n < n_owned; ++n)
    out_ready[chunk[n]] = out_ready[chunk[n]] > final_[n] ? out_ready[chunk[n]] : final_[n];
  for (int k = 0; k < K; ++k)
  {
    hp.out_off[k] = (int)hp.out_list.size();
    for (int d = 0; d < K; ++d)
      if (out_ready[d] == k)
        hp.out_list.push_back(d);
  }
  hp.out_off[K] = (int)hp.out_list.size();
  return dev_upload(c, &hp.d_work, work.data(), work.size());
}

} // namespace

extern "C" const char *
g5_version(void)
{
  return "g5gpu 0.1 (sm_103a)";
}

extern "C" int
g5_create(const G5Params * params, G5Context ** out_ctx)
{
  if (!params || !out_ctx)
    return G5_ERR_ARG;
  *out_ctx = nullptr;
  if (params->dim != 2 && params->dim != 3)
    return G5_ERR_ARG;
  if (params->bsize < 4 || (params->bsize & 1))
    return G5_ERR_ARG;
  if (!g5::step_supported(params->dim, params->bsize))
    return G5_ERR_UNSUPPORTED;
  if (params->integrator < 0 || params->integrator > 2)
    return G5_ERR_UNSUPPORTED;
  if (params->source_term != 0 && params->source_term != 1)
    return G5_ERR_UNSUPPORTED;
  if (params->prolongation < G5_PROLONG_SIMPLE_COPY || params->prolongation > G5_PROLONG_CONSERVATIVE_O4)
    return G5_ERR_ARG;
  for (int k = 0; k < 2; ++k)
    if (!(params->gamma[k] > 1.0))
      return G5_ERR_ARG;
  if (!g5::eos_params_valid(params))
    return G5_ERR_ARG;
  G5Context * c = new G5Context;
  c->shape[G5_MODE_FP64].reflux = 0; // the FP64 form has one record pass (the tuner's choice too)
  c->prm = *params;
  c->dim = params->dim;
  c->b = params->bsize;
  c->nv = params->dim == 2 ? 8 : 9;
  c->ns = params->dim == 2 ? 9 : 27;
  c->nch = params->dim == 2 ? 4 : 8;
  cudaGetDevice(&c->device);
  c->phys = g5::make_phys(params);
  if (cudaMalloc((void **)&c->d_status, sizeof(unsigned int)) != cudaSuccess ||
      cudaMemset(c->d_status, 0, sizeof(unsigned int)) != cudaSuccess)
  {
    delete c;
    return G5_ERR_CUDA;
  }
  c->bytes = sizeof(unsigned int);
  *out_ctx = c;
  return G5_OK;
}

extern "C" int
g5_destroy(G5Context * ctx)
{
  if (!ctx)
    return G5_ERR_ARG;
  free_mesh(ctx);
  free_pool(ctx);
  if (ctx->d_status)
    cudaFree(ctx->d_status);
  G5Context::HostPipe & hp = ctx->pipe;
  for (cudaEvent_t e : hp.ev_in)
    cudaEventDestroy(e);
  for (cudaEvent_t e : hp.ev_comp)
    cudaEventDestroy(e);
  for (cudaEvent_t e : hp.ev_step)
    cudaEventDestroy(e);
  for (cudaStream_t q : hp.s_c)
    if (q)
      cudaStreamDestroy(q);
  if (hp.ev_start)
    cudaEventDestroy(hp.ev_start);
  if (hp.ev_out)
    cudaEventDestroy(hp.ev_out);
  if (hp.ev_dt_read)
    cudaEventDestroy(hp.ev_dt_read);
  if (hp.h_dt_stage)
    cudaFreeHost(hp.h_dt_stage);
  if (hp.h_inv_stage)
    cudaFreeHost(hp.h_inv_stage);
  if (hp.s_in)
    cudaStreamDestroy(hp.s_in);
  if (hp.s_out)
    cudaStreamDestroy(hp.s_out);
  delete ctx;
  return G5_OK;
}

extern "C" int
g5_set_mesh(G5Context * c, const G5Mesh * m)
{
  // (a table without blocks, a rank that owns none, may pass NULL arrays)
  if (!c || !m || m->n_owned < 0 || m->n_outside < 0 || (m->n_owned + m->n_outside > 0 && (!m->level || !m->coord)))
    return G5_ERR_ARG;
  if (m->n_owned > 0 && (!m->nbr || !m->nbr_rel))
    return G5_ERR_ARG;
  if (m->n_outside > 0 && (!m->out_src || !m->out_normal || !m->out_border))
    return G5_ERR_ARG;
  const int n_owned = m->n_owned, n_total = m->n_owned + m->n_outside;
  const int n_inst = m->n_inst > 0 ? m->n_inst : 1;
  const int ns = c->ns, nch = c->nch, dim = c->dim;
  // ---- validate the table (the reference asserts these in StencilHelper / hashmap lookups)
  if (g5::validate_table(dim, m) != G5_OK)
    return G5_ERR_MESH;

  // ---- coarse/fine face records
  const int            nfaces = 2 * dim;
  std::vector<int32_t> reflux_slot((size_t)n_owned * nfaces, -1), defer_slot((size_t)n_owned * nfaces, -1), defer_list;
  int                  n_reflux = 0, n_defer = 0;
  for (int n = 0; n < n_owned; ++n)
    for (int f = 0; f < nfaces; ++f)
    {
      int d[3] = { 0, 0, 0 };
      d[f >> 1] = (f & 1) ? 1 : -1;
      const int s = (d[0] + 1) + 3 * (d[1] + 1) + (dim == 3 ? 9 * (d[2] + 1) : 0);
      const int rel = m->nbr_rel[(size_t)n * ns + s];
      const int * nb = m->nbr + ((size_t)n * ns + s) * nch;
      if (rel < 0 && nb[0] < n_owned)
        reflux_slot[(size_t)n * nfaces + f] = n_reflux++;
      if (rel > 0)
      {
        bool owned = true;
        for (int ch = 0; ch < nch; ++ch)
          if (nb[ch] >= n_owned)
            owned = false;
        if (owned)
        {
          defer_slot[(size_t)n * nfaces + f] = n_defer++;
          defer_list.push_back(n * 8 + f);
        }
      }
    }

  free_mesh(c);
  // work of the previous mesh may still run on another stream: the buffers
  // are reused in place below
  if (cudaDeviceSynchronize() != cudaSuccess)
    return G5_ERR_CUDA;
  const size_t face_cells = dim == 2 ? (size_t)c->b : (size_t)c->b * c->b;
  const size_t nf = dim == 2 ? 8 : 9;
  int          rc = 0;
  rc |= dev_upload(c, &c->d_level, m->level, (size_t)n_total);
  rc |= dev_upload(c, &c->d_coord, m->coord, (size_t)n_total * 3);
  rc |= dev_upload(c, &c->d_nbr, m->nbr, (size_t)n_owned * ns * nch);
  rc |= dev_upload(c, &c->d_nbr_rel, m->nbr_rel, (size_t)n_owned * ns);
  if (m->inst)
    rc |= dev_upload(c, &c->d_inst, m->inst, (size_t)n_total);
  if (m->n_outside > 0)
  {
    rc |= dev_upload(c, &c->d_out_src, m->out_src, (size_t)m->n_outside);
    rc |= dev_upload(c, &c->d_out_normal, m->out_normal, (size_t)m->n_outside * 3);
    rc |= dev_upload(c, &c->d_out_border, m->out_border, (size_t)m->n_outside * 6);
  }
  if (n_defer > 0)
  {
    rc |= dev_upload(c, &c->d_reflux_slot, reflux_slot.data(), reflux_slot.size());
    rc |= dev_upload(c, &c->d_defer_slot, defer_slot.data(), defer_slot.size());
    rc |= dev_alloc(c, &c->d_reflux_buf, (size_t)n_reflux * face_cells * nf);
    rc |= dev_alloc(c, &c->d_defer_buf, (size_t)n_defer * face_cells * 2 * dim * nf);
  }
  rc |= dev_alloc(c, &c->d_dt, (size_t)n_inst);
  rc |= dev_alloc(c, &c->d_invdt, (size_t)n_inst);
  rc |= dev_alloc(c, &c->d_ticket, 1);
  if (!rc && cudaMemset(c->d_ticket, 0, sizeof(unsigned int)) != cudaSuccess)
    rc = G5_ERR_CUDA;
  if (c->prm.integrator == 2)
    rc |= dev_alloc(c, &c->d_urk, (size_t)n_total * c->nv * (dim == 2 ? c->b * c->b : c->b * c->b * c->b));
  if (c->prm.prolongation != G5_PROLONG_SIMPLE_COPY)
  {
    // one slot of prolonged ghost states per owned block with a coarser neighbour
    std::vector<int32_t> pg_slot(n_owned, -1);
    int                  n_pg = 0;
    for (int n = 0; n < n_owned; ++n)
      for (int s = 0; s < ns; ++s)
        if (m->nbr_rel[(size_t)n * ns + s] < 0)
        {
          pg_slot[n] = n_pg++;
          break;
        }
    const size_t ng = dim == 2 ? (size_t)(c->b + 4) * (c->b + 4) : (size_t)(c->b + 4) * (c->b + 4) * (c->b + 4);
    rc |= dev_upload(c, &c->d_pg_slot, pg_slot.data(), pg_slot.size());
    if (n_pg > 0)
      rc |= dev_alloc(c, &c->d_pg, (size_t)n_pg * c->nv * ng);
  }
  if (rc)
  {
    free_mesh(c);
    return G5_ERR_CUDA;
  }
  c->n_owned = n_owned;
  c->n_outside = m->n_outside;
  c->n_total = n_total;
  c->n_inst = n_inst;
  c->n_defer = n_defer;
  c->n_reflux = n_reflux;
  if (plan_host_pipe(c, m, defer_slot, defer_list))
  {
    free_mesh(c);
    return G5_ERR_CUDA;
  }
  // owned blocks grouped by instance (counting sort, block order kept)
  c->inst_off.assign(n_inst + 1, 0);
  for (int n = 0; n < n_owned; ++n)
    ++c->inst_off[(m->inst ? m->inst[n] : 0) + 1];
  for (int i = 0; i < n_inst; ++i)
    c->inst_off[i + 1] += c->inst_off[i];
  c->inst_blocks.assign(n_owned, 0);
  {
    std::vector<int32_t> pos(c->inst_off.begin(), c->inst_off.end() - 1);
    for (int n = 0; n < n_owned; ++n)
      c->inst_blocks[pos[m->inst ? m->inst[n] : 0]++] = n;
  }
  if (dev_alloc(c, &c->d_batch_work, (size_t)n_owned) || dev_alloc(c, &c->d_inst_active, (size_t)n_inst))
  {
    free_mesh(c);
    return G5_ERR_CUDA;
  }
  // outside blocks per owned source block, with the face whose rule the
  // boundary fill applies last (FillOutside.cpp:71-170)
  {
    std::vector<int32_t> first((size_t)n_owned + 1, 0), list;
    std::vector<int32_t> entry((size_t)m->n_outside, -1);
    for (int o = 0; o < m->n_outside; ++o)
    {
      int last = -1;
      for (int f = 0; f < 2 * dim; ++f)
        if (m->out_border[o * 6 + f] && m->out_normal[o * 3 + (f >> 1)] != 0 && (c->prm.bc[f] == 2 || c->prm.bc[f] == 3))
          last = f;
      if (last >= 0)
      {
        entry[o] = (n_owned + o) * 8 + last;
        ++first[m->out_src[o] + 1];
      }
    }
    for (int n = 0; n < n_owned; ++n)
      first[n + 1] += first[n];
    list.assign((size_t)first[n_owned], 0);
    std::vector<int32_t> pos(first.begin(), first.end() - 1);
    for (int o = 0; o < m->n_outside; ++o)
      if (entry[o] >= 0)
        list[pos[m->out_src[o]]++] = entry[o];
    int trc = dev_upload(c, &c->d_twin_first, first.data(), first.size());
    if (!list.empty())
      trc |= dev_upload(c, &c->d_twin_list, list.data(), list.size());
    if (trc)
    {
      free_mesh(c);
      return G5_ERR_CUDA;
    }
    c->fused_fill = dim == 2 && m->n_outside > 0;
  }
  {
    // walk order of the full-mesh step: blocks with more neighbour slots at
    // another level first (their gathers restrict or prolong, they publish or
    // defer coarse/fine records: they cost more), so that the last round of
    // the persistent grid holds cheap same-level blocks
    std::vector<int32_t> order(n_owned), score(n_owned, 0);
    for (int n = 0; n < n_owned; ++n)
    {
      order[n] = n;
      for (int sl = 0; sl < ns; ++sl)
        score[n] += m->nbr_rel[(size_t)n * ns + sl] != 0;
    }
    std::stable_sort(order.begin(), order.end(), [&](int32_t x, int32_t y) { return score[x] > score[y]; });
    if (n_owned > 0 && dev_upload(c, &c->d_walk, order.data(), order.size()))
    {
      free_mesh(c);
      return G5_ERR_CUDA;
    }
  }
  if (n_defer > 0)
  {
    // records in the launch order of g5_step_host, and their reflux-pass rows
    const std::vector<int32_t> & recs = c->pipe.recs;
    const int stride = dim == 2 ? g5::DeferInfo<2>::STRIDE : g5::DeferInfo<3>::STRIDE;
    rc = dev_upload(c, &c->d_defer_list, recs.data(), recs.size());
    rc |= dev_alloc(c, &c->d_defer_info, recs.size() * (size_t)stride);
    if (!rc && (g5::launch_defer_info(dim, dev_mesh(c), c->d_defer_list, (int)recs.size(), c->d_defer_info, nullptr) != cudaSuccess ||
                cudaStreamSynchronize(nullptr) != cudaSuccess))
      rc = 1;
    // reflux in the step's tail (2D): per deferred block (a coarse block with
    // records) a counter of the arrivals that make its records final: the
    // block itself, each fine block face publishing into one of its records
    // (the pairs the reflux pass reads, found as in the DeferInfo rows), and
    // one claim by a CTA out of blocks.  Whoever brings it to zero finishes
    // the block's deferred cells, so nothing waits.
    if (!rc && dim == 2)
    {
      const int             ntg = nfaces + 1;
      std::vector<int32_t>  fin_of(n_owned, -1), tgt((size_t)n_owned * ntg, -1), frec;
      std::vector<uint32_t> init;
      auto                  add_tgt = [&](int blk, int j) {
        int32_t * row = &tgt[(size_t)blk * ntg];
        int       k = 0;
        while (k < ntg && row[k] >= 0)
          ++k;
        if (k == ntg)
          return false;
        row[k] = j;
        ++init[j];
        return true;
      };
      bool ok = true;
      for (size_t r = 0; r < recs.size() && ok; ++r)
      {
        const int nb = recs[r] >> 3, f = recs[r] & 7;
        if (fin_of[nb] < 0)
        {
          fin_of[nb] = (int)init.size();
          init.push_back(1); // the tail claim
          frec.insert(frec.end(), (size_t)nfaces, -1);
          ok = add_tgt(nb, fin_of[nb]);
        }
        const int j = fin_of[nb];
        int       k = 0;
        while (frec[(size_t)j * nfaces + k] >= 0)
          ++k;
        frec[(size_t)j * nfaces + k] = (int32_t)r;
        const int dir = f >> 1, side = f & 1;
        int       d[3] = { 0, 0, 0 };
        d[dir] = side ? 1 : -1;
        const int s = (d[0] + 1) + 3 * (d[1] + 1);
        for (int cc = 0; cc < 2 && ok; ++cc)
        {
          int ch[2] = { 0, 0 };
          ch[dir] = side ? 0 : 1;
          ch[dir == 0 ? 1 : 0] = cc & 1;
          const int F = m->nbr[((size_t)nb * ns + s) * nch + ch[0] + 2 * ch[1]];
          if (F >= 0 && F < n_owned && reflux_slot[(size_t)F * nfaces + (f ^ 1)] >= 0)
            ok = add_tgt(F, j);
        }
      }
      // (a table whose blocks count off more counters than a row holds keeps
      // the separate pass)
      c->n_fin = ok ? (int)init.size() : 0;
      if (c->n_fin > 0)
      {
        rc |= dev_upload(c, &c->d_fin_tgt, tgt.data(), tgt.size());
        rc |= dev_upload(c, &c->d_fin_rec, frec.data(), frec.size());
        rc |= dev_upload(c, &c->d_fin_init, init.data(), init.size());
        rc |= dev_upload(c, &c->d_fin_cnt, init.data(), init.size());
        rc |= dev_alloc(c, &c->d_fin_ticket, 1);
        if (!rc && cudaMemset(c->d_fin_ticket, 0, sizeof(unsigned int)) != cudaSuccess)
          rc = 1;
      }
    }
    if (rc)
    {
      free_mesh(c);
      return G5_ERR_CUDA;
    }
  }
  c->has_mesh = true;
  return G5_OK;
}

extern "C" int64_t
g5_mem_bytes(const G5Context * ctx)
{
  return ctx ? ctx->bytes : (int64_t)G5_ERR_ARG;
}

extern "C" int
g5_step_dev(G5Context * ctx, const double * d_U, double * d_U2, const double * d_dt, int mode, double * d_inv_dt_out, void * stream)
{
  return do_step(ctx, d_U, d_U2, d_dt, mode, d_inv_dt_out, (cudaStream_t)stream);
}

extern "C" int
g5_step(G5Context * ctx, const double * d_U, double * d_U2, const double * dt_host, int mode, double * d_inv_dt_out, void * stream)
{
  if (!ctx || !ctx->has_mesh || !dt_host)
    return G5_ERR_ARG;
  for (int i = 0; i < ctx->n_inst; ++i)
    if (!(dt_host[i] > 0.0))
      return G5_ERR_ARG;
  if (cudaMemcpyAsync(ctx->d_dt, dt_host, sizeof(double) * ctx->n_inst, cudaMemcpyHostToDevice, (cudaStream_t)stream) != cudaSuccess)
    return G5_ERR_CUDA;
  return do_step(ctx, d_U, d_U2, ctx->d_dt, mode, d_inv_dt_out, (cudaStream_t)stream);
}

namespace
{
void CUDART_CB
copy_inv_to_caller(void * arg)
{
  const G5Context::HostPipe::InvCopy * ic = static_cast<const G5Context::HostPipe::InvCopy *>(arg);
  std::memcpy(ic->dst, ic->src, ic->bytes);
}

// Enqueue one pipelined host-buffer step on s (captured into a graph or run
// directly).  U2 goes straight to host memory when d_U2_host (the device view
// of the caller's pinned U2) is given, otherwise through the device staging
// array and chunked copies on s_out.
bool
enqueue_host_step(G5Context * c, const double * h_U, double * h_U2, double * d_U2_host, int mode, bool want_inv,
                  const G5Context::HostPipe::InvCopy * inv, bool capturing, cudaStream_t s, int * launches)
{
  G5Context::HostPipe & hp = c->pipe;
  const int             K = hp.K;
  const size_t          blk = (size_t)c->nv * (c->dim == 2 ? c->b * c->b : c->b * c->b * c->b);
  const size_t          bb = blk * sizeof(double);
  const bool            staged_out = d_U2_host == nullptr;
  bool ok = cudaMemcpyAsync(c->d_dt, hp.h_dt_stage, sizeof(double) * c->n_inst, cudaMemcpyHostToDevice, s) == cudaSuccess;
  ok = ok && cudaEventRecordWithFlags(hp.ev_dt_read, s, capturing ? cudaEventRecordExternal : cudaEventRecordDefault) == cudaSuccess;
  if (want_inv)
    ok = ok && cudaMemsetAsync(c->d_invdt, 0, sizeof(double) * c->n_inst, s) == cudaSuccess;
  // the copy streams start after the work already queued on s
  ok = ok && cudaEventRecord(hp.ev_start, s) == cudaSuccess && cudaStreamWaitEvent(hp.s_in, hp.ev_start, 0) == cudaSuccess;
  if (staged_out)
    ok = ok && cudaStreamWaitEvent(hp.s_out, hp.ev_start, 0) == cudaSuccess;
  for (int k = 0; ok && k < K; ++k)
  {
    if (k == 0 && c->n_outside > 0)
      ok = cudaMemcpyAsync(hp.d_U + (size_t)c->n_owned * blk, h_U + (size_t)c->n_owned * blk, (size_t)c->n_outside * bb,
                           cudaMemcpyHostToDevice, hp.s_in) == cudaSuccess;
    const size_t n0 = (size_t)hp.lo[k], n1 = (size_t)hp.lo[k + 1];
    if (ok && n1 > n0)
      ok = cudaMemcpyAsync(hp.d_U + n0 * blk, h_U + n0 * blk, (n1 - n0) * bb, cudaMemcpyHostToDevice, hp.s_in) == cudaSuccess;
    ok = ok && cudaEventRecord(hp.ev_in[k], hp.s_in) == cudaSuccess;
  }
  // chunk launches on kComputeStreams streams, so that the (latency-bound)
  // launches of consecutive chunks run side by side; the coarse/fine records
  // of chunk k wait for the step launches of chunks 0..k
  const int P = G5Context::HostPipe::kComputeStreams;
  for (int q = 0; ok && q < P && q < K; ++q) // (a captured stream without work could not be joined)
    ok = cudaStreamWaitEvent(hp.s_c[q], hp.ev_start, 0) == cudaSuccess;
  for (int k = 0; ok && k < K; ++k)
  {
    cudaStream_t q = hp.s_c[k % P];
    ok = cudaStreamWaitEvent(q, hp.ev_in[k], 0) == cudaSuccess;
    g5::StepArgs a;
    a.U = hp.d_U;
    a.U2 = staged_out ? hp.d_U2 : d_U2_host;
    a.dt = c->d_dt;
    a.reflux_buf = c->d_reflux_buf;
    a.defer_buf = c->d_defer_buf;
    a.invdt = want_inv ? c->d_invdt : nullptr;
    a.status = c->d_status;
    a.work = hp.d_work + hp.work_off[k];
    a.n_work = hp.work_off[k + 1] - hp.work_off[k];
    a.m = dev_mesh(c);
    a.m.defer_list = nullptr;
    a.m.n_defer = 0;
    a.p = c->phys;
    a.reflux_layout = c->shape[mode].reflux;
    auto launch = [&](const g5::StepArgs & args) {
      const cudaError_t e = mode == G5_MODE_FP64 ? g5::launch_step_fp64(c->dim, c->b, args, c->shape[0].ctas_per_sm, q, launches)
                                                 : g5::launch_step_mixed(c->dim, c->b, args, c->shape[1].ctas_per_sm, q, launches);
      return e == cudaSuccess;
    };
    if (ok && a.n_work > 0)
      ok = launch(a);
    ok = ok && cudaEventRecord(hp.ev_step[k], q) == cudaSuccess;
    const int n_rec = hp.rec_off[k + 1] - hp.rec_off[k];
    if (ok && n_rec > 0)
    {
      for (int j = 0; ok && j < k; ++j)
        if (j % P != k % P)
          ok = cudaStreamWaitEvent(q, hp.ev_step[j], 0) == cudaSuccess;
      a.work = hp.d_work; // non-null with n_work == 0: the launcher runs the record pass only
      a.n_work = 0;
      a.m.defer_info = c->d_defer_info + (size_t)hp.rec_off[k] * (c->dim == 2 ? g5::DeferInfo<2>::STRIDE : g5::DeferInfo<3>::STRIDE);
      a.m.n_defer = n_rec;
      ok = ok && launch(a);
    }
    ok = ok && cudaEventRecord(hp.ev_comp[k], q) == cudaSuccess;
    if (!staged_out)
      continue;
    // s_out walks k in order, so it has waited for every launch 0..k
    ok = ok && cudaStreamWaitEvent(hp.s_out, hp.ev_comp[k], 0) == cudaSuccess;
    for (int t = hp.out_off[k]; ok && t < hp.out_off[k + 1]; ++t)
    {
      const int    d = hp.out_list[t];
      const size_t n0 = (size_t)hp.lo[d], n1 = (size_t)hp.lo[d + 1];
      if (n1 > n0)
        ok = cudaMemcpyAsync(h_U2 + n0 * blk, hp.d_U2 + n0 * blk, (n1 - n0) * bb, cudaMemcpyDeviceToHost, hp.s_out) == cudaSuccess;
    }
  }
  // join everything back into s
  for (int k = 0; ok && k < K; ++k)
    ok = cudaStreamWaitEvent(s, hp.ev_comp[k], 0) == cudaSuccess;
  if (staged_out)
    ok = ok && cudaEventRecord(hp.ev_out, hp.s_out) == cudaSuccess && cudaStreamWaitEvent(s, hp.ev_out, 0) == cudaSuccess;
  if (ok && inv)
    ok = cudaMemcpyAsync(hp.h_inv_stage, c->d_invdt, sizeof(double) * c->n_inst, cudaMemcpyDeviceToHost, s) == cudaSuccess &&
         cudaLaunchHostFunc(s, copy_inv_to_caller, (void *)inv) == cudaSuccess;
  return ok;
}
} // namespace

extern "C" int
g5_step_batched(G5Context * c, const double * d_U, double * d_U2, const double * d_dt, int mode, const int32_t * instances, int n_list,
                double * d_inv_dt_out, void * stream)
{
  if (!c || !c->has_mesh || !d_U || !d_U2 || !d_dt || n_list < 0 || (n_list > 0 && !instances))
    return G5_ERR_ARG;
  if (mode != G5_MODE_FP64 && mode != G5_MODE_MIXED)
    return G5_ERR_ARG;
  if (!g5::step_supported(c->dim, c->b))
    return G5_ERR_UNSUPPORTED;
  std::vector<uint8_t> active((size_t)c->n_inst, 0);
  for (int k = 0; k < n_list; ++k)
  {
    if (instances[k] < 0 || instances[k] >= c->n_inst)
      return G5_ERR_ARG;
    active[instances[k]] = 1;
  }
  std::vector<int32_t> work;
  for (int i = 0; i < c->n_inst; ++i)
    if (active[i])
      work.insert(work.end(), c->inst_blocks.begin() + c->inst_off[i], c->inst_blocks.begin() + c->inst_off[i + 1]);
  cudaStream_t s = (cudaStream_t)stream;
  c->last_launches = 0;
  if (work.empty())
    return G5_OK;
  // pageable sources: the copies are staged before the calls return
  if (cudaMemcpyAsync(c->d_batch_work, work.data(), work.size() * sizeof(int32_t), cudaMemcpyHostToDevice, s) != cudaSuccess ||
      cudaMemcpyAsync(c->d_inst_active, active.data(), active.size(), cudaMemcpyHostToDevice, s) != cudaSuccess)
    return G5_ERR_CUDA;
  g5::StepArgs a;
  a.U = d_U;
  a.U2 = d_U2;
  a.dt = d_dt;
  a.reflux_buf = c->d_reflux_buf;
  a.defer_buf = c->d_defer_buf;
  a.invdt = d_inv_dt_out;
  a.status = c->d_status;
  a.work = c->d_batch_work;
  a.n_work = (int)work.size();
  a.inst_active = c->d_inst_active;
  a.ticket = c->shape[mode].claim ? c->d_ticket : nullptr;
  a.reflux_layout = c->shape[mode].reflux;
  a.m = dev_mesh(c);
  a.p = c->phys;
  int         launches = 0;
  cudaError_t e = mode == G5_MODE_FP64 ? g5::launch_step_fp64(c->dim, c->b, a, c->shape[0].ctas_per_sm, s, &launches)
                                       : g5::launch_step_mixed(c->dim, c->b, a, c->shape[1].ctas_per_sm, s, &launches);
  c->last_launches = launches;
  return e == cudaSuccess ? G5_OK : G5_ERR_CUDA;
}

extern "C" int
g5_step_host(G5Context * c, const double * h_U, double * h_U2, const double * dt_host, int mode, double * h_inv_dt_out, void * stream)
{
  if (!c || !c->has_mesh || !h_U || !h_U2 || !dt_host)
    return G5_ERR_ARG;
  if (mode != G5_MODE_FP64 && mode != G5_MODE_MIXED)
    return G5_ERR_ARG;
  for (int i = 0; i < c->n_inst; ++i)
    if (!(dt_host[i] > 0.0))
      return G5_ERR_ARG;
  G5Context::HostPipe & hp = c->pipe;
  const int             K = hp.K;
  const size_t          blk = (size_t)c->nv * (c->dim == 2 ? c->b * c->b : c->b * c->b * c->b);
  if (!hp.s_in)
  {
    if (cudaStreamCreateWithFlags(&hp.s_in, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&hp.s_out, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&hp.ev_start, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&hp.ev_out, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&hp.ev_dt_read, cudaEventDisableTiming) != cudaSuccess)
      return G5_ERR_CUDA;
    for (cudaStream_t & q : hp.s_c)
      if (cudaStreamCreateWithFlags(&q, cudaStreamNonBlocking) != cudaSuccess)
        return G5_ERR_CUDA;
  }
  while ((int)hp.ev_in.size() < K)
  {
    cudaEvent_t a = nullptr, b = nullptr, e = nullptr;
    if (cudaEventCreateWithFlags(&a, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&b, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess)
      return G5_ERR_CUDA;
    hp.ev_in.push_back(a);
    hp.ev_comp.push_back(b);
    hp.ev_step.push_back(e);
  }
  if (hp.dt_pending)
  {
    // the previous call's step must have read the staged dt before it is overwritten
    if (cudaEventSynchronize(hp.ev_dt_read) != cudaSuccess)
      return G5_ERR_CUDA;
    hp.dt_pending = false;
  }
  if (hp.n_stage < c->n_inst)
  {
    if (hp.h_dt_stage)
      cudaFreeHost(hp.h_dt_stage);
    if (hp.h_inv_stage)
      cudaFreeHost(hp.h_inv_stage);
    hp.h_dt_stage = hp.h_inv_stage = nullptr;
    hp.n_stage = 0;
    if (cudaMallocHost((void **)&hp.h_dt_stage, sizeof(double) * c->n_inst) != cudaSuccess ||
        cudaMallocHost((void **)&hp.h_inv_stage, sizeof(double) * c->n_inst) != cudaSuccess)
      return G5_ERR_CUDA;
    hp.n_stage = c->n_inst;
  }
  if (!hp.d_U)
  {
    if (dev_alloc(c, &hp.d_U, (size_t)c->n_total * blk) || dev_alloc(c, &hp.d_U2, (size_t)(c->n_owned > 0 ? c->n_owned : 1) * blk))
      return G5_ERR_CUDA;
  }
  std::memcpy(hp.h_dt_stage, dt_host, sizeof(double) * c->n_inst);
  // pinned caller buffers: the step writes U2 straight into host memory and the
  // whole step is replayed from a graph; pageable buffers go through staging
  double * d_U2_host = nullptr;
  if (cudaHostGetDevicePointer((void **)&d_U2_host, h_U2, 0) != cudaSuccess)
  {
    cudaGetLastError();
    d_U2_host = nullptr;
  }
  cudaPointerAttributes attr;
  const bool            pinned_in = cudaPointerGetAttributes(&attr, h_U) == cudaSuccess && attr.type == cudaMemoryTypeHost;
  cudaGetLastError();
  cudaStream_t s = (cudaStream_t)stream;
  int          launches = 0;
  if (!pinned_in || !d_U2_host)
  {
    // pageable caller buffers: copies through the staging arrays, and the CFL
    // rate read back synchronously
    bool ok = enqueue_host_step(c, h_U, h_U2, nullptr, mode, h_inv_dt_out != nullptr, nullptr, false, s, &launches);
    hp.dt_pending = true;
    if (ok && h_inv_dt_out)
      ok = cudaMemcpyAsync(hp.h_inv_stage, c->d_invdt, sizeof(double) * c->n_inst, cudaMemcpyDeviceToHost, s) == cudaSuccess &&
           cudaStreamSynchronize(s) == cudaSuccess;
    if (ok && h_inv_dt_out)
      std::memcpy(h_inv_dt_out, hp.h_inv_stage, sizeof(double) * c->n_inst);
    c->last_launches = launches;
    return ok ? G5_OK : G5_ERR_CUDA;
  }
  G5Context::HostPipe::Graph * slot = nullptr;
  for (auto & g : hp.graphs)
    if (g.exec && g.hU == h_U && g.hU2 == h_U2 && g.mode == mode && g.inv == h_inv_dt_out)
      slot = &g;
  if (!slot)
  {
    slot = &hp.graphs[hp.next_graph];
    hp.next_graph = (hp.next_graph + 1) % G5Context::HostPipe::kGraphs;
    if (slot->exec)
      cudaGraphExecDestroy(slot->exec);
    *slot = G5Context::HostPipe::Graph();
    slot->inv_copy = { h_inv_dt_out, hp.h_inv_stage, sizeof(double) * c->n_inst };
    cudaStream_t cap;
    if (cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking) != cudaSuccess)
      return G5_ERR_CUDA;
    cudaGraph_t g = nullptr;
    if (cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
    {
      cudaStreamDestroy(cap);
      return G5_ERR_CUDA;
    }
    int         n = 0;
    const bool  ok = enqueue_host_step(c, h_U, h_U2, d_U2_host, mode, h_inv_dt_out != nullptr, h_inv_dt_out ? &slot->inv_copy : nullptr,
                                       true, cap, &n);
    cudaError_t e = cudaStreamEndCapture(cap, &g);
    cudaStreamDestroy(cap);
    if (!ok || e != cudaSuccess)
    {
      if (g)
        cudaGraphDestroy(g);
      return G5_ERR_CUDA;
    }
    e = cudaGraphInstantiate(&slot->exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess)
    {
      slot->exec = nullptr;
      return G5_ERR_CUDA;
    }
    slot->hU = h_U;
    slot->hU2 = h_U2;
    slot->inv = h_inv_dt_out;
    slot->mode = mode;
    slot->launches = n;
  }
  if (cudaGraphLaunch(slot->exec, s) != cudaSuccess)
    return G5_ERR_CUDA;
  hp.dt_pending = true;
  c->last_launches = slot->launches;
  return G5_OK;
}

extern "C" int
g5_derived_quantity(G5Context * c, const double * d_U, int quantity, int64_t oct_begin, int64_t num_octs, double * d_out, void * stream)
{
  if (!c || !d_U || !d_out || quantity < 0 || quantity > 7)
    return G5_ERR_ARG;
  // ComputeDerivedQuantities::check_args_validity (utils/ComputeDerivedQuantities.h:78-92)
  const int64_t nq = c->has_mesh ? c->n_total : 0;
  if (oct_begin < 0 || oct_begin >= nq || oct_begin + num_octs < 0 || oct_begin + num_octs > nq)
    return G5_ERR_ARG;
  return g5::launch_derived(c->dim, c->b, d_U, d_out, quantity, oct_begin, num_octs, c->phys, (cudaStream_t)stream) == cudaSuccess
           ? G5_OK
           : G5_ERR_CUDA;
}

extern "C" int
g5_pack_fields(G5Context * c, const double * d_U, const int32_t * fields, int nfields, int64_t oct_begin, int64_t num_octs, double * d_out,
               void * stream)
{
  if (!c || !c->has_mesh || !d_U || !d_out || !fields || nfields < 1 || nfields > G5_MAX_PACK_FIELDS)
    return G5_ERR_ARG;
  static_assert(G5_FIELD_DERIVED == g5::FIELD_DERIVED && G5_MAX_PACK_FIELDS == g5::MAX_PACK_FIELDS, "field codes");
  int codes[G5_MAX_PACK_FIELDS];
  for (int k = 0; k < nfields; ++k)
  {
    const int f = fields[k];
    if (!((f >= 0 && f < c->nv) || (f >= G5_FIELD_DERIVED && f <= G5_FIELD_DERIVED + G5_DQ_VZ)))
      return G5_ERR_ARG;
    codes[k] = f;
  }
  const int64_t nq = c->n_total;
  if (oct_begin < 0 || num_octs < 0 || oct_begin + num_octs > nq)
    return G5_ERR_ARG;
  return g5::launch_pack_fields(c->dim, c->b, d_U, d_out, codes, nfields, oct_begin, num_octs, c->phys, (cudaStream_t)stream) == cudaSuccess
           ? G5_OK
           : G5_ERR_CUDA;
}

extern "C" int
g5_compute_inv_dt(G5Context * ctx, const double * d_U, double * d_inv_dt, void * stream)
{
  if (!ctx || !ctx->has_mesh || !d_U || !d_inv_dt)
    return G5_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  if (cudaMemsetAsync(d_inv_dt, 0, sizeof(double) * ctx->n_inst, s) != cudaSuccess)
    return G5_ERR_CUDA;
  return g5::launch_inv_dt(ctx->dim, ctx->b, d_U, dev_mesh(ctx), ctx->phys, d_inv_dt, s) == cudaSuccess ? G5_OK : G5_ERR_CUDA;
}

extern "C" int
g5_fill_outside(G5Context * ctx, double * d_U, void * stream)
{
  if (!ctx || !ctx->has_mesh || !d_U)
    return G5_ERR_ARG;
  return g5::launch_fill_outside(ctx->dim, ctx->b, d_U, dev_mesh(ctx), ctx->phys, (cudaStream_t)stream) == cudaSuccess ? G5_OK
                                                                                                                    : G5_ERR_CUDA;
}

extern "C" int
g5_refine_flags(G5Context * ctx,
                const double * d_U,
                int            indicator,
                double         eps_refine,
                double         eps_coarsen,
                double         eps_lohner,
                int            level_min,
                int            level_max,
                int8_t *       d_flags,
                void *         stream)
{
  if (!ctx || !ctx->has_mesh || !d_U || !d_flags || indicator < 0 || indicator > 2)
    return G5_ERR_ARG;
  return g5::launch_refine_flags(ctx->dim, ctx->b, d_U, dev_mesh(ctx), indicator, eps_refine, eps_coarsen, eps_lohner, level_min,
                                 level_max, d_flags, (cudaStream_t)stream) == cudaSuccess
           ? G5_OK
           : G5_ERR_CUDA;
}

extern "C" int
g5_remap(G5Context * ctx, const G5Remap * r, const double * d_Uold, double * d_Unew, void * stream)
{
  if (!ctx || !r || r->n_new < 0 || r->n_old < 0 || (r->n_new > 0 && (!r->kind || !r->src || !d_Uold || !d_Unew)))
    return G5_ERR_ARG;
  if (r->n_new == 0)
    return G5_OK;
  const int nch = ctx->nch;
  // every index the kernel reads is checked here
  for (int j = 0; j < r->n_new; ++j)
  {
    const int32_t * s = r->src + (size_t)j * nch;
    const int       k = r->kind[j];
    if (k < 0 || k > 2)
      return G5_ERR_MESH;
    const int nread = k == 2 ? nch : 1;
    for (int t = 0; t < nread; ++t)
      if (s[t] < 0 || s[t] >= r->n_old)
        return G5_ERR_MESH;
    if (k == 1 && (s[1] < 0 || s[1] >= nch))
      return G5_ERR_MESH;
  }
  // refined blocks under a prolongation other than SIMPLE_COPY: prolonged over
  // the old mesh, which the context must still hold (g5_remap before
  // g5_set_mesh of the adapted mesh); one row per refined old block
  std::vector<int32_t> refine_rows;
  if (ctx->prm.prolongation != G5_PROLONG_SIMPLE_COPY)
  {
    std::vector<int32_t> row_of;
    for (int j = 0; j < r->n_new; ++j)
    {
      if (r->kind[j] != 1)
        continue;
      if (!ctx->has_mesh || r->n_old != ctx->n_owned)
        return G5_ERR_ARG;
      if (row_of.empty())
        row_of.assign(r->n_old, -1);
      const int32_t * s = r->src + (size_t)j * nch;
      if (row_of[s[0]] < 0)
      {
        row_of[s[0]] = (int)(refine_rows.size() / (nch + 1));
        refine_rows.push_back(s[0]);
        refine_rows.insert(refine_rows.end(), nch, -1);
      }
      int32_t & slot = refine_rows[(size_t)row_of[s[0]] * (nch + 1) + 1 + s[1]];
      if (slot >= 0)
        return G5_ERR_MESH;
      slot = j;
    }
    for (int32_t v : refine_rows)
      if (v < 0)
        return G5_ERR_MESH; // a refined block without all its children
  }
  cudaStream_t st = (cudaStream_t)stream;
  int8_t *     d_kind = nullptr;
  int32_t *    d_src = nullptr;
  const size_t nk = (size_t)r->n_new, ns = (size_t)r->n_new * nch * sizeof(int32_t);
  if (cudaMallocAsync((void **)&d_kind, nk, st) != cudaSuccess)
    return G5_ERR_CUDA;
  if (cudaMallocAsync((void **)&d_src, ns, st) != cudaSuccess)
  {
    cudaFreeAsync(d_kind, st);
    return G5_ERR_CUDA;
  }
  int rc = G5_OK;
  if (cudaMemcpyAsync(d_kind, r->kind, nk, cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemcpyAsync(d_src, r->src, ns, cudaMemcpyHostToDevice, st) != cudaSuccess ||
      g5::launch_remap(ctx->dim, ctx->b, d_Uold, d_Unew, d_kind, d_src, r->n_new, st) != cudaSuccess)
    rc = G5_ERR_CUDA;
  cudaFreeAsync(d_kind, st);
  cudaFreeAsync(d_src, st);
  ctx->last_launches = 1;
  if (rc == G5_OK && !refine_rows.empty())
  {
    int32_t *    d_rows = nullptr;
    const size_t nb = refine_rows.size() * sizeof(int32_t);
    if (cudaMallocAsync((void **)&d_rows, nb, st) != cudaSuccess)
      return G5_ERR_CUDA;
    if (cudaMemcpyAsync(d_rows, refine_rows.data(), nb, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        g5::launch_remap_prolong(ctx->dim, ctx->b, ctx->prm.prolongation, d_Uold, d_Unew, dev_mesh(ctx), d_rows,
                                 (int)(refine_rows.size() / (nch + 1)), ctx->d_status, st) != cudaSuccess)
      rc = G5_ERR_CUDA;
    cudaFreeAsync(d_rows, st);
    ctx->last_launches = 2;
  }
  return rc;
}

namespace
{
// one step of the device-driven solver loop: dt <- cfl / inv_dt(U); U2 <- step(U); fill outside of U2
int
loop_step(G5Context * c, const double * U, double * U2, int mode, double * dt_out, cudaStream_t s, int * launches)
{
  if (g5::launch_dt_update(c->d_invdt, c->d_dt, dt_out, c->n_inst, c->phys.cfl, s) != cudaSuccess)
    return G5_ERR_CUDA;
  ++*launches;
  if (c->prm.integrator == 2)
  {
    // RK2_SSP (SolverGodunovFiveEq.cpp:496-524): U_RK = step(U); fill;
    // U2 = step(U_RK); U2 = 0.5 U + 0.5 U2 (with the CFL rate of the result)
    int rc = do_step(c, U, c->d_urk, c->d_dt, mode, nullptr, s);
    if (rc)
      return rc;
    *launches += c->last_launches;
    if (c->n_outside > 0)
    {
      if (g5::launch_fill_outside(c->dim, c->b, c->d_urk, dev_mesh(c), c->phys, s) != cudaSuccess)
        return G5_ERR_CUDA;
      ++*launches;
    }
    rc = do_step(c, c->d_urk, U2, c->d_dt, mode, nullptr, s);
    if (rc)
      return rc;
    *launches += c->last_launches;
    if (g5::launch_rk2_combine(c->dim, c->b, mode == G5_MODE_MIXED, U, U2, dev_mesh(c), c->phys, c->d_invdt, s) != cudaSuccess)
      return G5_ERR_CUDA;
    ++*launches;
    if (c->n_outside > 0)
    {
      if (g5::launch_fill_outside(c->dim, c->b, U2, dev_mesh(c), c->phys, s) != cudaSuccess)
        return G5_ERR_CUDA;
      ++*launches;
    }
    return G5_OK;
  }
  // 2D: the step kernel fills the outside blocks of U2 itself (and the
  // reflux pass patches the cells it finishes), so no separate fill launch
  int rc = do_step(c, U, U2, c->d_dt, mode, c->d_invdt, s, c->fused_fill);
  if (rc)
    return rc;
  *launches += c->last_launches;
  if (c->n_outside > 0 && !c->fused_fill)
  {
    if (g5::launch_fill_outside(c->dim, c->b, U2, dev_mesh(c), c->phys, s) != cudaSuccess)
      return G5_ERR_CUDA;
    ++*launches;
  }
  return G5_OK;
}
} // namespace

extern "C" int
g5_begin(G5Context * c, double * d_U, void * stream)
{
  if (!c || !c->has_mesh || !d_U)
    return G5_ERR_ARG;
  int rc = g5_fill_outside(c, d_U, stream);
  if (rc)
    return rc;
  rc = g5_compute_inv_dt(c, d_U, c->d_invdt, stream);
  c->last_launches = 2;
  return rc;
}

extern "C" int
g5_advance(G5Context * c, const double * d_U, double * d_U2, int mode, double * d_dt_out, void * stream)
{
  if (!c || !c->has_mesh || !d_U || !d_U2 || d_U == d_U2)
    return G5_ERR_ARG;
  if (mode != G5_MODE_FP64 && mode != G5_MODE_MIXED)
    return G5_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  // cached graph of one loop step for (U, U2, mode, dt_out)
  G5Context::GraphSlot * slot = nullptr;
  for (auto & g : c->graphs)
    if (g.exec && g.U == d_U && g.U2 == d_U2 && g.mode == mode && g.dt_out == d_dt_out)
      slot = &g;
  if (!slot)
  {
    slot = &c->graphs[c->next_graph];
    c->next_graph = (c->next_graph + 1) % G5Context::kGraphs;
    if (slot->exec)
    {
      cudaGraphExecDestroy(slot->exec);
      slot->exec = nullptr;
    }
    cudaStream_t cap;
    if (cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking) != cudaSuccess)
      return G5_ERR_CUDA;
    int         n = 0;
    cudaGraph_t g = nullptr;
    if (cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
    {
      cudaStreamDestroy(cap);
      return G5_ERR_CUDA;
    }
    int         rc = loop_step(c, d_U, d_U2, mode, d_dt_out, cap, &n);
    cudaError_t e = cudaStreamEndCapture(cap, &g);
    cudaStreamDestroy(cap);
    if (rc || e != cudaSuccess)
    {
      if (g)
        cudaGraphDestroy(g);
      return rc ? rc : G5_ERR_CUDA;
    }
    e = cudaGraphInstantiate(&slot->exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess)
    {
      slot->exec = nullptr;
      return G5_ERR_CUDA;
    }
    slot->U = d_U;
    slot->U2 = d_U2;
    slot->mode = mode;
    slot->dt_out = d_dt_out;
    slot->launches = n;
  }
  if (cudaGraphLaunch(slot->exec, s) != cudaSuccess)
    return G5_ERR_CUDA;
  c->last_launches = slot->launches;
  return G5_OK;
}

extern "C" int
g5_run(G5Context * c, double * d_U, double * d_U2, int nsteps, int mode, double * d_dt_hist, void * stream)
{
  if (!c || !c->has_mesh || !d_U || !d_U2 || nsteps < 0)
    return G5_ERR_ARG;
  if (mode != G5_MODE_FP64 && mode != G5_MODE_MIXED)
    return G5_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  int          rc = g5_begin(c, d_U, stream);
  if (rc)
    return rc;
  int launches = 2;
  for (int k = 0; k < nsteps; ++k)
  {
    double * A = (k & 1) ? d_U2 : d_U;
    double * B = (k & 1) ? d_U : d_U2;
    if (d_dt_hist)
      rc = loop_step(c, A, B, mode, d_dt_hist + (size_t)k * c->n_inst, s, &launches);
    else
    {
      rc = g5_advance(c, A, B, mode, nullptr, stream);
      launches += c->last_launches;
    }
    if (rc)
      return rc;
  }
  if (nsteps & 1)
  {
    // the final state is in U2: copy it back so that d_U holds it
    const size_t bytes = (size_t)c->n_total * c->nv * (c->dim == 2 ? c->b * c->b : c->b * c->b * c->b) * sizeof(double);
    if (cudaMemcpyAsync(d_U, d_U2, bytes, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
      return G5_ERR_CUDA;
  }
  c->last_launches = launches;
  return G5_OK;
}

extern "C" int
g5_status(G5Context * ctx, void * stream)
{
  if (!ctx)
    return G5_ERR_ARG;
  unsigned int h = 0;
  cudaStream_t s = (cudaStream_t)stream;
  if (cudaMemcpyAsync(&h, ctx->d_status, sizeof(h), cudaMemcpyDeviceToHost, s) != cudaSuccess)
    return G5_ERR_CUDA;
  if (cudaMemsetAsync(ctx->d_status, 0, sizeof(unsigned int), s) != cudaSuccess)
    return G5_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess)
    return G5_ERR_CUDA;
  return (int)h;
}

namespace
{
// packed launch shape: ctas_per_sm + 16 claim + 32 walk + 64 reflux
int
pack_shape(const G5Context::Shape & sh)
{
  return sh.ctas_per_sm + 16 * sh.claim + 32 * sh.walk + 64 * sh.reflux;
}
} // namespace

extern "C" int
g5_tune_pick(const float * ms, int n, int default_index, float margin)
{
  if (!ms || n <= 0 || default_index < 0 || default_index >= n || !(margin >= 0.0f))
    return G5_ERR_ARG;
  int best = -1;
  for (int i = 0; i < n; ++i)
    if (ms[i] > 0.0f && (best < 0 || ms[i] < ms[best]))
      best = i;
  if (best < 0)
    return G5_ERR_ARG;
  // the default shape stays unless another one is faster by more than the margin
  if (ms[default_index] > 0.0f && ms[default_index] <= ms[best] * (1.0f + margin))
    return default_index;
  return best;
}

extern "C" int
g5_tune(G5Context * c, const double * d_U, double * d_U2, int mode, void * stream)
{
  if (!c || !c->has_mesh || !d_U || !d_U2 || (mode != G5_MODE_FP64 && mode != G5_MODE_MIXED))
    return G5_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  const int    occ = mode == G5_MODE_FP64 ? g5::step_max_ctas_per_sm_fp64(c->dim, c->b) : g5::step_max_ctas_per_sm_mixed(c->dim, c->b);
  if (occ <= 0)
    return G5_ERR_UNSUPPORTED;
  // dt from the state itself
  int rc = g5_compute_inv_dt(c, d_U, c->d_invdt, stream);
  if (rc)
    return rc;
  if (g5::launch_dt_update(c->d_invdt, c->d_dt, nullptr, c->n_inst, c->phys.cfl, s) != cudaSuccess)
    return G5_ERR_CUDA;
  // candidates: CTAs per SM x block claiming x walk order x reflux layout
  // (the last only where it exists: the FP32-bulk 2D pass with records)
  std::vector<G5Context::Shape> cand;
  const int nreflux = (mode == G5_MODE_MIXED && c->dim == 2 && c->n_defer > 0) ? (c->n_fin > 0 ? 3 : 2) : 1;
  for (int k = 1; k <= occ && k < 16; ++k)
    for (int claim = 1; claim >= 0; --claim)
      for (int walk = 1; walk >= 0; --walk)
        for (int rf = 0; rf < nreflux; ++rf)
        {
          G5Context::Shape sh;
          sh.ctas_per_sm = k;
          sh.claim = claim;
          sh.walk = walk;
          sh.reflux = rf;
          cand.push_back(sh);
        }
  // the default: the occupancy maximum, claiming, coarse/fine-first walk,
  // records finished in the step's tail where that layout exists, else lanes
  const int def_reflux = nreflux == 3 ? 2 : 0;
  int       def = 0;
  for (size_t i = 0; i < cand.size(); ++i)
    if (cand[i].ctas_per_sm == occ && cand[i].claim == 1 && cand[i].walk == 1 && cand[i].reflux == def_reflux)
      def = (int)i;
  const G5Context::Shape saved = c->shape[mode];
  std::vector<float>     ms(cand.size(), 0.0f);
  cudaEvent_t            e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess)
    return G5_ERR_CUDA;
  if (cudaEventCreate(&e1) != cudaSuccess)
  {
    cudaEventDestroy(e0);
    return G5_ERR_CUDA;
  }
  constexpr int reps = 3;
  for (int pass = 0; pass < 2 && !rc; ++pass) // two passes, the best of both per candidate
    for (size_t i = 0; i < cand.size() && !rc; ++i)
    {
      c->shape[mode] = cand[i];
      rc = do_step(c, d_U, d_U2, c->d_dt, mode, nullptr, s); // warm-up
      if (rc)
        break;
      cudaEventRecord(e0, s);
      for (int r = 0; r < reps && !rc; ++r)
        rc = do_step(c, d_U, d_U2, c->d_dt, mode, nullptr, s);
      cudaEventRecord(e1, s);
      if (cudaEventSynchronize(e1) != cudaSuccess)
        rc = G5_ERR_CUDA;
      float t = 0.f;
      cudaEventElapsedTime(&t, e0, e1);
      t /= reps;
      ms[i] = (pass == 0 || t < ms[i]) ? t : ms[i];
    }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc)
  {
    c->shape[mode] = saved;
    return rc;
  }
  const int pick = g5_tune_pick(ms.data(), (int)ms.size(), def, 0.02f);
  c->shape[mode] = cand[pick < 0 ? def : pick];
  c->tune_log[mode].clear();
  for (size_t i = 0; i < cand.size(); ++i)
    c->tune_log[mode].emplace_back(pack_shape(cand[i]), ms[i]);
  drop_graphs(c);
  return pack_shape(c->shape[mode]);
}

extern "C" int
g5_tune_choice(const G5Context * c, int mode, int32_t * out4)
{
  if (!c || !out4 || (mode != G5_MODE_FP64 && mode != G5_MODE_MIXED))
    return G5_ERR_ARG;
  const G5Context::Shape & sh = c->shape[mode];
  const int occ = mode == G5_MODE_FP64 ? g5::step_max_ctas_per_sm_fp64(c->dim, c->b) : g5::step_max_ctas_per_sm_mixed(c->dim, c->b);
  out4[0] = sh.ctas_per_sm > 0 ? sh.ctas_per_sm : occ;
  out4[1] = sh.claim;
  out4[2] = sh.walk;
  out4[3] = sh.reflux;
  return G5_OK;
}

extern "C" int
g5_tune_report(const G5Context * c, int mode, int32_t * shapes, float * ms, int cap)
{
  if (!c || (mode != G5_MODE_FP64 && mode != G5_MODE_MIXED) || cap < 0)
    return G5_ERR_ARG;
  const auto & log = c->tune_log[mode];
  for (int i = 0; i < cap && i < (int)log.size(); ++i)
  {
    if (shapes)
      shapes[i] = log[i].first;
    if (ms)
      ms[i] = log[i].second;
  }
  return (int)log.size();
}

extern "C" int
g5_set_shape(G5Context * c, int mode, const int32_t * shape4)
{
  if (!c || !shape4 || (mode != G5_MODE_FP64 && mode != G5_MODE_MIXED))
    return G5_ERR_ARG;
  if (shape4[0] < 0 || shape4[0] > 15 || (shape4[1] & ~1) || (shape4[2] & ~1) || shape4[3] < 0 || shape4[3] > 2)
    return G5_ERR_ARG;
  G5Context::Shape sh;
  sh.ctas_per_sm = shape4[0];
  sh.claim = shape4[1];
  sh.walk = shape4[2];
  sh.reflux = shape4[3];
  c->shape[mode] = sh;
  drop_graphs(c);
  return G5_OK;
}

extern "C" int
g5_last_launch_count(const G5Context * ctx)
{
  return ctx ? ctx->last_launches : G5_ERR_ARG;
}
