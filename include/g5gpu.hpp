// g5gpu.hpp — C++17 host mirror of the reference's GodunovImplemBase over the
// C ABI of include/g5gpu.h (header-only; link libg5gpu.so and cudart).
//
// godunov_five_eq::GodunovImplemGB300<dim> keeps the member names and the
// argument meaning of the reference's GodunovImplemBase
// (scheme/GodunovImplemBase.h:59-198) and GodunovImplemV0
// (scheme/GodunovImplemV0.h:42-214):
//   resize_auxiliary_data(mesh)        <- block table of the new mesh
//   total_mem_size_in_bytes()
//   do_time_step(U, U2, dt)            U2 <- one step of U (device arrays)
//   do_time_step(U, U2, t, dt)         same (t unused, as in V0)
// plus the pieces of SolverGodunovFiveEq the step depends on:
//   compute_dt_local(U)                ComputeDtFiveEqFunctor + cfl / invDt
//   fill_outside_quadrants(U)          FillOutsideCellFunctor
//   remap_block_data(map, Uold, Unew)  UserDataRemapper after a mesh adaptation
//   compute_derived_quantity(U, q, o)  ComputeDerivedQuantities (output path)
//   pack_output_fields(U, f, n, out)   the datasets of one output, packed in one pass
//   do_time_step_host(hU, hU2, dt)     do_time_step on host-resident arrays
//   tune(U, U2), tune_choice(), set_shape(s)  launch shape of the step (no
//                                      counterpart: the reference's policies are fixed)
// Errors from the C ABI are thrown as g5::Error (the reference aborts).
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "g5gpu.h"

namespace g5
{

class Error : public std::runtime_error
{
public:
  Error(int code, const std::string & what)
    : std::runtime_error(what + ": g5 error " + std::to_string(code))
    , code_(code)
  {}
  int code() const { return code_; }

private:
  int code_;
};

inline void
check(int rc, const char * what)
{
  if (rc < 0)
    throw Error(rc, what);
}

// Stand-in for the reference's DataArrayBlock<dim, real_t, device_t>: a device
// array [n_blocks][nv][bsize^dim] of FP64 owned by the caller.
struct BlockArray
{
  double * data = nullptr;
  int      n_blocks = 0;
};

// Host copy of a block table (the arrays G5Mesh points to).
struct BlockTable
{
  int                  n_owned = 0, n_outside = 0, n_inst = 1;
  std::vector<int32_t> level, coord, nbr, out_src, inst;
  std::vector<int8_t>  nbr_rel, out_normal, out_border;

  G5Mesh view() const
  {
    G5Mesh m{};
    m.n_owned = n_owned;
    m.n_outside = n_outside;
    m.n_inst = n_inst;
    m.level = level.data();
    m.coord = coord.data();
    m.nbr = nbr.data();
    m.nbr_rel = nbr_rel.data();
    m.out_src = out_src.empty() ? nullptr : out_src.data();
    m.out_normal = out_normal.empty() ? nullptr : out_normal.data();
    m.out_border = out_border.empty() ? nullptr : out_border.data();
    m.inst = inst.empty() ? nullptr : inst.data();
    return m;
  }
};

// Uniform single-level block table on an nx x ny brick of blocks (2D), with
// the outside blocks of the non-periodic directions (one twin per border block
// and outside normal, as the reference's outside quadrants).  Blocks are
// ordered row by row.
inline BlockTable
uniform_block_table_2d(int nx, int ny, bool periodic_x, bool periodic_y, int level)
{
  BlockTable t;
  t.n_owned = nx * ny;
  auto id = [&](int i, int j) { return i + nx * j; };
  std::vector<int> okey; // outside blocks keyed by (i, j) position
  std::vector<int> oi, oj;
  auto find_out = [&](int i, int j) {
    for (size_t k = 0; k < oi.size(); ++k)
      if (oi[k] == i && oj[k] == j)
        return (int)k;
    return -1;
  };
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i)
    {
      t.level.push_back(level);
      t.coord.insert(t.coord.end(), { i, j, 0 });
    }
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i)
    {
      const int tx[3] = { 0, i == 0 && !periodic_x ? -1 : 0, i == nx - 1 && !periodic_x ? 1 : 0 };
      const int ty[3] = { 0, j == 0 && !periodic_y ? -1 : 0, j == ny - 1 && !periodic_y ? 1 : 0 };
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b)
        {
          const int nxo = tx[a], nyo = ty[b];
          if ((a > 0 && nxo == 0) || (b > 0 && nyo == 0) || (nxo == 0 && nyo == 0))
            continue;
          oi.push_back(i + nxo);
          oj.push_back(j + nyo);
          t.out_src.push_back(id(i, j));
          t.out_normal.insert(t.out_normal.end(), { (int8_t)nxo, (int8_t)nyo, 0 });
          t.out_border.insert(t.out_border.end(),
                              { (int8_t)(i == 0), (int8_t)(i == nx - 1), (int8_t)(j == 0), (int8_t)(j == ny - 1), 0, 0 });
          t.level.push_back(level);
          t.coord.insert(t.coord.end(), { i + nxo, j + nyo, 0 });
        }
    }
  t.n_outside = (int)oi.size();
  t.nbr.assign((size_t)t.n_owned * 9 * 4, -1);
  t.nbr_rel.assign((size_t)t.n_owned * 9, 0);
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i)
      for (int dy = -1; dy <= 1; ++dy)
        for (int dx = -1; dx <= 1; ++dx)
        {
          if (!dx && !dy)
            continue;
          int       ii = i + dx, jj = j + dy;
          const int s = (dx + 1) + 3 * (dy + 1);
          if (periodic_x)
            ii = (ii + nx) % nx;
          if (periodic_y)
            jj = (jj + ny) % ny;
          int n;
          if (ii >= 0 && ii < nx && jj >= 0 && jj < ny)
            n = id(ii, jj);
          else
            n = t.n_owned + find_out(ii, jj);
          t.nbr[((size_t)id(i, j) * 9 + s) * 4] = n;
        }
  (void)okey;
  return t;
}

// The host block forest of the dynamic AMR cycle (g5_forest_*): the
// adaptation that p4est performs in the reference, the old -> new block map
// for remap_block_data and the block table for resize_auxiliary_data.
class Forest
{
public:
  //! uniform at spec.level_min when `leaves` is empty, else those leaves ((level, x, y, z) rows)
  explicit Forest(const G5ForestSpec & spec, const std::vector<int32_t> & leaves = {})
    : m_dim(spec.dim)
  {
    check(g5_forest_create(&spec, leaves.empty() ? nullptr : leaves.data(), (int64_t)(leaves.size() / 4), &m_f), "g5_forest_create");
  }
  ~Forest()
  {
    if (m_f)
      g5_forest_destroy(m_f);
  }
  Forest(const Forest &) = delete;
  Forest & operator=(const Forest &) = delete;

  int64_t num_leaves() const { return g5_forest_num_leaves(m_f); }

  //! the leaves in table order, 4 int32 each
  std::vector<int32_t> leaves() const
  {
    std::vector<int32_t> out((size_t)num_leaves() * 4);
    check(g5_forest_leaves(m_f, out.data()), "g5_forest_leaves");
    return out;
  }

  int refine(const std::vector<int32_t> & keys) { return check(g5_forest_refine(m_f, keys.data(), (int64_t)(keys.size() / 4)), "g5_forest_refine"); }
  int balance() { return check(g5_forest_balance(m_f), "g5_forest_balance"); }

  //! one adaptation from ComputeRefineFlags codes (one per leaf, table order);
  //! fills kind / src (G5Remap's arrays) and returns the map
  G5Remap adapt(const std::vector<int8_t> & flags, std::vector<int8_t> & kind, std::vector<int32_t> & src)
  {
    const int64_t nc = (int64_t)1 << m_dim, cap = (int64_t)flags.size() * nc;
    kind.assign((size_t)cap, 0);
    src.assign((size_t)(cap * nc), -1);
    const int64_t n_new = g5_forest_adapt(m_f, flags.data(), (int64_t)flags.size(), kind.data(), src.data(), cap);
    if (n_new < 0)
      throw Error((int)n_new, "g5_forest_adapt");
    kind.resize((size_t)n_new);
    src.resize((size_t)(n_new * nc));
    G5Remap r{};
    r.n_old = (int32_t)flags.size();
    r.n_new = (int32_t)n_new;
    r.kind = kind.data();
    r.src = src.data();
    return r;
  }

  //! the block table of the current leaves
  BlockTable table()
  {
    int32_t no = 0, nt = 0;
    check(g5_forest_table_sizes(m_f, &no, &nt), "g5_forest_table_sizes");
    const int  ns = m_dim == 2 ? 9 : 27, nc = 1 << m_dim;
    BlockTable t;
    t.n_owned = no;
    t.n_outside = nt;
    t.level.resize((size_t)(no + nt));
    t.coord.resize((size_t)(no + nt) * 3);
    t.nbr.resize((size_t)no * ns * nc);
    t.nbr_rel.resize((size_t)no * ns);
    t.out_src.resize((size_t)nt);
    t.out_normal.resize((size_t)nt * 3);
    t.out_border.resize((size_t)nt * 6);
    check(g5_forest_table(m_f, t.level.data(), t.coord.data(), t.nbr.data(), t.nbr_rel.data(), t.out_src.data(), t.out_normal.data(),
                          t.out_border.data()),
          "g5_forest_table");
    return t;
  }

private:
  static int check(int rc, const char * what)
  {
    if (rc < 0)
      throw Error(rc, what);
    return rc;
  }
  int        m_dim;
  G5Forest * m_f = nullptr;
};

} // namespace g5

namespace godunov_five_eq
{

// GB300 implementation of GodunovImplemBase (implementation_version 3).
template <size_t dim>
class GodunovImplemGB300
{
public:
  static constexpr int implementation_version = 3;

  GodunovImplemGB300(const G5Params & params, int mode = G5_MODE_FP64, cudaStream_t stream = nullptr)
    : m_params(params)
    , m_mode(mode)
    , m_stream(stream)
  {
    if (params.dim != (int)dim)
      throw g5::Error(G5_ERR_ARG, "GodunovImplemGB300: dim mismatch");
    g5::check(g5_create(&params, &m_ctx), "g5_create");
  }
  ~GodunovImplemGB300()
  {
    if (m_ctx)
      g5_destroy(m_ctx);
  }
  GodunovImplemGB300(const GodunovImplemGB300 &) = delete;
  GodunovImplemGB300 & operator=(const GodunovImplemGB300 &) = delete;

  //! resize only auxiliary data array (GodunovImplemV0.cpp:37-61)
  void resize_auxiliary_data(const g5::BlockTable & table)
  {
    m_table = table;
    const G5Mesh m = m_table.view();
    g5::check(g5_set_mesh(m_ctx, &m), "g5_set_mesh");
  }

  //! memory footprint monitoring
  uint64_t total_mem_size_in_bytes() const { return (uint64_t)g5_mem_bytes(m_ctx); }

  //! Perform actual time integration: U2 <- step(U) (GodunovImplemV0.cpp:85-151)
  void do_time_step(const g5::BlockArray & U, const g5::BlockArray & U2, double dt)
  {
    std::vector<double> dts(m_table.n_inst, dt);
    g5::check(g5_step(m_ctx, U.data, U2.data, dts.data(), m_mode, nullptr, m_stream), "g5_step");
  }

  //! Perform actual time integration (t is unused, as in GodunovImplemV0)
  void do_time_step(const g5::BlockArray & U, const g5::BlockArray & U2, double /*t*/, double dt) { do_time_step(U, U2, dt); }

  //! SolverGodunovFiveEq::compute_dt_local: dt = cfl / max over cells of sum (c+|u_d|)/dx
  double compute_dt_local(const g5::BlockArray & U)
  {
    double * d_inv = nullptr;
    if (cudaMalloc(&d_inv, sizeof(double) * m_table.n_inst) != cudaSuccess)
      throw g5::Error(G5_ERR_CUDA, "cudaMalloc");
    int                 rc = g5_compute_inv_dt(m_ctx, U.data, d_inv, m_stream);
    std::vector<double> inv(m_table.n_inst);
    if (rc == 0 && cudaMemcpyAsync(inv.data(), d_inv, sizeof(double) * inv.size(), cudaMemcpyDeviceToHost, m_stream) != cudaSuccess)
      rc = G5_ERR_CUDA;
    if (rc == 0 && cudaStreamSynchronize(m_stream) != cudaSuccess)
      rc = G5_ERR_CUDA;
    cudaFree(d_inv);
    g5::check(rc, "g5_compute_inv_dt");
    return m_params.cfl / inv[0];
  }

  //! do_time_step for a solver whose U and U2 live in host memory (pinned for the
  //! copies to overlap the step): g5_step_host, then wait for the result
  void do_time_step_host(const double * h_U, double * h_U2, double dt)
  {
    std::vector<double> dts(m_table.n_inst, dt);
    g5::check(g5_step_host(m_ctx, h_U, h_U2, dts.data(), m_mode, nullptr, m_stream), "g5_step_host");
    if (cudaStreamSynchronize(m_stream) != cudaSuccess)
      throw g5::Error(G5_ERR_CUDA, "cudaStreamSynchronize");
  }

  //! ComputeDerivedQuantities::run (utils/ComputeDerivedQuantities.h:96-180) on all blocks:
  //! out[n_blocks][1][bsize^dim] receives quantity G5_DQ_*
  void compute_derived_quantity(const g5::BlockArray & U, int quantity, const g5::BlockArray & out)
  {
    g5::check(g5_derived_quantity(m_ctx, U.data, quantity, 0, U.n_blocks, out.data, m_stream), "g5_derived_quantity");
  }

  //! the datasets of one output of SolverGodunovFiveEq::save_solution_hdf5
  //! (SolverGodunovFiveEq.cpp:809-886) for blocks [0, n_blocks) of U: fields
  //! are state variable ids or G5_FIELD_DERIVED + G5_DQ_*, out holds
  //! fields.size() x n_blocks x bsize^dim doubles on the device
  void pack_output_fields(const g5::BlockArray & U, const std::vector<int32_t> & fields, int64_t n_blocks, double * d_out)
  {
    g5::check(g5_pack_fields(m_ctx, U.data, fields.data(), (int)fields.size(), 0, n_blocks, d_out, m_stream), "g5_pack_fields");
  }

  //! SolverGodunovFiveEq::fill_outside_quadrants
  void fill_outside_quadrants(const g5::BlockArray & U) { g5::check(g5_fill_outside(m_ctx, U.data, m_stream), "g5_fill_outside"); }

  //! SolverGodunovFiveEq::map_userdata_after_adapt (SolverGodunovFiveEq.cpp:1137-1169):
  //! owned blocks of U_new from U_old by the old -> new block map of one adaptation
  void remap_block_data(const G5Remap & remap, const g5::BlockArray & U_old, const g5::BlockArray & U_new)
  {
    g5::check(g5_remap(m_ctx, &remap, U_old.data, U_new.data, m_stream), "g5_remap");
  }

  //! device status word (G5_STATUS_* bits), cleared by the read
  int status() { return g5_status(m_ctx, m_stream); }

  //! launch shape of the step for the current mesh and the context's mode:
  //! every candidate timed on U -> U2 (U2 overwritten, the stream
  //! synchronised), the fastest kept; returns {CTAs per SM, claim, walk, reflux layout}
  std::vector<int32_t> tune(const g5::BlockArray & U, const g5::BlockArray & U2)
  {
    g5::check(g5_tune(m_ctx, U.data, U2.data, m_mode, m_stream), "g5_tune");
    return tune_choice();
  }

  //! the launch shape in use for the context's mode
  std::vector<int32_t> tune_choice() const
  {
    std::vector<int32_t> s(4);
    g5::check(g5_tune_choice(m_ctx, m_mode, s.data()), "g5_tune_choice");
    return s;
  }

  //! set the launch shape by hand ({CTAs per SM (0: occupancy maximum), claim, walk, reflux layout})
  void set_shape(const std::vector<int32_t> & shape4)
  {
    if (shape4.size() != 4)
      throw g5::Error(G5_ERR_ARG, "set_shape: four values");
    g5::check(g5_set_shape(m_ctx, m_mode, shape4.data()), "g5_set_shape");
  }

  G5Context * context() const { return m_ctx; }

private:
  G5Params       m_params;
  int            m_mode;
  cudaStream_t   m_stream;
  G5Context *    m_ctx = nullptr;
  g5::BlockTable m_table;
};

} // namespace godunov_five_eq
