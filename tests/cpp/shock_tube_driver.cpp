// C++ integration driver: the gas-water shock tube (ZERO_GRADIENT in x,
// periodic in y, 16x2 blocks of 8x8) advanced with
// godunov_five_eq::GodunovImplemGB300<2> (include/g5gpu.hpp) the way the
// reference's SolverGodunovFiveEq::godunov_unsplit drives its implementation
// (fill outside quadrants, dt, do_time_step, swap), checked bit for bit
// against the CPU oracle on the same block table; then one step through host
// buffers (g5_step_host) against the device step and the derived thermal
// pressure against the oracle.  Prints "OK" on success.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/g5gpu.hpp"
#include "../../oracle/g5_oracle.h"

int
main(int argc, char ** argv)
{
  const int nsteps = argc > 1 ? std::atoi(argv[1]) : 10;
  const int b = 8, nx = 16, ny = 2, level = 1, nv = 8, nc = b * b;
  G5Params  p{};
  p.dim = 2;
  p.bsize = b;
  p.integrator = 0;
  p.bc[0] = p.bc[1] = G5_BC_ZERO_GRADIENT;
  p.bc[2] = p.bc[3] = p.bc[4] = p.bc[5] = G5_BC_PERIODIC;
  p.gamma[0] = 4.4;
  p.gamma[1] = 1.4;
  p.pinf[0] = 6e8;
  p.pinf[1] = 0.0;
  p.smallr = 1e-10;
  p.smallc = 1e-10;
  p.slope_type = 1.0;
  p.cfl = 0.4;
  const double scaling = 1.0 / (nx >> level);
  for (int l = 0; l < 32; ++l)
    p.level_dx[l] = (1.0 / (double)(b << l)) * scaling;

  g5::BlockTable      t = g5::uniform_block_table_2d(nx, ny, false, true, level);
  const int           n_total = t.n_owned + t.n_outside;
  std::vector<double> U((size_t)n_total * nv * nc, 0.0);
  // water at x < 0.5 (p = 1e9), air at x > 0.5 (p = 1e5), both at rest
  for (int n = 0; n < t.n_owned; ++n)
    for (int c = 0; c < nc; ++c)
    {
      const double x = (t.coord[n * 3] * b + c % b + 0.5) * p.level_dx[level];
      const bool   left = x < 0.5;
      const double a0 = left ? 1 - 1e-6 : 1e-6, ar0 = a0 * 1000.0, ar1 = (1 - a0) * 50.0, pr = left ? 1e9 : 1e5;
      const double xi0 = 1 / (p.gamma[0] - 1), xi1 = 1 / (p.gamma[1] - 1);
      const double S = a0 * xi0 + (1 - a0) * xi1, PI = a0 * p.gamma[0] * p.pinf[0] * xi0;
      double *     u = &U[(size_t)n * nv * nc + c];
      u[0 * nc] = ar0 + ar1;
      u[1 * nc] = pr * S + PI;
      u[4 * nc] = a0;
      u[5 * nc] = ar0;
      u[6 * nc] = 1 - a0;
      u[7 * nc] = ar1;
    }

  // ---- GPU: the reference's step loop over the C++ mirror
  godunov_five_eq::GodunovImplemGB300<2> impl(p);
  impl.resize_auxiliary_data(t);
  g5::BlockArray A, B;
  const size_t   bytes = U.size() * sizeof(double);
  if (cudaMalloc(&A.data, bytes) != cudaSuccess || cudaMalloc(&B.data, bytes) != cudaSuccess)
    return 2;
  A.n_blocks = B.n_blocks = n_total;
  cudaMemcpy(A.data, U.data(), bytes, cudaMemcpyHostToDevice);
  cudaMemcpy(B.data, U.data(), bytes, cudaMemcpyHostToDevice);
  // the launch shape tuned for this mesh (every candidate gives the same bits;
  // B is overwritten by the timing runs), read back and set again by hand
  impl.fill_outside_quadrants(A);
  const std::vector<int32_t> shape = impl.tune(A, B);
  if (shape.size() != 4 || shape[0] < 0 || impl.tune_choice() != shape)
  {
    std::printf("tune: unexpected shape\n");
    return 1;
  }
  impl.set_shape(shape);
  std::vector<double> dts;
  for (int k = 0; k < nsteps; ++k)
  {
    impl.fill_outside_quadrants(A);
    const double dt = impl.compute_dt_local(A);
    dts.push_back(dt);
    impl.do_time_step(A, B, dt);
    std::swap(A, B);
  }
  std::vector<double> G(U.size());
  cudaMemcpy(G.data(), A.data, bytes, cudaMemcpyDeviceToHost);
  if (impl.status() != 0)
  {
    std::printf("device status raised\n");
    return 1;
  }

  // ---- oracle on the same table
  G5OParams op{};
  op.dim = 2;
  op.b = b;
  std::memcpy(op.bc, p.bc, sizeof(op.bc));
  std::memcpy(op.gamma, p.gamma, sizeof(op.gamma));
  std::memcpy(op.pinf, p.pinf, sizeof(op.pinf));
  op.smallr = p.smallr;
  op.smallc = p.smallc;
  op.slope_type = p.slope_type;
  op.cfl = p.cfl;
  std::memcpy(op.level_dx, p.level_dx, sizeof(op.level_dx));
  G5OMesh om{};
  const G5Mesh gm = t.view();
  om.n_owned = gm.n_owned;
  om.n_outside = gm.n_outside;
  om.n_inst = 1;
  om.level = gm.level;
  om.coord = gm.coord;
  om.nbr = gm.nbr;
  om.nbr_rel = gm.nbr_rel;
  om.out_src = gm.out_src;
  om.out_normal = gm.out_normal;
  om.out_border = gm.out_border;
  om.inst = gm.inst;
  void *              o = g5o_create(&om, &op, 0);
  std::vector<double> R = U, R2 = U;
  for (int k = 0; k < nsteps; ++k)
  {
    g5o_fill_outside(o, R.data());
    double inv = 0;
    g5o_inv_dt(o, R.data(), &inv);
    const double dt = op.cfl / inv;
    if (dt != dts[k])
    {
      std::printf("dt differs at step %d: %.17g vs %.17g\n", k, dt, dts[k]);
      return 1;
    }
    g5o_step(o, R.data(), R2.data(), &dt);
    std::swap(R, R2);
  }
  g5o_destroy(o);
  size_t diff = 0;
  for (size_t i = 0; i < (size_t)t.n_owned * nv * nc; ++i)
    diff += G[i] != R[i];
  if (diff)
  {
    std::printf("%zu values differ\n", diff);
    return 1;
  }
  // ---- one more step through host buffers (g5_step_host) against the device step
  {
    double * hU = nullptr;
    double * hO = nullptr;
    if (cudaMallocHost(&hU, bytes) != cudaSuccess || cudaMallocHost(&hO, bytes) != cudaSuccess)
      return 2;
    impl.fill_outside_quadrants(A);
    const double dt = impl.compute_dt_local(A);
    cudaMemcpy(hU, A.data, bytes, cudaMemcpyDeviceToHost);
    impl.do_time_step_host(hU, hO, dt);
    impl.do_time_step(A, B, dt);
    std::vector<double> D(U.size());
    cudaMemcpy(D.data(), B.data, bytes, cudaMemcpyDeviceToHost);
    size_t hd = 0;
    for (size_t i = 0; i < (size_t)t.n_owned * nv * nc; ++i)
      hd += hO[i] != D[i];
    cudaFreeHost(hU);
    cudaFreeHost(hO);
    if (hd)
    {
      std::printf("host-buffer step: %zu values differ\n", hd);
      return 1;
    }
  }
  // ---- derived quantity (thermal pressure) against the oracle
  {
    g5::BlockArray P;
    P.n_blocks = n_total;
    if (cudaMalloc(&P.data, (size_t)n_total * nc * sizeof(double)) != cudaSuccess)
      return 2;
    impl.compute_derived_quantity(A, G5_DQ_THERMAL_PRESSURE, P);
    std::vector<double> GP((size_t)n_total * nc), OP((size_t)n_total * nc);
    cudaMemcpy(GP.data(), P.data, GP.size() * sizeof(double), cudaMemcpyDeviceToHost);
    cudaMemcpy(G.data(), A.data, bytes, cudaMemcpyDeviceToHost);
    g5o_derived(&op, G.data(), G5_DQ_THERMAL_PRESSURE, 0, n_total, OP.data());
    cudaFree(P.data);
    size_t pd = 0;
    for (size_t i = 0; i < GP.size(); ++i)
      pd += GP[i] != OP[i];
    if (pd)
    {
      std::printf("derived pressure: %zu values differ\n", pd);
      return 1;
    }
  }
  std::printf("OK %d steps, %d blocks, %zu bytes of context memory\n", nsteps, t.n_owned, (size_t)impl.total_mem_size_in_bytes());
  cudaFree(A.data);
  cudaFree(B.data);
  return 0;
}
