// Stand-ins for the parts of the external kalypsso core that the reference's
// scheme functors name (kalypsso_data_container.h, utils_block.h,
// orchard keys, AMRMeshInfo, conformal face status, StencilHelper, the time
// integrator and THINC settings, gravity, the Youngs normal, cell lengths).
// Test infrastructure: it lets the reference's own scheme code compile and run
// serially on one block of same-level neighbours, so that its results pin the
// CPU oracle.  Every arithmetic definition here is a restatement (the core is
// absent) and is the same as the oracle's:
//   * compute_cell_length(level, bx) = 1 / (bx 2^level) (scaling applied by
//     the caller, as in the reference);
//   * Youngs normal: (1,2,1)-weighted central differences of the volume
//     fraction, n = -grad / |grad|;
//   * tanh: the oracle's own g5o_tanh (libm's tanh differs between hosts),
//     substituted through kalypsso::tanh, which the reference's unqualified
//     tanh calls find first.
//   * StencilHelper's neighbour lookup on a periodic tile of same-level
//     blocks (the refinement indicators read their neighbours through it).
// What a same-level block never reaches (finer-neighbour face sums and
// averages through StencilHelper) aborts if called.
#pragma once
#include <algorithm>
#include <array>
#include <cstdint>
#include <string>
#include <utility>
#include <vector>

#include <../better-enums/enum.h>
#include <kalypsso/core/kokkos_shared.h>
#include <kalypsso/core/real_type.h>
#include <kalypsso/utils/config/ConfigMap.h>
#include <kalypsso/utils/log/kalypsso_log.h>

extern "C" double g5o_tanh(double);

// element-wise arithmetic of small state arrays, in namespace Kokkos so that
// argument-dependent lookup finds it wherever the reference uses it
namespace Kokkos
{
template <typename T, size_t N>
Kokkos::Array<T, N>
operator+(Kokkos::Array<T, N> const & a, Kokkos::Array<T, N> const & b)
{
  Kokkos::Array<T, N> r;
  for (size_t i = 0; i < N; ++i)
    r[i] = a[i] + b[i];
  return r;
}
template <typename T, size_t N>
Kokkos::Array<T, N>
operator-(Kokkos::Array<T, N> const & a, Kokkos::Array<T, N> const & b)
{
  Kokkos::Array<T, N> r;
  for (size_t i = 0; i < N; ++i)
    r[i] = a[i] - b[i];
  return r;
}
template <typename T, size_t N, typename S>
Kokkos::Array<T, N>
operator*(Kokkos::Array<T, N> const & a, S s)
{
  Kokkos::Array<T, N> r;
  for (size_t i = 0; i < N; ++i)
    r[i] = a[i] * s;
  return r;
}
template <typename T, size_t N, typename S>
Kokkos::Array<T, N>
operator/(Kokkos::Array<T, N> const & a, S s)
{
  Kokkos::Array<T, N> r;
  for (size_t i = 0; i < N; ++i)
    r[i] = a[i] / s;
  return r;
}

} // namespace Kokkos

namespace kalypsso
{
// the oracle's tanh for the reference's unqualified tanh(...) calls
inline double
tanh(double x)
{
  return g5o_tanh(x);
}

enum : int
{
  IX = 0,
  IY = 1,
  IZ = 2
};
using iOct_t = int32_t;

template <size_t dim, typename T = int32_t>
using coord_t = Kokkos::Array<T, dim>;
template <size_t dim>
using shift_t = Kokkos::Array<int32_t, dim>;
template <size_t dim>
using block_size_t = Kokkos::Array<int32_t, dim>;
template <size_t dim>
using brick_size_t = Kokkos::Array<int32_t, dim>;

template <typename T, size_t N>
constexpr Kokkos::Array<T, N>
init_kokkos_array(T v)
{
  Kokkos::Array<T, N> a{};
  for (size_t i = 0; i < N; ++i)
    a[i] = v;
  return a;
}

template <typename T>
KOKKOS_INLINE_FUNCTION void
my_swap(T & a, T & b)
{
  T t = a;
  a = b;
  b = t;
}

#define assertm(exp, msg) ((void)0)

template <size_t dim>
KOKKOS_INLINE_FUNCTION coord_t<dim>
cell_index_unravel(int64_t index, block_size_t<dim> const & shape)
{
  coord_t<dim> c{};
  c[IX] = static_cast<int32_t>(index % shape[IX]);
  c[IY] = static_cast<int32_t>((index / shape[IX]) % shape[IY]);
  if constexpr (dim == 3)
    c[IZ] = static_cast<int32_t>(index / (shape[IX] * shape[IY]));
  return c;
}

template <size_t dim>
KOKKOS_INLINE_FUNCTION coord_t<dim>
cellindex_to_coord(int64_t index, block_size_t<dim> const & ghosted_size, shift_t<dim> const & shift)
{
  coord_t<dim> c = cell_index_unravel<dim>(index, ghosted_size);
  for (size_t e = 0; e < dim; ++e)
    c[e] -= shift[e];
  return c;
}

template <size_t dim>
KOKKOS_INLINE_FUNCTION coord_t<dim>
cellindex_to_coord(int64_t index, block_size_t<dim> const & block_size)
{
  return cell_index_unravel<dim>(index, block_size);
}

template <size_t dim>
KOKKOS_INLINE_FUNCTION coord_t<dim>
get_unit_vector(int dir)
{
  coord_t<dim> u{};
  for (size_t e = 0; e < dim; ++e)
    u[e] = (static_cast<int>(e) == dir) ? 1 : 0;
  return u;
}

template <size_t dim>
block_size_t<dim>
get_flux_block_sizes(block_size_t<dim> bs, int direction)
{
  bs[direction] += 1;
  return bs;
}

// block array [n_quadrants][n_vars][cells], cell index x fastest
template <size_t dim, typename T, typename device_t>
class DataArrayBlock
{
public:
  std::shared_ptr<std::vector<T>> s;
  block_size_t<dim>               bs{};
  int32_t                         nvar = 0, nquad = 0;
  DataArrayBlock() = default;
  DataArrayBlock(block_size_t<dim> b, int32_t nv, int32_t nq)
    : s(std::make_shared<std::vector<T>>((size_t)Kokkos::dim_prod(b) * nv * nq))
    , bs(b)
    , nvar(nv)
    , nquad(nq)
  {}
  int32_t           num_cells() const { return Kokkos::dim_prod(bs); }
  int32_t           num_vars() const { return nvar; }
  int32_t           num_quadrants() const { return nquad; }
  block_size_t<dim> block_size() const { return bs; }
  block_size_t<dim> shape() const { return bs; }
  void              reshape(block_size_t<dim> b) { bs = b; }
  T *               data() const { return s->data(); }
  T &               operator()(int64_t cell, int var, int64_t oct) const
  {
    return (*s)[((size_t)oct * nvar + var) * num_cells() + cell];
  }
  T & operator()(int32_t i, int32_t j, int var, int32_t oct) const { return (*this)(i + (int64_t)bs[IX] * j, var, oct); }
  T & operator()(int32_t i, int32_t j, int32_t k, int var, int32_t oct) const
  {
    return (*this)(i + (int64_t)bs[IX] * (j + (int64_t)bs[IY] * k), var, oct);
  }
};

// ghosted block array: cells -g .. b+g-1 along each direction
template <size_t dim, typename T, typename device_t>
class DataArrayGhostedBlock
{
public:
  std::shared_ptr<std::vector<T>> s;
  block_size_t<dim>               bs{}, gbs{};
  int32_t                         g = 0, nvar = 0, nquad = 0;
  DataArrayGhostedBlock() = default;
  DataArrayGhostedBlock(block_size_t<dim> b, int32_t ghost, int32_t nv, int32_t nq)
    : bs(b)
    , g(ghost)
    , nvar(nv)
    , nquad(nq)
  {
    for (size_t e = 0; e < dim; ++e)
      gbs[e] = b[e] + 2 * ghost;
    s = std::make_shared<std::vector<T>>((size_t)Kokkos::dim_prod(gbs) * nv * nq);
  }
  int32_t           num_cells() const { return Kokkos::dim_prod(gbs); }
  int32_t           num_vars() const { return nvar; }
  int32_t           num_quadrants() const { return nquad; }
  block_size_t<dim> block_size() const { return bs; }
  block_size_t<dim> ghosted_block_size() const { return gbs; }
  shift_t<dim>      shift() const { return init_kokkos_array<int32_t, dim>(g); }
  int32_t           ghost_width() const { return g; }
  T *               data() const { return s->data(); }
  T &               operator()(int64_t cell, int var, int64_t oct) const
  {
    return (*s)[((size_t)oct * nvar + var) * num_cells() + cell];
  }
  T & operator()(int32_t i, int32_t j, int var, int32_t oct) const
  {
    return (*this)((i + g) + (int64_t)gbs[IX] * (j + g), var, oct);
  }
  T & operator()(int32_t i, int32_t j, int32_t k, int var, int32_t oct) const
  {
    return (*this)((i + g) + (int64_t)gbs[IX] * ((j + g) + (int64_t)gbs[IY] * (k + g)), var, oct);
  }
};

// orchard keys: the shim's key is the block's AMR level
template <typename device_t>
struct orchard_key_base_t
{
  using key_t = uint64_t;
  using view_t = Kokkos::View<uint64_t *, device_t>;
};
// The boundary fill's view of the block table (FillOutside pin, set by the
// refpin driver): keys are block indices (owned blocks first, then the outside
// quadrants); per outside quadrant o its inside source block, its outside
// normal and the domain-border faces of that source block, as the block table
// of the GPU path describes them.
namespace refpin_fill
{
struct Table
{
  int32_t         n_owned = 0, n_outside = 0;
  const int32_t * out_src = nullptr;    // [n_outside]
  const int8_t *  out_normal = nullptr; // [n_outside * 3]
  const int8_t *  out_border = nullptr; // [n_outside * 6]
  std::vector<int8_t> border_of;        // [n_owned * 6] from out_border by source block
};
inline Table &
table()
{
  static Table t;
  return t;
}
} // namespace refpin_fill

template <size_t dim>
struct orchard_key_t
{
  static KOKKOS_INLINE_FUNCTION int level(uint64_t key) { return static_cast<int>(key); }
  // FillOutside pin (refpin_fill keys)
  static Kokkos::Array<int32_t, dim> get_outside_normal(uint64_t key, brick_size_t<dim> const &, Kokkos::Array<bool, dim> const &)
  {
    const auto &                tb = refpin_fill::table();
    Kokkos::Array<int32_t, dim> nrm{};
    for (size_t e = 0; e < dim; ++e)
      nrm[e] = tb.out_normal[(size_t)(key - tb.n_owned) * 3 + e];
    return nrm;
  }
  static int32_t is_touching_face(uint64_t key, int dir)
  {
    const auto & tb = refpin_fill::table();
    return tb.out_normal[(size_t)(key - tb.n_owned) * 3 + dir] != 0 ? 1 : 0;
  }
  static int32_t is_touching_face_X(uint64_t key) { return is_touching_face(key, 0); }
  static int32_t is_touching_face_Y(uint64_t key) { return is_touching_face(key, 1); }
  static int32_t is_touching_face_Z(uint64_t key) { return is_touching_face(key, 2); }
  static uint64_t get_neighbor_key_same_level(uint64_t key, Kokkos::Array<int32_t, dim> const &, brick_size_t<dim> const &,
                                              Kokkos::Array<bool, dim> const &)
  {
    const auto & tb = refpin_fill::table();
    return (uint64_t)tb.out_src[key - tb.n_owned];
  }
  static void reset_outside_bits(uint64_t &) {}
  static bool is_at_domain_border(uint64_t key_inside, int face, brick_size_t<dim> const &)
  {
    return refpin_fill::table().border_of[(size_t)key_inside * 6 + face] != 0;
  }
  static bool is_outside_dir(uint64_t key_outside, int dir) { return is_touching_face(key_outside, dir) != 0; }
};

template <typename device_t>
struct hashmap_base_t
{
  struct map_t
  {};
};

class AMRMeshInfo
{
public:
  int32_t n_owned = 0, n_ghosts = 0, n_outside = 0;
  AMRMeshInfo() = default;
  AMRMeshInfo(int32_t o, int32_t g, int32_t out = 0)
    : n_owned(o)
    , n_ghosts(g)
    , n_outside(out)
  {}
  int32_t local_num_quadrants() const { return n_owned; }
  int32_t local_num_ghosts() const { return n_ghosts; }
  // outside quadrants follow the owned ones (no ghosts in a one-rank pin)
  int32_t first_outside_quad_local_id() const { return n_owned + n_ghosts; }
  int32_t total_local_number_of_outside_quads() const { return n_outside; }
};

// faces xmin xmax ymin ymax zmin zmax and directions
namespace Face
{
using face_t = int;
template <size_t dim>
constexpr Kokkos::Array<int, 2 * dim>
get_all_faces()
{
  Kokkos::Array<int, 2 * dim> f{};
  for (size_t i = 0; i < 2 * dim; ++i)
    f[i] = (int)i;
  return f;
}
KOKKOS_INLINE_FUNCTION constexpr bool
is_left_face(int face)
{
  return (face & 1) == 0;
}
} // namespace Face
namespace Dir
{
using dir_t = int;
}

template <size_t dim>
constexpr Kokkos::Array<bool, dim>
get_bool_array(bool v)
{
  Kokkos::Array<bool, dim> a{};
  for (size_t i = 0; i < dim; ++i)
    a[i] = v;
  return a;
}

// brick settings read by functor constructors (unused by the pin's keys)
template <size_t dim>
brick_size_t<dim>
get_brick_sizes(ConfigMap const & cm)
{
  brick_size_t<dim> b{};
  for (size_t e = 0; e < dim; ++e)
    b[e] = cm.getInteger("refpin", "brick" + std::to_string(e), 1);
  return b;
}
template <size_t dim>
Kokkos::Array<bool, dim>
get_brick_periodicity(ConfigMap const & cm)
{
  Kokkos::Array<bool, dim> p{};
  for (size_t e = 0; e < dim; ++e)
    p[e] = cm.getBool("refpin", "periodic" + std::to_string(e), false);
  return p;
}

// border conditions per face from the config ("refpin/bc<face>" integers,
// the enum's integral values), as BorderConditionsConfig hands them over
template <typename BC>
struct BorderConditionsConfig
{
  template <size_t dim>
  using bc_array_t = Kokkos::Array<BC, 2 * dim>;
  template <size_t dim, size_t... I>
  static bc_array_t<dim> read_faces(ConfigMap const & cm, std::index_sequence<I...>)
  {
    return bc_array_t<dim>{ { BC(static_cast<typename BC::_enumerated>(cm.getInteger("refpin", "bc" + std::to_string(I), 0)))... } };
  }
  template <size_t dim, typename PE>
  static bc_array_t<dim> read_border_condition(ConfigMap const & cm, PE const &)
  {
    return read_faces<dim>(cm, std::make_index_sequence<2 * dim>{});
  }
};

// the block index of a key (refpin_fill keys are block indices)
template <typename M>
std::pair<bool, int32_t>
key_to_value(uint64_t key, M const &)
{
  return { true, static_cast<int32_t>(key) };
}

// conformal face status: 2 bits per face (xmin xmax ymin ymax zmin zmax)
enum class conformal_neighbor_status : uint8_t
{
  NEIGHBOR_IS_SAME_SIZE = 0,
  NEIGHBOR_IS_LARGER = 1,
  NEIGHBOR_IS_FINER = 2,
  NEIGHBOR_IS_OUTSIDE = 3
};
template <size_t dim, typename device_t>
using conformal_status_view_t = Kokkos::View<uint16_t *, device_t>;
template <size_t dim>
struct conformal_face_status_t
{
  static conformal_neighbor_status face(uint16_t s, int f) { return static_cast<conformal_neighbor_status>((s >> (2 * f)) & 3u); }
  static conformal_neighbor_status face_xmin(uint16_t s) { return face(s, 0); }
  static conformal_neighbor_status face_xmax(uint16_t s) { return face(s, 1); }
  static conformal_neighbor_status face_ymin(uint16_t s) { return face(s, 2); }
  static conformal_neighbor_status face_ymax(uint16_t s) { return face(s, 3); }
  static conformal_neighbor_status face_zmin(uint16_t s) { return face(s, 4); }
  static conformal_neighbor_status face_zmax(uint16_t s) { return face(s, 5); }
};

template <size_t dim, typename device_t>
struct AMRContext
{
  using amrflags_view_t = Kokkos::View<int8_t *, device_t>;
};

template <size_t dim>
struct CellLocation
{
  coord_t<dim> ijk;
  uint64_t     key;
  int32_t      iOct;
  bool         is_ghost;
  bool         is_outside_domain = false;
  int          level() const { return static_cast<int>(key); }
};

template <size_t dim>
KOKKOS_INLINE_FUNCTION int32_t
coord_to_cellindex(coord_t<dim> const & c, block_size_t<dim> const & bs)
{
  int32_t i = c[IX] + bs[IX] * c[IY];
  if constexpr (dim == 3)
    i += bs[IX] * bs[IY] * c[IZ];
  return i;
}

template <size_t dim, int dir>
constexpr shift_t<dim>
get_shift_left()
{
  shift_t<dim> s{};
  s[dir] = -1;
  return s;
}
template <size_t dim, int dir>
constexpr shift_t<dim>
get_shift_right()
{
  shift_t<dim> s{};
  s[dir] = 1;
  return s;
}

// refinement flags of the AMR context (-1 init, 0 coarsen, 1 nothing, 2 refine)
struct AMRContextBase
{
  using amrflag_t = int8_t;
  static constexpr amrflag_t KALYPSSO_FLAG_INIT = -1;
  static constexpr amrflag_t KALYPSSO_DO_COARSEN = 0;
  static constexpr amrflag_t KALYPSSO_DO_NOTHING = 1;
  static constexpr amrflag_t KALYPSSO_DO_REFINE = 2;
};

BETTER_ENUM(Indicator, int, LOHNER_SPLIT, LOHNER_UNSPLIT, SIMPLE_GRADIENT)
struct RefineIndicatorData
{
  Indicator indicator = Indicator::SIMPLE_GRADIENT;
  real_t    epsilon = 0.02;
  real_t    refine_th = 0.1;
  real_t    coarsen_th = 0.0125;
  int       level_min = 0;
  int       level_max = 30;
};

namespace KokkosExt
{
template <typename T>
KOKKOS_INLINE_FUNCTION T
max_val(T a, T b)
{
  return a > b ? a : b;
}
} // namespace KokkosExt

template <typename T, typename device_t>
using DataArrayLeaf = Kokkos::View<T *, device_t>;

struct ParallelEnv
{};

// |x| of the reference's unqualified abs(...) on reals
inline double
abs(double x)
{
  return std::fabs(x);
}

// Neighbour lookup on a periodic tile of same-level blocks (blocks numbered x
// fastest over the brick of the constructor, level in the key): the cell at
// ijk + shift, in this block or in the neighbour block it falls in.  The
// lookups across levels (finer neighbours' face sums and averages) are not
// reached by such tiles and abort if called.
template <size_t dim, typename device_t>
class StencilHelper
{
public:
  typename orchard_key_base_t<device_t>::view_t keys;
  block_size_t<dim>                             bs{};
  brick_size_t<dim>                             nb{};
  StencilHelper() = default;
  template <typename M>
  StencilHelper(M const &, typename orchard_key_base_t<device_t>::view_t const & k, block_size_t<dim> b, brick_size_t<dim> n,
                Kokkos::Array<bool, dim>)
    : keys(k)
    , bs(b)
    , nb(n)
  {}
  uint64_t          key(int32_t iOct) const { return keys(iOct); }
  CellLocation<dim> getNeighLoc(CellLocation<dim> const & loc, shift_t<dim> const & shift) const
  {
    CellLocation<dim> out = loc;
    int32_t           bc[3] = { 0, 0, 0 }, o = loc.iOct;
    for (size_t e = 0; e < dim; ++e)
    {
      bc[e] = o % nb[e];
      o /= nb[e];
    }
    int32_t oct = 0, mul = 1;
    for (size_t e = 0; e < dim; ++e)
    {
      int32_t c = loc.ijk[e] + shift[e];
      int32_t b = bc[e];
      while (c < 0)
      {
        c += bs[e];
        b -= 1;
      }
      while (c >= bs[e])
      {
        c -= bs[e];
        b += 1;
      }
      b = ((b % nb[e]) + nb[e]) % nb[e];
      out.ijk[e] = c;
      oct += b * mul;
      mul *= nb[e];
    }
    out.iOct = oct;
    out.key = keys(oct);
    out.is_outside_domain = false;
    return out;
  }
  CellLocation<dim> getNeighLocFinerNearer(CellLocation<dim> const &, shift_t<dim> const &) const
  {
    Kokkos::abort("refpin: finer-neighbour lookup is outside the same-level pin");
    return {};
  }
  template <typename A>
  real_t compute_face_siblings_sum(CellLocation<dim> const &, int, A const &, bool) const
  {
    Kokkos::abort("refpin: finer-neighbour face sum is outside the same-level pin");
    return 0;
  }
  template <typename A>
  real_t compute_siblings_average(CellLocation<dim> const &, block_size_t<dim> const &, int, A const &) const
  {
    Kokkos::abort("refpin: finer-neighbour average is outside the same-level pin");
    return 0;
  }
};

template <size_t dim>
struct UniformGravityField
{
  real_t            g[3] = { 0, 0, 0 };
  KOKKOS_INLINE_FUNCTION real_t operator[](int e) const { return g[e]; }
};
template <size_t dim>
UniformGravityField<dim>
get_uniform_gravity_vector(ConfigMap const &)
{
  return UniformGravityField<dim>{};
}

BETTER_ENUM(TimeIntegrator, int, HANCOCK, RK1, RK2_SSP)
struct TimeIntegratorConfig
{
  static TimeIntegrator get_time_integrator(ConfigMap const & c)
  {
    const int v = c.getInteger("refpin", "integrator", 0);
    return v == 1 ? TimeIntegrator(TimeIntegrator::RK1) : (v == 2 ? TimeIntegrator(TimeIntegrator::RK2_SSP) : TimeIntegrator(TimeIntegrator::HANCOCK));
  }
};

struct THINCParams
{
  bool   enabled = false;
  real_t beta = 1.6;
  real_t epsilon = 1e-3;
  THINCParams() = default;
  explicit THINCParams(ConfigMap const & c)
    : enabled(c.getBool("THINC", "enabled", false))
    , beta(c.getReal("THINC", "beta", 1.6))
    , epsilon(c.getReal("THINC", "epsilon", 1e-3))
  {}
};

inline real_t
get_scaling_factor(ConfigMap const & c)
{
  return c.getReal("refpin", "scaling", 1.0);
}

template <size_t dim>
KOKKOS_INLINE_FUNCTION real_t
compute_cell_length(int level, int32_t bx)
{
  return 1.0 / (static_cast<real_t>(bx) * static_cast<real_t>(1LL << level));
}

namespace core
{
BETTER_ENUM(VolFracAdvectionSourceTermType, int, ALLAIRE_KOKH, MILLER_PUCKETT)
inline VolFracAdvectionSourceTermType
get_volume_fraction_advection_source_term_type(ConfigMap const & c)
{
  return c.getInteger("refpin", "source_term", 0) == 1 ? VolFracAdvectionSourceTermType(VolFracAdvectionSourceTermType::MILLER_PUCKETT)
                                                       : VolFracAdvectionSourceTermType(VolFracAdvectionSourceTermType::ALLAIRE_KOKH);
}
} // namespace core

namespace vof
{
// Youngs normal of variable `ivar` at cell ijs of a ghosted block (unit cell
// size): (1,2,1)-weighted central differences, n = -grad / |grad|
template <typename A, size_t dim>
KOKKOS_INLINE_FUNCTION Kokkos::Array<real_t, dim>
youngs_normal_inplace(A const & q, coord_t<dim> const & c, int ivar, int32_t iOct, Kokkos::Array<real_t, dim> const &)
{
  real_t g[3] = { 0, 0, 0 };
  if constexpr (dim == 2)
  {
    auto Q = [&](int a, int b) { return q(c[IX] + a, c[IY] + b, ivar, iOct); };
    g[0] = (Q(1, -1) + 2.0 * Q(1, 0) + Q(1, 1)) - (Q(-1, -1) + 2.0 * Q(-1, 0) + Q(-1, 1));
    g[1] = (Q(-1, 1) + 2.0 * Q(0, 1) + Q(1, 1)) - (Q(-1, -1) + 2.0 * Q(0, -1) + Q(1, -1));
  }
  else
  {
    auto         Q = [&](int a, int b, int cc) { return q(c[IX] + a, c[IY] + b, c[IZ] + cc, ivar, iOct); };
    const real_t w[3] = { 1.0, 2.0, 1.0 };
    for (int cc = -1; cc <= 1; ++cc)
      for (int b = -1; b <= 1; ++b)
      {
        const real_t ww = w[b + 1] * w[cc + 1];
        g[0] += ww * (Q(1, b, cc) - Q(-1, b, cc));
        g[1] += ww * (Q(b, 1, cc) - Q(b, -1, cc));
        g[2] += ww * (Q(b, cc, 1) - Q(b, cc, -1));
      }
  }
  real_t nrm = g[0] * g[0] + g[1] * g[1];
  if constexpr (dim == 3)
    nrm += g[2] * g[2];
  nrm = std::sqrt(nrm);
  Kokkos::Array<real_t, dim> n;
  for (size_t e = 0; e < dim; ++e)
    n[e] = (nrm > 0.0) ? -g[e] / nrm : 0.0;
  return n;
}
} // namespace vof

} // namespace kalypsso
