// Minimal stand-ins for the Kokkos names used by the reference's model and
// scheme code (host-only, serial build of the reference's device functions;
// test infrastructure).  Views share their storage on copy, as Kokkos views
// do; parallel loops run in index order on the calling thread.
#pragma once
#include <cfloat>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <memory>
#include <string>
#include <type_traits>
#include <vector>
#define KOKKOS_INLINE_FUNCTION inline
#define KOKKOS_FUNCTION
#define KOKKOS_ASSERT(x)
#define KALYPSSO_STATIC_MATH_CONSTANT(name, value) static constexpr double name = (value)
namespace Kokkos
{
template <typename T, std::size_t N>
struct Array
{
  T                            data_[N];
  constexpr T &                operator[](std::size_t i) { return data_[i]; }
  constexpr const T &          operator[](std::size_t i) const { return data_[i]; }
  static constexpr std::size_t size() { return N; }
  T *                          data() { return data_; }
  const T *                    data() const { return data_; }
  T *                          begin() { return data_; }
  T *                          end() { return data_ + N; }
  const T *                    begin() const { return data_; }
  const T *                    end() const { return data_ + N; }
};
template <typename T, std::size_t N>
constexpr bool
operator==(Array<T, N> const & a, Array<T, N> const & b)
{
  for (std::size_t i = 0; i < N; ++i)
    if (!(a[i] == b[i]))
      return false;
  return true;
}
inline void
abort(const char * msg)
{
  std::fprintf(stderr, "%s\n", msg);
  std::abort();
}
inline void
fence()
{}
inline void
fence(const char *)
{}

struct Serial
{};
struct HostSpace
{};

template <typename... P>
struct RangePolicy
{
  std::int64_t b, e;
  RangePolicy(std::int64_t b_, std::int64_t e_)
    : b(b_)
    , e(e_)
  {}
};
namespace shim_detail
{
template <typename... P>
struct tag_of
{
  using type = void;
};
template <typename E, typename T>
struct tag_of<E, T>
{
  using type = T;
};
} // namespace shim_detail
template <typename... P, typename F>
void
parallel_for(const std::string &, RangePolicy<P...> const & r, F const & f)
{
  using Tag = typename shim_detail::tag_of<P...>::type;
  for (std::int64_t i = r.b; i < r.e; ++i)
  {
    if constexpr (std::is_void_v<Tag>)
      f(i);
    else
      f(Tag{}, static_cast<std::int32_t>(i));
  }
}
template <typename T>
struct Max
{
  T & ref;
  explicit Max(T & r)
    : ref(r)
  {}
};
template <typename... P, typename F, typename T>
void
parallel_reduce(const std::string &, RangePolicy<P...> const & r, F const & f, Max<T> red)
{
  T v = -DBL_MAX;
  for (std::int64_t i = r.b; i < r.e; ++i)
    f(static_cast<std::int32_t>(i), v);
  red.ref = v;
}

// one-dimensional view with shared storage
template <typename T, typename... P>
class View;
template <typename T, typename... P>
class View<T *, P...>
{
public:
  using value_type = T;
  std::shared_ptr<std::vector<T>> s;
  View() = default;
  View(const std::string &, std::size_t n)
    : s(std::make_shared<std::vector<T>>(n))
  {}
  T &         operator()(std::size_t i) const { return (*s)[i]; }
  std::size_t extent(int) const { return s ? s->size() : 0; }
  std::size_t size() const { return extent(0); }
  T *         data() const { return s ? s->data() : nullptr; }
};
template <typename V>
V
create_mirror_view(V const & v)
{
  return v;
}
template <typename A, typename B>
void
deep_copy(A const & a, B const & b)
{
  if (a.s != b.s)
    *a.s = *b.s;
}

template <typename T>
struct reduction_identity
{
  static constexpr T max() { return -DBL_MAX; }
};
template <typename T>
KOKKOS_INLINE_FUNCTION void
atomic_max(T * p, T v)
{
  if (v > *p)
    *p = v;
}

template <typename T, std::size_t N>
constexpr T
dim_prod(Array<T, N> const & a)
{
  T p = 1;
  for (std::size_t i = 0; i < N; ++i)
    p *= a[i];
  return p;
}
} // namespace Kokkos
using std::fabs;
using std::fmax;
using std::fmin;
using std::sqrt;

namespace kalypsso
{
struct DefaultDevice
{
  using execution_space = Kokkos::Serial;
  using memory_space = Kokkos::HostSpace;
};
using HostDevice = DefaultDevice;
} // namespace kalypsso
