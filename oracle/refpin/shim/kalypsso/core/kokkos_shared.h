// Minimal stand-ins for the Kokkos names used by the reference's model headers
// (host-only build of the reference's device functions; test infrastructure).
#pragma once
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <cmath>
#define KOKKOS_INLINE_FUNCTION inline
#define KOKKOS_FUNCTION
#define KOKKOS_ASSERT(x)
#define KALYPSSO_STATIC_MATH_CONSTANT(name, value) static constexpr double name = (value)
namespace Kokkos
{
template <typename T, std::size_t N>
struct Array
{
  T data_[N];
  T &       operator[](std::size_t i) { return data_[i]; }
  const T & operator[](std::size_t i) const { return data_[i]; }
  static constexpr std::size_t size() { return N; }
};
inline void
abort(const char * msg)
{
  std::fprintf(stderr, "%s\n", msg);
  std::abort();
}
} // namespace Kokkos
using std::fmax;
using std::fmin;
using std::sqrt;
using std::fabs;
