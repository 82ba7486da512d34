// tecs/kokkos_compat.hpp -- the Kokkos names the reference's user programs
// call inside their force laws and initialisers: math functions
// (Kokkos::acos, pow, sqrt, ...), Kokkos::numbers::pi_v,
// Kokkos::Experimental::epsilon_v / finite_max_v and the atomics on device
// values (Kokkos::atomic_fetch_add(counter.data(), 1)).  They follow the
// standard library's overloads (float in, float out; integral arguments and
// mixed float/double promoted to double), on the host through <cmath> and in
// device code through CUDA's math, so such programs compile unchanged.  A
// program that includes the real Kokkos keeps Kokkos's own.
#ifndef TECS_CXX_KOKKOS_COMPAT_HPP
#define TECS_CXX_KOKKOS_COMPAT_HPP

#if !defined(KOKKOS_VERSION)

#include <cmath>
#include <limits>
#include <type_traits>

#include "vector.hpp"

namespace Kokkos {

namespace tecs_detail {
template <typename T>
using promote_t = std::conditional_t<std::is_integral_v<T>, double, T>;
template <typename A, typename B>
using promote2_t = std::conditional_t<std::is_same_v<promote_t<A>, float> && std::is_same_v<promote_t<B>, float>,
                                      float, double>;
}  // namespace tecs_detail

#define TECS_KOKKOS_UNARY(NAME)                                                          \
  TECS_HD inline float NAME(float x) { return ::NAME##f(x); }                           \
  TECS_HD inline double NAME(double x) { return ::NAME(x); }                            \
  template <typename I, std::enable_if_t<std::is_integral_v<I>, int> = 0>               \
  TECS_HD inline double NAME(I x) {                                                     \
    return ::NAME(static_cast<double>(x));                                              \
  }
TECS_KOKKOS_UNARY(acos)
TECS_KOKKOS_UNARY(asin)
TECS_KOKKOS_UNARY(atan)
TECS_KOKKOS_UNARY(cbrt)
TECS_KOKKOS_UNARY(ceil)
TECS_KOKKOS_UNARY(cos)
TECS_KOKKOS_UNARY(exp)
TECS_KOKKOS_UNARY(floor)
TECS_KOKKOS_UNARY(log)
TECS_KOKKOS_UNARY(round)
TECS_KOKKOS_UNARY(sin)
TECS_KOKKOS_UNARY(sqrt)
TECS_KOKKOS_UNARY(tan)
TECS_KOKKOS_UNARY(trunc)
#undef TECS_KOKKOS_UNARY

TECS_HD inline float abs(float x) { return ::fabsf(x); }
TECS_HD inline double abs(double x) { return ::fabs(x); }
TECS_HD inline int abs(int x) { return x < 0 ? -x : x; }

#define TECS_KOKKOS_BINARY(NAME)                                                                    \
  template <typename A, typename B, std::enable_if_t<std::is_arithmetic_v<A> && std::is_arithmetic_v<B>, int> = 0> \
  TECS_HD inline tecs_detail::promote2_t<A, B> NAME(A a, B b) {                                     \
    using R = tecs_detail::promote2_t<A, B>;                                                        \
    if constexpr (std::is_same_v<R, float>) return ::NAME##f(a, b);                                 \
    else return ::NAME(static_cast<double>(a), static_cast<double>(b));                             \
  }
TECS_KOKKOS_BINARY(atan2)
TECS_KOKKOS_BINARY(fmax)
TECS_KOKKOS_BINARY(fmin)
#undef TECS_KOKKOS_BINARY

// pow as std::pow: (float, float) in float, anything else in double.  A
// square (an integral exponent 2) is the exact product in double, which is
// what a correctly rounded pow returns for it.
template <typename A, typename B, std::enable_if_t<std::is_arithmetic_v<A> && std::is_arithmetic_v<B>, int> = 0>
TECS_HD inline tecs_detail::promote2_t<A, B> pow(A a, B b) {
  using R = tecs_detail::promote2_t<A, B>;
  if constexpr (std::is_integral_v<B>) {
    if (b == 2) return static_cast<R>(static_cast<double>(a) * static_cast<double>(a));
  }
  if constexpr (std::is_same_v<R, float>) return ::powf(a, b);
  else return ::pow(static_cast<double>(a), static_cast<double>(b));
}

template <class T>
TECS_HD constexpr const T& min(const T& a, const T& b) {
  return b < a ? b : a;
}
template <class T>
TECS_HD constexpr const T& max(const T& a, const T& b) {
  return a < b ? b : a;
}
template <class T>
TECS_HD constexpr T clamp(const T& v, const T& lo, const T& hi) {
  return v < lo ? lo : (hi < v ? hi : v);
}

namespace numbers {
template <class T>
inline constexpr T pi_v = static_cast<T>(3.141592653589793238462643383279502884L);
inline constexpr double pi = pi_v<double>;
}  // namespace numbers

namespace Experimental {
template <class T>
inline constexpr T epsilon_v = std::numeric_limits<T>::epsilon();
template <class T>
inline constexpr T finite_max_v = std::numeric_limits<T>::max();
template <class T>
inline constexpr T finite_min_v = std::numeric_limits<T>::lowest();
}  // namespace Experimental

// atomics on a device value (device code) or its host copy (host code, which
// the drop-in layer runs single-threaded)
template <class T, class U>
TECS_HD inline T atomic_fetch_add(T* p, const U& v) {
#if defined(__CUDA_ARCH__)
  return atomicAdd(p, static_cast<T>(v));
#else
  const T old = *p;
  *p += static_cast<T>(v);
  return old;
#endif
}
template <class T, class U>
TECS_HD inline void atomic_add(T* p, const U& v) {
  atomic_fetch_add(p, v);
}
template <class T, class U>
TECS_HD inline T atomic_add_fetch(T* p, const U& v) {
  return atomic_fetch_add(p, v) + static_cast<T>(v);
}
template <class T>
TECS_HD inline void atomic_increment(T* p) {
  atomic_fetch_add(p, 1);
}

}  // namespace Kokkos

#endif  // !KOKKOS_VERSION
#endif  // TECS_CXX_KOKKOS_COMPAT_HPP
