// Kokkos_Core.hpp -- minimal, single-threaded stand-in for the subset of the
// Kokkos 5 API that the TECS reference headers use, written for this project
// from Kokkos's documented semantics (not from Kokkos sources).
//
// Purpose: compile the reference's own headers unmodified on the host so that
// their results pin the oracle.  Execution model = Kokkos::Serial: every
// parallel pattern is a sequential loop in index order, teams have one
// member, reductions start from the reduction identity and accumulate in
// iteration order.  Views are reference-counted host arrays, zero-initialised
// on allocation.  Part of the test oracle only.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <limits>
#include <memory>
#include <numbers>
#include <stdexcept>
#include <string>
#include <tuple>
#include <type_traits>
#include <utility>

#define KOKKOS_INLINE_FUNCTION inline
#define KOKKOS_FORCEINLINE_FUNCTION inline
#define KOKKOS_FUNCTION
#define KOKKOS_LAMBDA [=]
#define KOKKOS_CLASS_LAMBDA [=, *this]
#define TECS_SHIM_EXPAND(...) __VA_ARGS__
#define KOKKOS_IF_ON_HOST(CODE) { TECS_SHIM_EXPAND CODE }
#define KOKKOS_IF_ON_DEVICE(CODE) {}
#define KOKKOS_VERSION 50100

namespace Kokkos {

struct HostSpace {};
struct Serial {
  using memory_space = HostSpace;
  using execution_space = Serial;
  using size_type = std::size_t;
};
using DefaultExecutionSpace = Serial;
using DefaultHostExecutionSpace = Serial;

template <class A, class B>
struct SpaceAccessibility {
  static constexpr bool accessible = true;
  static constexpr bool assignable = true;
};

namespace shim_detail {
inline bool& initialized_flag() {
  static bool f = false;
  return f;
}
}  // namespace shim_detail
inline void initialize() { shim_detail::initialized_flag() = true; }
inline void initialize(int&, char**) { initialize(); }
inline void finalize() { shim_detail::initialized_flag() = false; }
inline bool is_initialized() { return shim_detail::initialized_flag(); }
inline void fence() {}
inline void fence(const std::string&) {}

template <class T1, class T2>
struct pair {
  T1 first;
  T2 second;
};
template <class T1, class T2>
KOKKOS_INLINE_FUNCTION pair<T1, T2> make_pair(T1 a, T2 b) {
  return pair<T1, T2>{a, b};
}

struct ALL_t {};
constexpr ALL_t ALL{};

// -------------------------------------------------------------------------
// View: rank 0 (T) and rank 1 (T*)
namespace shim_detail {
template <class D>
struct rank_of {
  using value = D;
  static constexpr unsigned rank = 0;
};
template <class T>
struct rank_of<T*> {
  using value = T;
  static constexpr unsigned rank = 1;
};
template <class T>
struct rank_of<T[]> {
  using value = T;
  static constexpr unsigned rank = 1;
};
}  // namespace shim_detail

struct WithoutInitializing_t {};
constexpr WithoutInitializing_t WithoutInitializing{};

template <class DataType, class... Props>
class View {
  using R = shim_detail::rank_of<DataType>;

 public:
  using value_type = typename R::value;
  using non_const_value_type = std::remove_const_t<value_type>;
  using const_value_type = const non_const_value_type;
  using pointer_type = value_type*;
  using reference_type = value_type&;
  using data_type = DataType;
  using memory_space = HostSpace;
  using execution_space = Serial;
  using device_type = Serial;
  using size_type = std::size_t;
  using HostMirror = View<DataType, Props...>;
  using host_mirror_type = HostMirror;
  using array_layout = void;
  static constexpr unsigned rank = R::rank;
  static constexpr unsigned rank_dynamic = R::rank;

  View() = default;
  explicit View(const std::string& label, std::size_t n0 = 0) { allocate(label, rank == 0 ? 1 : n0); }
  View(const char* label, std::size_t n0 = 0) { allocate(label, rank == 0 ? 1 : n0); }
  View(value_type* ptr, std::size_t n0) : ptr_(ptr), n_(n0) {}

  template <class D2, class... P2, std::enable_if_t<std::is_convertible_v<typename View<D2, P2...>::value_type*, value_type*>, int> = 0>
  View(const View<D2, P2...>& o) : owner_(o.owner_), ptr_(o.ptr_), n_(o.n_), label_(o.label_) {}

  KOKKOS_INLINE_FUNCTION reference_type operator()(std::size_t i) const { return ptr_[i]; }
  KOKKOS_INLINE_FUNCTION reference_type operator()() const { return ptr_[0]; }
  KOKKOS_INLINE_FUNCTION reference_type operator[](std::size_t i) const { return ptr_[i]; }
  KOKKOS_INLINE_FUNCTION std::size_t extent(int d) const { return (rank >= 1 && d == 0) ? n_ : 1; }
  KOKKOS_INLINE_FUNCTION int extent_int(int d) const { return (int)extent(d); }
  KOKKOS_INLINE_FUNCTION std::size_t size() const { return rank == 0 ? 1 : n_; }
  KOKKOS_INLINE_FUNCTION std::size_t span() const { return size(); }
  KOKKOS_INLINE_FUNCTION value_type* data() const { return ptr_; }
  KOKKOS_INLINE_FUNCTION bool is_allocated() const { return ptr_ != nullptr; }
  std::string label() const { return label_; }
  int use_count() const { return (int)owner_.use_count(); }

  void allocate(const std::string& label, std::size_t n) {
    label_ = label;
    n_ = n;
    if (n == 0) {
      owner_.reset();
      ptr_ = nullptr;
      return;
    }
    std::shared_ptr<non_const_value_type[]> p(new non_const_value_type[n]());
    owner_ = p;
    ptr_ = p.get();
  }

  // public so that converting constructors and helpers can reach them
  std::shared_ptr<non_const_value_type[]> owner_;
  value_type* ptr_ = nullptr;
  std::size_t n_ = 0;
  std::string label_;
};

template <class V>
struct is_view : std::false_type {};
template <class D, class... P>
struct is_view<View<D, P...>> : std::true_type {};

template <class D, class... P>
View<D, P...> create_mirror_view(const View<D, P...>& v) {
  return v;
}
template <class Space, class D, class... P>
View<D, P...> create_mirror_view(const Space&, const View<D, P...>& v) {
  return v;
}
template <class D, class... P>
View<D, P...> create_mirror(const View<D, P...>& v) {
  View<D, P...> m(v.label(), v.extent(0));
  for (std::size_t i = 0; i < v.size(); ++i) m.data()[i] = v.data()[i];
  return m;
}

template <class D1, class... P1, class D2, class... P2>
void deep_copy(const View<D1, P1...>& dst, const View<D2, P2...>& src) {
  if (dst.data() == src.data()) return;
  const std::size_t n = std::min(dst.size(), src.size());
  for (std::size_t i = 0; i < n; ++i) dst.data()[i] = src.data()[i];
}
template <class D, class... P, class T, std::enable_if_t<!is_view<T>::value, int> = 0>
void deep_copy(const View<D, P...>& dst, const T& value) {
  for (std::size_t i = 0; i < dst.size(); ++i) dst.data()[i] = value;
}
template <class T, class D, class... P, std::enable_if_t<!is_view<T>::value, int> = 0>
void deep_copy(T& dst, const View<D, P...>& src) {
  dst = src.data()[0];
}
template <class Exec, class A, class B>
void deep_copy(const Exec&, A&& dst, B&& src) {
  deep_copy(std::forward<A>(dst), std::forward<B>(src));
}

template <class D, class... P>
void resize(View<D, P...>& v, std::size_t n) {
  View<D, P...> nv(v.label(), n);
  const std::size_t m = std::min(n, v.size());
  for (std::size_t i = 0; i < m; ++i) nv.data()[i] = v.data()[i];
  v = nv;
}
template <class D, class... P>
void realloc(View<D, P...>& v, std::size_t n) {
  v = View<D, P...>(v.label(), n);
}

template <class D, class... P, class I>
View<D, P...> subview(const View<D, P...>& v, const pair<I, I>& r) {
  View<D, P...> s;
  s.owner_ = v.owner_;
  s.ptr_ = v.ptr_ + r.first;
  s.n_ = (std::size_t)(r.second - r.first);
  s.label_ = v.label_;
  return s;
}
template <class D, class... P, class I1, class I2>
View<D, P...> subview(const View<D, P...>& v, const std::pair<I1, I2>& r) {
  return subview(v, pair<std::size_t, std::size_t>{(std::size_t)r.first, (std::size_t)r.second});
}

// -------------------------------------------------------------------------
// atomics (single-threaded: plain read-modify-write)
template <class T, class U>
KOKKOS_INLINE_FUNCTION void atomic_add(T* p, const U& v) {
  *p += v;
}
template <class T, class U>
KOKKOS_INLINE_FUNCTION T atomic_fetch_add(T* p, const U& v) {
  T old = *p;
  *p += v;
  return old;
}
template <class T, class U>
KOKKOS_INLINE_FUNCTION T atomic_add_fetch(T* p, const U& v) {
  *p += v;
  return *p;
}
template <class T, class U>
KOKKOS_INLINE_FUNCTION void atomic_sub(T* p, const U& v) {
  *p -= v;
}
template <class T>
KOKKOS_INLINE_FUNCTION void atomic_increment(T* p) {
  ++*p;
}

// -------------------------------------------------------------------------
// math
using std::abs;
using std::acos;
using std::asin;
using std::atan;
using std::atan2;
using std::cbrt;
using std::ceil;
using std::cos;
using std::exp;
using std::floor;
using std::fmax;
using std::fmin;
using std::log;
using std::pow;
using std::round;
using std::sin;
using std::sqrt;
using std::tan;
using std::trunc;
template <class T>
KOKKOS_INLINE_FUNCTION constexpr const T& min(const T& a, const T& b) {
  return b < a ? b : a;
}
template <class T>
KOKKOS_INLINE_FUNCTION constexpr const T& max(const T& a, const T& b) {
  return a < b ? b : a;
}
template <class T>
KOKKOS_INLINE_FUNCTION constexpr T clamp(const T& v, const T& lo, const T& hi) {
  return v < lo ? lo : (hi < v ? hi : v);
}
namespace numbers {
template <class T>
inline constexpr T pi_v = std::numbers::pi_v<T>;
inline constexpr double pi = std::numbers::pi;
}  // namespace numbers
namespace Experimental {
template <class T>
inline constexpr T epsilon_v = std::numeric_limits<T>::epsilon();
template <class T>
inline constexpr T finite_max_v = std::numeric_limits<T>::max();
template <class T>
inline constexpr T finite_min_v = std::numeric_limits<T>::lowest();
template <class T>
inline constexpr T infinity_v = std::numeric_limits<T>::infinity();
}  // namespace Experimental

// -------------------------------------------------------------------------
// reductions
template <class T>
struct reduction_identity {
  KOKKOS_FORCEINLINE_FUNCTION static constexpr T sum() { return T(); }
  KOKKOS_FORCEINLINE_FUNCTION static constexpr T prod() { return static_cast<T>(1); }
  KOKKOS_FORCEINLINE_FUNCTION static constexpr T min() { return std::numeric_limits<T>::max(); }
  KOKKOS_FORCEINLINE_FUNCTION static constexpr T max() { return std::numeric_limits<T>::lowest(); }
};

template <class T, class Space = HostSpace>
struct Sum {
  using reducer = Sum;
  using value_type = std::remove_cv_t<T>;
  value_type* ref;
  explicit Sum(value_type& r) : ref(&r) {}
  void init(value_type& v) const { v = reduction_identity<value_type>::sum(); }
  void join(value_type& a, const value_type& b) const { a += b; }
  value_type& reference() const { return *ref; }
};
template <class T, class Space = HostSpace>
struct Min {
  using reducer = Min;
  using value_type = std::remove_cv_t<T>;
  value_type* ref;
  explicit Min(value_type& r) : ref(&r) {}
  void init(value_type& v) const { v = reduction_identity<value_type>::min(); }
  void join(value_type& a, const value_type& b) const { if (b < a) a = b; }
  value_type& reference() const { return *ref; }
};
template <class T, class Space = HostSpace>
struct Max {
  using reducer = Max;
  using value_type = std::remove_cv_t<T>;
  value_type* ref;
  explicit Max(value_type& r) : ref(&r) {}
  void init(value_type& v) const { v = reduction_identity<value_type>::max(); }
  void join(value_type& a, const value_type& b) const { if (a < b) a = b; }
  value_type& reference() const { return *ref; }
};

template <class R, class = void>
struct is_reducer : std::false_type {};
template <class R>
struct is_reducer<R, std::void_t<typename R::reducer>> : std::true_type {};

// -------------------------------------------------------------------------
// policies
struct AUTO_t {
  constexpr const AUTO_t& operator()() const { return *this; }
};
inline constexpr AUTO_t AUTO{};

template <class... Args>
struct RangePolicy {
  std::int64_t b = 0, e = 0;
  RangePolicy(std::int64_t begin, std::int64_t end) : b(begin), e(end) {}
  template <class Exec>
  RangePolicy(const Exec&, std::int64_t begin, std::int64_t end) : b(begin), e(end) {}
};
template <class T>
struct IndexType {};
template <unsigned N>
struct Rank {
  static constexpr unsigned rank = N;
};
template <class R, class... Args>
struct MDRangePolicy {
  static constexpr unsigned N = R::rank;
  std::int64_t lo[N], hi[N];
  template <class A, class B>
  MDRangePolicy(std::initializer_list<A> l, std::initializer_list<B> h) {
    unsigned k = 0;
    for (auto v : l) lo[k++] = (std::int64_t)v;
    k = 0;
    for (auto v : h) hi[k++] = (std::int64_t)v;
  }
};

class TeamMember {
 public:
  explicit TeamMember(int league_rank, int league_size) : lr_(league_rank), ls_(league_size) {}
  KOKKOS_INLINE_FUNCTION int league_rank() const { return lr_; }
  KOKKOS_INLINE_FUNCTION int league_size() const { return ls_; }
  KOKKOS_INLINE_FUNCTION int team_rank() const { return 0; }
  KOKKOS_INLINE_FUNCTION int team_size() const { return 1; }
  KOKKOS_INLINE_FUNCTION void team_barrier() const {}

 private:
  int lr_, ls_;
};

template <class... Args>
struct TeamPolicy {
  using member_type = TeamMember;
  int league = 0;
  TeamPolicy(int league_size, int) : league(league_size) {}
  TeamPolicy(int league_size, AUTO_t) : league(league_size) {}
  template <class Exec>
  TeamPolicy(const Exec&, int league_size, AUTO_t) : league(league_size) {}
};

template <class I>
struct NestedRange {
  I b, e;
};
template <class I>
KOKKOS_INLINE_FUNCTION NestedRange<I> TeamThreadRange(const TeamMember&, I n) {
  return {I(0), n};
}
template <class I1, class I2>
KOKKOS_INLINE_FUNCTION NestedRange<std::common_type_t<I1, I2>> TeamThreadRange(const TeamMember&, I1 b, I2 e) {
  return {std::common_type_t<I1, I2>(b), std::common_type_t<I1, I2>(e)};
}
template <class I>
KOKKOS_INLINE_FUNCTION NestedRange<I> ThreadVectorRange(const TeamMember&, I n) {
  return {I(0), n};
}
template <class I1, class I2>
KOKKOS_INLINE_FUNCTION NestedRange<std::common_type_t<I1, I2>> ThreadVectorRange(const TeamMember&, I1 b, I2 e) {
  return {std::common_type_t<I1, I2>(b), std::common_type_t<I1, I2>(e)};
}
template <class I>
KOKKOS_INLINE_FUNCTION NestedRange<I> TeamVectorRange(const TeamMember& m, I n) {
  return {I(0), n};
}

struct PerTeamTag {
  const TeamMember& m;
};
struct PerThreadTag {
  const TeamMember& m;
};
inline PerTeamTag PerTeam(const TeamMember& m) { return {m}; }
inline PerThreadTag PerThread(const TeamMember& m) { return {m}; }
template <class F>
KOKKOS_INLINE_FUNCTION void single(const PerTeamTag&, const F& f) {
  f();
}
template <class F>
KOKKOS_INLINE_FUNCTION void single(const PerThreadTag&, const F& f) {
  f();
}

// -------------------------------------------------------------------------
// parallel_for
template <class F>
void parallel_for(std::size_t n, const F& f) {
  for (std::size_t i = 0; i < n; ++i) f(i);
}
template <class... A, class F>
void parallel_for(const RangePolicy<A...>& p, const F& f) {
  for (std::int64_t i = p.b; i < p.e; ++i) f(i);
}
template <class... A, class F>
void parallel_for(const TeamPolicy<A...>& p, const F& f) {
  for (int l = 0; l < p.league; ++l) f(TeamMember(l, p.league));
}
template <class R, class... A, class F>
void parallel_for(const MDRangePolicy<R, A...>& p, const F& f) {
  if constexpr (R::rank == 2) {
    for (auto i = p.lo[0]; i < p.hi[0]; ++i)
      for (auto j = p.lo[1]; j < p.hi[1]; ++j) f(i, j);
  } else if constexpr (R::rank == 3) {
    for (auto i = p.lo[0]; i < p.hi[0]; ++i)
      for (auto j = p.lo[1]; j < p.hi[1]; ++j)
        for (auto k = p.lo[2]; k < p.hi[2]; ++k) f(i, j, k);
  }
}
template <class I, class F>
KOKKOS_INLINE_FUNCTION void parallel_for(const NestedRange<I>& r, const F& f) {
  for (I i = r.b; i < r.e; ++i) f(i);
}
template <class P, class F>
void parallel_for(const std::string&, const P& p, const F& f) {
  if constexpr (std::is_integral_v<P>) parallel_for((std::size_t)p, f);
  else parallel_for(p, f);
}
template <class P, class F>
void parallel_for(const char* label, const P& p, const F& f) {
  parallel_for(std::string(label), p, f);
}

// -------------------------------------------------------------------------
// parallel_reduce: accumulators start from the identity (reducers) or from a
// value-initialised object (plain results), the functor runs in index order
namespace shim_detail {
template <class R>
struct acc_for {
  using type = std::conditional_t<is_reducer<std::decay_t<R>>::value, typename std::decay_t<R>::value_type,
                                  std::decay_t<R>>;
};
template <class R>
void init_acc(const R& r, typename acc_for<R>::type& v) {
  if constexpr (is_reducer<std::decay_t<R>>::value) r.init(v);
  else v = typename acc_for<R>::type();
}
template <class R>
void store(R&& r, const typename acc_for<R>::type& v) {
  if constexpr (is_reducer<std::decay_t<R>>::value) r.reference() = v;
  else r = v;
}
template <class Loop, class F, class... Rs>
void reduce_impl(const Loop& loop, const F& f, Rs&&... rs) {
  std::tuple<typename acc_for<Rs>::type...> acc;
  std::apply([&](auto&... a) { (init_acc(rs, a), ...); }, acc);
  loop([&](auto... idx) { std::apply([&](auto&... a) { f(idx..., a...); }, acc); });
  std::apply([&](auto&... a) { (store(std::forward<Rs>(rs), a), ...); }, acc);
}
}  // namespace shim_detail

template <class F, class... Rs>
void parallel_reduce(std::size_t n, const F& f, Rs&&... rs) {
  shim_detail::reduce_impl([&](auto&& body) { for (std::size_t i = 0; i < n; ++i) body(i); }, f,
                           std::forward<Rs>(rs)...);
}
template <class... A, class F, class... Rs>
void parallel_reduce(const RangePolicy<A...>& p, const F& f, Rs&&... rs) {
  shim_detail::reduce_impl([&](auto&& body) { for (std::int64_t i = p.b; i < p.e; ++i) body(i); }, f,
                           std::forward<Rs>(rs)...);
}
template <class I, class F, class... Rs>
KOKKOS_INLINE_FUNCTION void parallel_reduce(const NestedRange<I>& r, const F& f, Rs&&... rs) {
  shim_detail::reduce_impl([&](auto&& body) { for (I i = r.b; i < r.e; ++i) body(i); }, f, std::forward<Rs>(rs)...);
}
template <class P, class F, class... Rs>
void parallel_reduce(const std::string&, const P& p, const F& f, Rs&&... rs) {
  if constexpr (std::is_integral_v<P>) parallel_reduce((std::size_t)p, f, std::forward<Rs>(rs)...);
  else parallel_reduce(p, f, std::forward<Rs>(rs)...);
}
template <class P, class F, class... Rs>
void parallel_reduce(const char* label, const P& p, const F& f, Rs&&... rs) {
  parallel_reduce(std::string(label), p, f, std::forward<Rs>(rs)...);
}

}  // namespace Kokkos
