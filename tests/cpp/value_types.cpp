// value_types.cpp -- the known answers of the reference's value-type tests
// (tests/test_vector.cpp:7-170, tests/test_polarity.cpp:9-73) checked on the
// drop-in layer's VectorN / Polarity_, for float and double and every
// dimension the reference tests.  Exit code 0 when every check holds, 1
// otherwise (the failing checks are listed on stderr).
#include <cmath>
#include <cstdio>
#include <numbers>
#include <type_traits>

#include "tecs/vector.hpp"

using namespace tecs;

static int failures = 0;
#define CHECK(cond)                                                         \
  do {                                                                      \
    if (!(cond)) {                                                          \
      std::fprintf(stderr, "%s:%d: check failed: %s\n", __FILE__, __LINE__, #cond); \
      ++failures;                                                           \
    }                                                                       \
  } while (0)

template <typename S, int D>
void vector_checks() {
  using V = VectorN<S, D>;
  // construction and accessors
  V zero;
  V seven(S(7));
  for (int i = 0; i < D; ++i) CHECK(zero[i] == S(0) && seven[i] == S(7));
  CHECK(V::size() == D);
  CHECK(seven.x() == S(7));
  if constexpr (D > 1) CHECK(seven.y() == S(7));
  if constexpr (D > 2) CHECK(seven.z() == S(7));
  if constexpr (D > 3) CHECK(seven.w() == S(7));
  // addition: 2800 + 7
  const V sum = V(S(2800)) + V(S(7));
  for (int i = 0; i < D; ++i) CHECK(sum[i] == S(2807));
  // arithmetic with vectors, scalars and scalars on the left
  const V a(S(10)), b(S(2));
  const V vadd = a + b, vsub = a - b, vmul = a * b, vdiv = a / b;
  const V sadd = a + S(2), ssub = a - S(2), smul = a * S(2), sdiv = a / S(2);
  const V rsub = S(10) - b, rdiv = S(10) / b;
  for (int i = 0; i < D; ++i) {
    CHECK(vadd[i] == S(12) && vsub[i] == S(8) && vmul[i] == S(20) && vdiv[i] == S(5));
    CHECK(sadd[i] == S(12) && ssub[i] == S(8) && smul[i] == S(20) && sdiv[i] == S(5));
    CHECK(rsub[i] == S(8) && rdiv[i] == S(5));
  }
  // compound assignment
  V c(S(10));
  c += b;
  for (int i = 0; i < D; ++i) CHECK(c[i] == S(12));
  c -= b;
  for (int i = 0; i < D; ++i) CHECK(c[i] == S(10));
  c *= b;
  for (int i = 0; i < D; ++i) CHECK(c[i] == S(20));
  c /= b;
  for (int i = 0; i < D; ++i) CHECK(c[i] == S(10));
  c += S(2);
  for (int i = 0; i < D; ++i) CHECK(c[i] == S(12));
  c -= S(2);
  c *= S(2);
  for (int i = 0; i < D; ++i) CHECK(c[i] == S(20));
  c /= S(2);
  for (int i = 0; i < D; ++i) CHECK(c[i] == S(10));
  // dot, norms, distances
  const V two(S(2)), three(S(3));
  CHECK(two.dot(three) == S(6 * D));
  CHECK(two.length_squared() == S(4 * D));
  CHECK(two.distance_to_squared(three) == S(D));
  if constexpr (std::is_floating_point_v<S>) CHECK(std::abs(two.normalized().length_squared() - S(1)) < S(1e-4));
  // unary
  const V five(S(5));
  for (int i = 0; i < D; ++i) CHECK((-five)[i] == S(-5) && (+five)[i] == S(5));
}

template <typename S>
void cross_checks() {
  const Vector3<S> ex(S(1), S(0), S(0)), ey(S(0), S(1), S(0));
  const Vector3<S> ez = ex.cross(ey);
  CHECK(ez.x() == S(0) && ez.y() == S(0) && ez.z() == S(1));
}

template <typename S>
void polarity_checks() {
  const S pi = std::numbers::pi_v<S>, half_pi = pi / S(2);
  Polarity_<S> p0;
  CHECK(p0.theta() == S(0) && p0.phi() == S(0));
  Polarity_<S> p1(S(1.5), S(2.5));
  CHECK(p1.theta() == S(1.5) && p1.phi() == S(2.5));
  Polarity_<S> p2(S(2));
  CHECK(p2.theta() == S(2) && p2.phi() == S(2));
  // +Z and +X axes, and back
  const auto pz = Polarity_<S>::from_vector3(Vector3<S>(0, 0, 1), S(1));
  CHECK(std::abs(pz.theta()) <= S(1e-5) && std::abs(pz.phi()) <= S(1e-5));
  const auto px = Polarity_<S>::from_vector3(Vector3<S>(1, 0, 0));
  CHECK(std::abs(px.theta() - half_pi) <= S(1e-5) && std::abs(px.phi()) <= S(1e-5));
  const auto back = px.to_vector3();
  CHECK(std::abs(back.x() - S(1)) <= S(1e-4) && std::abs(back.y()) <= S(1e-4) && std::abs(back.z()) <= S(1e-4));
  // self dots 1, orthogonal dots 0
  const Polarity_<S> dx(half_pi, S(0)), dy(half_pi, half_pi), dz(S(0), S(0));
  CHECK(std::abs(dx.dot(dx) - S(1)) < S(1e-4) && std::abs(dy.dot(dy) - S(1)) < S(1e-4) &&
        std::abs(dz.dot(dz) - S(1)) < S(1e-4));
  CHECK(std::abs(dx.dot(dy)) < S(1e-4) && std::abs(dx.dot(dz)) < S(1e-4) && std::abs(dy.dot(dz)) < S(1e-4));
}

int main() {
  vector_checks<float, 1>();
  vector_checks<float, 2>();
  vector_checks<float, 3>();
  vector_checks<float, 4>();
  vector_checks<double, 2>();
  vector_checks<double, 3>();
  vector_checks<int, 3>();
  cross_checks<float>();
  cross_checks<double>();
  polarity_checks<float>();
  polarity_checks<double>();
  if (failures) std::fprintf(stderr, "%d checks failed\n", failures);
  return failures ? 1 : 0;
}
