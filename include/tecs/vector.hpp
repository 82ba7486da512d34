// tecs/vector.hpp -- host-side value types of the C++20 drop-in layer.
//
// VectorN<Scalar, D> and Polarity_<Scalar> keep the reference's names,
// operators and memory layout (D, respectively 2, contiguous scalars;
// include/types/vector.hpp:34-436, include/types/polarity.hpp:28-124), so a
// View<VectorN<float, 3>> is exactly the AoS float[n][3] array the C ABI
// (tecs_gpu.h) uploads and downloads.  Compiled by nvcc their members are
// also device functions, for the user pairwise laws of tecs/pairwise.cuh.
#ifndef TECS_CXX_VECTOR_HPP
#define TECS_CXX_VECTOR_HPP

#include <cfloat>
#include <cmath>
#include <cstddef>
#include <type_traits>

#if defined(__CUDACC__)
#define TECS_HD __host__ __device__
#else
#define TECS_HD
#endif

namespace tecs {

namespace detail {
// the square root of float or double, on the host and the device
TECS_HD inline float sqrt_(float v) { return sqrtf(v); }
TECS_HD inline double sqrt_(double v) { return sqrt(v); }
TECS_HD inline float fmax_(float a, float b) { return fmaxf(a, b); }
TECS_HD inline double fmax_(double a, double b) { return fmax(a, b); }
TECS_HD inline float exp_(float v) { return expf(v); }
TECS_HD inline double exp_(double v) { return exp(v); }
TECS_HD inline float pow_(float a, float b) { return powf(a, b); }
TECS_HD inline double pow_(double a, double b) { return pow(a, b); }
// the machine epsilon (Kokkos::Experimental::epsilon_v)
template <typename Scalar>
TECS_HD constexpr Scalar epsilon_() {
  return sizeof(Scalar) == sizeof(float) ? Scalar(FLT_EPSILON) : Scalar(DBL_EPSILON);
}
}  // namespace detail

template <typename Scalar, int dimensions>
struct VectorN {
  static_assert(dimensions >= 1 && dimensions <= 4, "VectorN holds 1 to 4 components");
  using value_type = Scalar;
  static constexpr int components = dimensions;

  Scalar data_[dimensions] = {};

  constexpr VectorN() = default;
  // every component set to v (the reference's Vector(-20) bounds idiom)
  TECS_HD constexpr explicit VectorN(Scalar v) {
    for (int d = 0; d < dimensions; ++d) data_[d] = v;
  }
  template <typename... Ts>
    requires(sizeof...(Ts) == dimensions && dimensions > 1 && (std::is_arithmetic_v<Ts> && ...))
  TECS_HD constexpr VectorN(Ts... v) : data_{static_cast<Scalar>(v)...} {}

  TECS_HD static constexpr int size() { return dimensions; }
  TECS_HD constexpr Scalar& operator[](int d) { return data_[d]; }
  TECS_HD constexpr const Scalar& operator[](int d) const { return data_[d]; }
  TECS_HD constexpr Scalar& x() { return data_[0]; }
  TECS_HD constexpr const Scalar& x() const { return data_[0]; }
  TECS_HD constexpr Scalar& y() requires(dimensions >= 2) { return data_[1]; }
  TECS_HD constexpr const Scalar& y() const requires(dimensions >= 2) { return data_[1]; }
  TECS_HD constexpr Scalar& z() requires(dimensions >= 3) { return data_[2]; }
  TECS_HD constexpr const Scalar& z() const requires(dimensions >= 3) { return data_[2]; }
  TECS_HD constexpr Scalar& w() requires(dimensions >= 4) { return data_[3]; }
  TECS_HD constexpr const Scalar& w() const requires(dimensions >= 4) { return data_[3]; }

  // component-wise with a vector or a scalar
#define TECS_CXX_VEC_OP(OP)                                                                        \
  TECS_HD constexpr VectorN& operator OP##=(const VectorN& o) {                                    \
    for (int d = 0; d < dimensions; ++d) data_[d] OP## = o.data_[d];                               \
    return *this;                                                                                  \
  }                                                                                                \
  TECS_HD constexpr VectorN& operator OP##=(Scalar s) {                                            \
    for (int d = 0; d < dimensions; ++d) data_[d] OP## = s;                                        \
    return *this;                                                                                  \
  }                                                                                                \
  friend TECS_HD constexpr VectorN operator OP(VectorN a, const VectorN& b) { return a OP## = b; } \
  friend TECS_HD constexpr VectorN operator OP(VectorN a, Scalar s) { return a OP## = s; }         \
  friend TECS_HD constexpr VectorN operator OP(Scalar s, VectorN a) {                              \
    for (int d = 0; d < dimensions; ++d) a.data_[d] = s OP a.data_[d];                             \
    return a;                                                                                      \
  }
  TECS_CXX_VEC_OP(+)
  TECS_CXX_VEC_OP(-)
  TECS_CXX_VEC_OP(*)
  TECS_CXX_VEC_OP(/)
#undef TECS_CXX_VEC_OP

  friend TECS_HD constexpr VectorN operator-(VectorN a) {
    for (int d = 0; d < dimensions; ++d) a.data_[d] = -a.data_[d];
    return a;
  }
  friend TECS_HD constexpr VectorN operator+(const VectorN& a) { return a; }
  friend TECS_HD constexpr bool operator==(const VectorN& a, const VectorN& b) {
    for (int d = 0; d < dimensions; ++d)
      if (a.data_[d] != b.data_[d]) return false;
    return true;
  }

  // index-order sums, as the reference's dot / length_squared / distance_to_squared
  TECS_HD constexpr Scalar dot(const VectorN& o) const {
    Scalar r{};
    for (int d = 0; d < dimensions; ++d) r += data_[d] * o.data_[d];
    return r;
  }
  TECS_HD constexpr Scalar length_squared() const { return dot(*this); }
  TECS_HD Scalar length() const { return detail::sqrt_(length_squared()); }
  TECS_HD constexpr Scalar distance_to_squared(const VectorN& o) const {
    Scalar r{};
    for (int d = 0; d < dimensions; ++d) {
      const Scalar e = data_[d] - o.data_[d];
      r += e * e;
    }
    return r;
  }
  TECS_HD Scalar distance_to(const VectorN& o) const { return detail::sqrt_(distance_to_squared(o)); }
  TECS_HD VectorN normalized() const { return *this / length(); }
  // Gram-Schmidt against a unit vector u: (v - (v.u) u) / |v - (v.u) u|
  // (vector.hpp:385-400)
  TECS_HD VectorN orthonormal(const VectorN& u) const {
    const VectorN normal = *this - dot(u) * u;
    return normal / detail::sqrt_(normal.dot(normal));
  }
  TECS_HD constexpr VectorN cross(const VectorN& o) const requires(dimensions == 3) {
    return VectorN(data_[1] * o.data_[2] - data_[2] * o.data_[1], data_[2] * o.data_[0] - data_[0] * o.data_[2],
                   data_[0] * o.data_[1] - data_[1] * o.data_[0]);
  }
};

template <typename Scalar>
using Vector3 = VectorN<Scalar, 3>;

// Apical-basal polarity as spherical angles (theta, phi).
template <typename Scalar>
struct Polarity_ : VectorN<Scalar, 2> {
  using Base = VectorN<Scalar, 2>;

  constexpr Polarity_() = default;
  TECS_HD constexpr explicit Polarity_(Scalar v) : Base(v) {}
  // any arithmetic angles, converted (Polarity{acos(...), 2.0 * pi * u} as the reference's programs write it)
  template <typename A, typename B>
    requires(std::is_arithmetic_v<A> && std::is_arithmetic_v<B>)
  TECS_HD constexpr Polarity_(A theta, B phi) : Base(static_cast<Scalar>(theta), static_cast<Scalar>(phi)) {}
  // the direction of v (polarity.hpp:62-77), its length given or computed
  TECS_HD explicit Polarity_(const Vector3<Scalar>& v) : Polarity_(from_vector3(v)) {}
  TECS_HD Polarity_(const Vector3<Scalar>& v, Scalar length) : Polarity_(from_vector3(v, length)) {}
  TECS_HD constexpr Polarity_(const Base& b) : Base(b) {}

  TECS_HD constexpr Scalar& theta() { return this->data_[0]; }
  TECS_HD constexpr const Scalar& theta() const { return this->data_[0]; }
  TECS_HD constexpr Scalar& phi() { return this->data_[1]; }
  TECS_HD constexpr const Scalar& phi() const { return this->data_[1]; }

  // theta = acos(clamp(z / |v|, -1, 1)), phi = atan2(y, x) (polarity.hpp:62-76)
  TECS_HD static Polarity_ from_vector3(const Vector3<Scalar>& v, Scalar length) {
    return Polarity_(std::acos(std::fmin(Scalar(1), std::fmax(Scalar(-1), v[2] / length))), std::atan2(v[1], v[0]));
  }
  TECS_HD static Polarity_ from_vector3(const Vector3<Scalar>& v) { return from_vector3(v, v.length()); }
  TECS_HD static Vector3<Scalar> to_vector3(const Polarity_& p) {
    return Vector3<Scalar>(std::sin(p.theta()) * std::cos(p.phi()), std::sin(p.theta()) * std::sin(p.phi()),
                           std::cos(p.theta()));
  }
  TECS_HD Vector3<Scalar> to_vector3() const { return to_vector3(*this); }
  // cosine of the angle between the two directions (polarity.hpp:132-136)
  TECS_HD Scalar dot(const Polarity_& o) const {
    return std::sin(theta()) * std::sin(o.theta()) * std::cos(phi() - o.phi()) +
           std::cos(theta()) * std::cos(o.theta());
  }

  // The force laws of the reference's polarity programs, with its operations
  // (polarity.hpp:138-198).  The angular gradient of dot(other) that turns
  // this polarity towards other; no phi term where sin(theta) is within
  // epsilon of 0.
  TECS_HD Polarity_ unidirectional_polarization_force(const Polarity_& other) const {
    Polarity_ r(std::cos(theta()) * std::sin(other.theta()) * std::cos(phi() - other.phi()) -
                    std::sin(theta()) * std::cos(other.theta()),
                Scalar(0));
    const Scalar st = std::sin(theta());
    if (std::abs(st) > detail::epsilon_<Scalar>())
      r[1] = -std::sin(other.theta()) * std::sin(phi() - other.phi()) / st;
    return r;
  }
  // the same, scaled by the alignment dot(other)
  TECS_HD Polarity_ bidirectional_polarization_force(const Polarity_& other) const {
    return Polarity_(dot(other) * unidirectional_polarization_force(other));
  }
  struct BendingForceResult {
    Vector3<Scalar> vector;  // force on the cell
    Polarity_ polarity;      // change of its polarity
  };
  // Bending between this cell and a neighbour at displacement (this - other).
  // The squares prod^2 / distance^2 are formed in double, as the reference's
  // pow(Scalar, int) promotes them; a float's square is exact in double.
  TECS_HD BendingForceResult bending_force(const Vector3<Scalar>& displacement, const Polarity_& other_polarity,
                                           const Scalar distance) const {
    const Vector3<Scalar> this_vector = to_vector3();
    const Scalar prod_i = this_vector.dot(displacement) / distance;
    const Vector3<Scalar> other_vector = to_vector3(other_polarity);
    const Scalar prod_j = other_vector.dot(displacement) / distance;
    const double d2 = double(distance) * double(distance);
    const Scalar ci = Scalar(double(prod_i) * double(prod_i) / d2);
    const Scalar cj = Scalar(double(prod_j) * double(prod_j) / d2);
    return BendingForceResult{-prod_i / distance * this_vector + ci * displacement + -prod_j / distance * other_vector +
                                  cj * displacement,
                              Polarity_(-prod_i * unidirectional_polarization_force(Polarity_(displacement, distance)))};
  }
  // Bending towards a preferred angle between the polarity and the
  // displacement (polarity.hpp:212-229): bending_force with cos(angle) added
  // to this cell's projection and taken from the neighbour's.
  TECS_HD BendingForceResult apical_constriction_force(const Vector3<Scalar>& displacement, const Scalar distance,
                                                       const Polarity_& other_polarity,
                                                       const Scalar preferred_angle) const {
    const Vector3<Scalar> this_vector = to_vector3();
    const Scalar prod_i = this_vector.dot(displacement) / distance + std::cos(preferred_angle);
    const Vector3<Scalar> other_vector = to_vector3(other_polarity);
    const Scalar prod_j = other_vector.dot(displacement) / distance - std::cos(preferred_angle);
    const double d2 = double(distance) * double(distance);
    const Scalar ci = Scalar(double(prod_i) * double(prod_i) / d2);
    const Scalar cj = Scalar(double(prod_j) * double(prod_j) / d2);
    return BendingForceResult{-prod_i / distance * this_vector + ci * displacement + -prod_j / distance * other_vector +
                                  cj * displacement,
                              Polarity_(-prod_i * unidirectional_polarization_force(Polarity_(displacement, distance)))};
  }
  // Migration along polarities (polarity.hpp:244-274): pulled around a
  // neighbour that lies behind this polarity (alignment with the
  // displacement <= -0.15), pushed by a neighbour whose polarity points at
  // this cell (>= 0.15); each term 0.6 along the polarity plus 0.8 across it.
  TECS_HD Vector3<Scalar> migration_force(const Vector3<Scalar>& displacement, const Polarity_& other_polarity,
                                          const Scalar distance) const {
    Vector3<Scalar> result{};
    const Polarity_ displacement_polarity = from_vector3(displacement, distance);
    if (this->data_[0] != 0 || this->data_[1] != 0) {
      if (double(dot(displacement_polarity)) <= -0.15) {
        const Vector3<Scalar> this_vector = to_vector3();
        const Vector3<Scalar> this_vector_t = displacement.orthonormal(this_vector);
        result = Scalar(0.6) * this_vector + Scalar(0.8) * this_vector_t;
      }
    }
    if (other_polarity[0] > detail::epsilon_<Scalar>() || other_polarity[1] > detail::epsilon_<Scalar>()) {
      if (double(other_polarity.dot(displacement_polarity)) >= 0.15) {
        const Vector3<Scalar> other_vector = to_vector3(other_polarity);
        const Vector3<Scalar> other_vector_t = (-displacement).orthonormal(other_vector);
        result -= Scalar(0.6) * other_vector + Scalar(0.8) * other_vector_t;
      }
    }
    return result;
  }
};

static_assert(sizeof(VectorN<float, 3>) == 12 && sizeof(VectorN<float, 2>) == 8 && sizeof(Polarity_<float>) == 8,
              "host views must match the C ABI's AoS layout");

}  // namespace tecs

#endif  // TECS_CXX_VECTOR_HPP
