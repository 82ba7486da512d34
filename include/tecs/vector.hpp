// tecs/vector.hpp -- host-side value types of the C++20 drop-in layer.
//
// VectorN<Scalar, D> and Polarity_<Scalar> keep the reference's names and
// memory layout (D, respectively 2, contiguous scalars; include/types/vector.hpp:34-436,
// include/types/polarity.hpp:28-198), so a View<VectorN<float, 3>> is exactly
// the AoS float[n][3] array the C ABI (tecs_gpu.h) uploads and downloads.
// They are host types: the arithmetic of a step runs in the CUDA library.
#ifndef TECS_CXX_VECTOR_HPP
#define TECS_CXX_VECTOR_HPP

#include <cmath>
#include <cstddef>
#include <type_traits>

namespace tecs {

template <typename Scalar, int dimensions>
struct VectorN {
  static_assert(dimensions >= 1 && dimensions <= 3, "VectorN holds 1 to 3 components");
  using value_type = Scalar;
  static constexpr int size = dimensions;

  Scalar data_[dimensions] = {};

  constexpr VectorN() = default;
  // every component set to v (the reference's Vector(-20) bounds idiom)
  constexpr explicit VectorN(Scalar v) {
    for (int d = 0; d < dimensions; ++d) data_[d] = v;
  }
  template <typename... Ts>
    requires(sizeof...(Ts) == dimensions && dimensions > 1 && (std::is_arithmetic_v<Ts> && ...))
  constexpr VectorN(Ts... v) : data_{static_cast<Scalar>(v)...} {}

  constexpr Scalar& operator[](int d) { return data_[d]; }
  constexpr const Scalar& operator[](int d) const { return data_[d]; }
  constexpr Scalar& x() { return data_[0]; }
  constexpr const Scalar& x() const { return data_[0]; }
  constexpr Scalar& y() requires(dimensions >= 2) { return data_[1]; }
  constexpr const Scalar& y() const requires(dimensions >= 2) { return data_[1]; }
  constexpr Scalar& z() requires(dimensions >= 3) { return data_[2]; }
  constexpr const Scalar& z() const requires(dimensions >= 3) { return data_[2]; }

  constexpr VectorN& operator+=(const VectorN& o) {
    for (int d = 0; d < dimensions; ++d) data_[d] += o.data_[d];
    return *this;
  }
  constexpr VectorN& operator-=(const VectorN& o) {
    for (int d = 0; d < dimensions; ++d) data_[d] -= o.data_[d];
    return *this;
  }
  constexpr VectorN& operator*=(Scalar s) {
    for (int d = 0; d < dimensions; ++d) data_[d] *= s;
    return *this;
  }
  constexpr VectorN& operator/=(Scalar s) {
    for (int d = 0; d < dimensions; ++d) data_[d] /= s;
    return *this;
  }
  friend constexpr VectorN operator+(VectorN a, const VectorN& b) { return a += b; }
  friend constexpr VectorN operator-(VectorN a, const VectorN& b) { return a -= b; }
  friend constexpr VectorN operator-(VectorN a) {
    for (int d = 0; d < dimensions; ++d) a.data_[d] = -a.data_[d];
    return a;
  }
  friend constexpr VectorN operator*(VectorN a, Scalar s) { return a *= s; }
  friend constexpr VectorN operator*(Scalar s, VectorN a) { return a *= s; }
  friend constexpr VectorN operator/(VectorN a, Scalar s) { return a /= s; }
  friend constexpr bool operator==(const VectorN& a, const VectorN& b) {
    for (int d = 0; d < dimensions; ++d)
      if (a.data_[d] != b.data_[d]) return false;
    return true;
  }

  // index-order sums, as the reference's dot / length_squared / distance_to_squared
  constexpr Scalar dot(const VectorN& o) const {
    Scalar r{};
    for (int d = 0; d < dimensions; ++d) r += data_[d] * o.data_[d];
    return r;
  }
  constexpr Scalar length_squared() const { return dot(*this); }
  Scalar length() const { return std::sqrt(length_squared()); }
  constexpr Scalar distance_to_squared(const VectorN& o) const {
    Scalar r{};
    for (int d = 0; d < dimensions; ++d) {
      const Scalar e = data_[d] - o.data_[d];
      r += e * e;
    }
    return r;
  }
  Scalar distance_to(const VectorN& o) const { return std::sqrt(distance_to_squared(o)); }
};

// Apical-basal polarity as spherical angles (theta, phi).
template <typename Scalar>
struct Polarity_ {
  using value_type = Scalar;
  Scalar data_[2] = {};

  constexpr Polarity_() = default;
  constexpr Polarity_(Scalar theta, Scalar phi) : data_{theta, phi} {}
  // from a direction: theta = acos(z / |v|), phi = atan2(y, x) (types/polarity.hpp:74-77)
  explicit Polarity_(const VectorN<Scalar, 3>& v) {
    const Scalar len = v.length();
    data_[0] = std::acos(v[2] / len);
    data_[1] = std::atan2(v[1], v[0]);
  }

  constexpr Scalar& operator[](int d) { return data_[d]; }
  constexpr const Scalar& operator[](int d) const { return data_[d]; }
  constexpr Scalar& theta() { return data_[0]; }
  constexpr const Scalar& theta() const { return data_[0]; }
  constexpr Scalar& phi() { return data_[1]; }
  constexpr const Scalar& phi() const { return data_[1]; }

  // unit vector of the angles
  VectorN<Scalar, 3> to_vector3() const {
    return VectorN<Scalar, 3>(std::sin(data_[0]) * std::cos(data_[1]), std::sin(data_[0]) * std::sin(data_[1]),
                              std::cos(data_[0]));
  }
};

static_assert(sizeof(VectorN<float, 3>) == 12 && sizeof(VectorN<float, 2>) == 8 && sizeof(Polarity_<float>) == 8,
              "host views must match the C ABI's AoS layout");

}  // namespace tecs

#endif  // TECS_CXX_VECTOR_HPP
