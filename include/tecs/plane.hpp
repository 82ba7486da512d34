// tecs/plane.hpp -- PlaneN, the plane of the reference's wall forces
// (include/types/plane.hpp:33-99): d+1 coefficients (normal, offset)
// normalised so that the normal has unit length; signed_distance(p) =
// offset + normal . p, summed in the reference's order.
#ifndef TECS_CXX_PLANE_HPP
#define TECS_CXX_PLANE_HPP

#include <cmath>

#include "vector.hpp"

namespace tecs {

template <typename Scalar, int dimensions>
struct PlaneN {
  using Vector = VectorN<Scalar, dimensions>;
  VectorN<Scalar, dimensions + 1> coefficients;

  // the plane x_{d-1} = 0 (plane.hpp:41-44)
  TECS_HD PlaneN() { coefficients[dimensions - 1] = Scalar(1); }
  // coefficients (n_0, ..., n_{d-1}, offset), scaled by 1 / |n| (plane.hpp:52-62)
  template <typename... Scalars>
    requires(sizeof...(Scalars) == dimensions + 1)
  TECS_HD PlaneN(const Scalars... scalars) : coefficients(static_cast<Scalar>(scalars)...) {
    Scalar squared_sum = Scalar(0);
    for (int i = 0; i < dimensions; ++i) squared_sum += coefficients[i] * coefficients[i];
    const Scalar inv_norm = Scalar(1) / detail::sqrt_(squared_sum);
    for (int i = 0; i < dimensions + 1; ++i) coefficients[i] *= inv_norm;
  }

  TECS_HD Scalar signed_distance(const Vector& point) const {
    Scalar result = coefficients[dimensions];
    for (int i = 0; i < dimensions; ++i) result += coefficients[i] * point[i];
    return result;
  }
  TECS_HD Vector normal() const {
    Vector n;
    for (int i = 0; i < dimensions; ++i) n[i] = coefficients[i];
    return n;
  }
};

template <typename Scalar>
using Plane2 = PlaneN<Scalar, 2>;
template <typename Scalar>
using Plane3 = PlaneN<Scalar, 3>;

}  // namespace tecs

#endif  // TECS_CXX_PLANE_HPP
