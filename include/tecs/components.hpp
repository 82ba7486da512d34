// tecs/components.hpp -- the pair finders, integrators, centre-of-mass fixers
// and force laws a simulation config selects, as the C++20 drop-in layer
// names them.
//
// The reference's components are class templates that do the work
// themselves; here each one is a selector that keeps the reference's name,
// template signature and Settings (field names and defaults), and carries the
// enum of the CUDA implementation behind include/tecs_gpu.h:
//
//   pair_finders::NaiveAllPairs, BinnedAllPairs, NaiveGabriel, BinnedGabriel,
//     their *Symmetric variants, NaiveDelaunay    include/pair_finders/*.hpp
//   integrators::Euler, Heun                      include/integrators/{euler,heun}.hpp
//   com_fixers::NoComFixer, GlobalComFixer        include/com_fixers/com_fixers.hpp:11-45
//   forces::Spring2R, PolaritySpring              the built-in pairwise laws
//   forces::Spring, PiecewiseLinear, PiecewiseQuadratic, Cubic, Morse,
//   LennardJones, HertzContact (+Potential)       the force functions of user laws
#ifndef TECS_CXX_COMPONENTS_HPP
#define TECS_CXX_COMPONENTS_HPP

#include <string>

#include "../tecs_gpu.h"
#include "vector.hpp"

namespace tecs {

namespace pair_finders {

namespace detail {
template <int Id, bool Sym>
struct Tag {
  static constexpr int finder_id = Id;
  static constexpr bool symmetric = Sym;
  static constexpr bool binned = Id == TECS_FINDER_BINNED_ALL_PAIRS || Id == TECS_FINDER_BINNED_GABRIEL;
  static constexpr bool gabriel = Id == TECS_FINDER_NAIVE_GABRIEL || Id == TECS_FINDER_BINNED_GABRIEL;
};

// Settings of the naive finders: none (naive_all_pairs.hpp, naive_delaunay.hpp)
template <typename Scalar, int dimensions>
struct NoSettings {};

// naive_gabriel.hpp: the Gabriel coefficient only
template <typename Scalar, int dimensions>
struct GabrielSettings {
  Scalar gabriel_coefficient = Scalar(0.8);
};

// binned_all_pairs.hpp:20-25
template <typename Scalar, int dimensions>
struct BinnedSettings {
  VectorN<Scalar, dimensions> min_bounds = VectorN<Scalar, dimensions>(Scalar(-20));
  VectorN<Scalar, dimensions> max_bounds = VectorN<Scalar, dimensions>(Scalar(20));
  Scalar bin_size_scale = Scalar(1);
  int rebuild_every_n = 0;
};

// binned_gabriel.hpp:20-26
template <typename Scalar, int dimensions>
struct BinnedGabrielSettings {
  Scalar gabriel_coefficient = Scalar(0.8);
  VectorN<Scalar, dimensions> min_bounds = VectorN<Scalar, dimensions>(Scalar(-20));
  VectorN<Scalar, dimensions> max_bounds = VectorN<Scalar, dimensions>(Scalar(20));
  Scalar bin_size_scale = Scalar(1);
  int rebuild_every_n = 0;
};
}  // namespace detail

#define TECS_CXX_FINDER(NAME, ID, SYM, SETTINGS)                                 \
  template <typename PositionsView, typename Scalar, int dimensions>             \
  struct NAME : detail::Tag<ID, SYM> {                                           \
    using positions_view_type = PositionsView;                                   \
    using Settings = detail::SETTINGS<Scalar, dimensions>;                       \
  };

TECS_CXX_FINDER(NaiveAllPairs, TECS_FINDER_NAIVE_ALL_PAIRS, false, NoSettings)
TECS_CXX_FINDER(NaiveAllPairsSymmetric, TECS_FINDER_NAIVE_ALL_PAIRS, true, NoSettings)
TECS_CXX_FINDER(BinnedAllPairs, TECS_FINDER_BINNED_ALL_PAIRS, false, BinnedSettings)
TECS_CXX_FINDER(BinnedAllPairsSymmetric, TECS_FINDER_BINNED_ALL_PAIRS, true, BinnedSettings)
TECS_CXX_FINDER(NaiveGabriel, TECS_FINDER_NAIVE_GABRIEL, false, GabrielSettings)
TECS_CXX_FINDER(NaiveGabrielSymmetric, TECS_FINDER_NAIVE_GABRIEL, true, GabrielSettings)
TECS_CXX_FINDER(BinnedGabriel, TECS_FINDER_BINNED_GABRIEL, false, BinnedGabrielSettings)
TECS_CXX_FINDER(BinnedGabrielSymmetric, TECS_FINDER_BINNED_GABRIEL, true, BinnedGabrielSettings)
TECS_CXX_FINDER(NaiveDelaunay, TECS_FINDER_NAIVE_DELAUNAY, false, NoSettings)
#undef TECS_CXX_FINDER

}  // namespace pair_finders

namespace integrators {
// Any template arguments are accepted (the reference's integrators take the
// finder, fixer, force-field and view types); only the method matters here.
template <typename... Ts>
struct Euler {
  static constexpr int integrator_id = TECS_EULER;
};
template <typename... Ts>
struct Heun {
  static constexpr int integrator_id = TECS_HEUN;
};
}  // namespace integrators

namespace com_fixers {
template <typename SimulationConfig>
struct NoComFixer {
  static constexpr int com_fix = 0;
};
// subtracts sum(delta) / capacity from every delta (com_fixers.hpp:24-45)
template <typename SimulationConfig>
struct GlobalComFixer {
  static constexpr int com_fix = 1;
};
}  // namespace com_fixers

namespace forces {
// The reference's predefined force functions for pairwise laws written as
// PAIRWISE_FORCE lambdas (include/forces/predefined.hpp:60-144), with its
// operation order: a vector displacement * F / distance, zero at distance 0.
template <typename Scalar>
TECS_HD Scalar SpringPotential(const Scalar distance, const Scalar homeostatic_radius, const Scalar scale = Scalar(1)) {
  return scale * (homeostatic_radius - distance);
}
template <typename Scalar, typename Vector>
TECS_HD Vector Spring(const Vector& displacement, const Scalar distance, const Scalar homeostatic_radius,
                      const Scalar scale = Scalar(1)) {
  if (distance == Scalar(0)) return Vector{Scalar(0)};
  const Scalar F = SpringPotential(distance, homeostatic_radius, scale);
  return displacement * F / distance;
}
template <typename Scalar>
TECS_HD Scalar PiecewiseLinearPotential(const Scalar distance, const Scalar homeostatic_radius,
                                        const Scalar repulsion_scale = Scalar(1),
                                        const Scalar adhesion_scale = Scalar(1)) {
  return repulsion_scale * tecs::detail::fmax_(homeostatic_radius - distance, Scalar(0)) -
         adhesion_scale * tecs::detail::fmax_(distance - homeostatic_radius, Scalar(0));
}
template <typename Scalar, typename Vector>
TECS_HD Vector PiecewiseLinear(const Vector& displacement, const Scalar distance, const Scalar homeostatic_radius,
                               const Scalar repulsion_scale = Scalar(1), const Scalar adhesion_scale = Scalar(1)) {
  if (distance == Scalar(0)) return Vector{Scalar(0)};
  const Scalar F = PiecewiseLinearPotential(distance, homeostatic_radius, repulsion_scale, adhesion_scale);
  return displacement * F / distance;
}

// The other predefined laws (include/forces/predefined.hpp:167-491), each a
// magnitude F(d) and the vector displacement * F / distance (zero at d == 0):
//   PiecewiseQuadratic  k_rep (d - d_c)(d - d_rep) below d_c, k_adh (d - d_c)(d - d_sigma) below d_sigma, else 0
//   Cubic               mu (d_sigma - d)^2 (d_c - d) below d_sigma, else 0
//   Morse               2 F0 (exp(-2a(d - d_c)) - exp(-a(d - d_c)))
//   LennardJones        24 eps / d * (2 (sigma/d)^12 - (d_c/d)^6), 0 at d == 0
//   HertzContact        4/3 E* sqrt(R*) (R_i + R_j - d)^(3/2) below R_i + R_j, else 0,
//                       1/E* = (1 - v_i^2)/E_i + (1 - v_j^2)/E_j, R* = R_i R_j / (R_i + R_j)
// evaluated in the operation order written there.
template <typename Scalar>
TECS_HD Scalar PiecewiseQuadraticPotential(const Scalar distance, const Scalar homeostatic_radius,
                                           const Scalar repulsion_radius, const Scalar cutoff_distance,
                                           const Scalar repulsion_scale = Scalar(1),
                                           const Scalar adhesion_scale = Scalar(1)) {
  if (distance < homeostatic_radius)
    return repulsion_scale * (distance - homeostatic_radius) * (distance - repulsion_radius);
  if (distance < cutoff_distance) return adhesion_scale * (distance - homeostatic_radius) * (distance - cutoff_distance);
  return Scalar(0);
}
template <typename Scalar, typename Vector>
TECS_HD Vector PiecewiseQuadratic(const Vector& displacement, const Scalar distance, const Scalar homeostatic_radius,
                                  const Scalar repulsion_radius, const Scalar cutoff_distance,
                                  const Scalar repulsion_scale = Scalar(1), const Scalar adhesion_scale = Scalar(1)) {
  if (distance == Scalar(0)) return Vector{Scalar(0)};
  const Scalar F = PiecewiseQuadraticPotential(distance, homeostatic_radius, repulsion_radius, cutoff_distance,
                                               repulsion_scale, adhesion_scale);
  return displacement * F / distance;
}
template <typename Scalar>
TECS_HD Scalar CubicPotential(const Scalar distance, const Scalar homeostatic_radius, const Scalar cutoff_distance,
                              const Scalar scale = Scalar(1)) {
  if (distance >= cutoff_distance) return Scalar(0);
  const Scalar overlap = cutoff_distance - distance;
  const Scalar diff = homeostatic_radius - distance;
  return scale * overlap * overlap * diff;
}
template <typename Scalar, typename Vector>
TECS_HD Vector Cubic(const Vector& displacement, const Scalar distance, const Scalar homeostatic_radius,
                     const Scalar cutoff_distance, const Scalar scale = Scalar(1)) {
  if (distance == Scalar(0)) return Vector{Scalar(0)};
  const Scalar F = CubicPotential(distance, homeostatic_radius, cutoff_distance, scale);
  return displacement * F / distance;
}
template <typename Scalar>
TECS_HD Scalar MorsePotential(const Scalar distance, const Scalar equilibrium_distance, const Scalar slope = Scalar(1),
                              const Scalar scaling_factor = Scalar(1)) {
  const Scalar dx = distance - equilibrium_distance;
  const Scalar repulsion = tecs::detail::exp_(-Scalar(2) * slope * dx);
  const Scalar adhesion = tecs::detail::exp_(-slope * dx);
  return Scalar(2) * scaling_factor * (repulsion - adhesion);
}
template <typename Scalar, typename Vector>
TECS_HD Vector Morse(const Vector& displacement, const Scalar distance, const Scalar equilibrium_distance,
                     const Scalar slope = Scalar(1), const Scalar scaling_factor = Scalar(1)) {
  if (distance == Scalar(0)) return Vector{Scalar(0)};
  const Scalar F = MorsePotential(distance, equilibrium_distance, slope, scaling_factor);
  return displacement * F / distance;
}
template <typename Scalar>
TECS_HD Scalar LennardJonesPotential(const Scalar distance, const Scalar sigma, const Scalar equilibrium_distance,
                                     const Scalar epsilon = Scalar(1)) {
  if (distance == Scalar(0)) return Scalar(0);
  const Scalar s6 = tecs::detail::pow_(sigma / distance, Scalar(6));
  const Scalar s12 = s6 * s6;
  const Scalar e6 = tecs::detail::pow_(equilibrium_distance / distance, Scalar(6));
  return (Scalar(24) * epsilon / distance) * (Scalar(2) * s12 - e6);
}
template <typename Scalar, typename Vector>
TECS_HD Vector LennardJones(const Vector& displacement, const Scalar distance, const Scalar sigma,
                            const Scalar equilibrium_distance, const Scalar epsilon = Scalar(1)) {
  if (distance == Scalar(0)) return Vector{Scalar(0)};
  const Scalar F = LennardJonesPotential(distance, sigma, equilibrium_distance, epsilon);
  return displacement * F / distance;
}
template <typename Scalar>
TECS_HD Scalar HertzContactPotential(const Scalar distance, const Scalar radius_i, const Scalar radius_j,
                                     const Scalar young_modulus_i = Scalar(1), const Scalar young_modulus_j = Scalar(1),
                                     const Scalar poisson_ratio_i = Scalar(0),
                                     const Scalar poisson_ratio_j = Scalar(0)) {
  const Scalar contact = radius_i + radius_j;
  if (distance >= contact) return Scalar(0);
  // v^2 as an exact square, which a correctly rounded pow(v, 2) also gives
  const Scalar vi2 = poisson_ratio_i * poisson_ratio_i;
  const Scalar vj2 = poisson_ratio_j * poisson_ratio_j;
  const Scalar e_star = young_modulus_i * young_modulus_j /
                        ((Scalar(1) - vi2) * young_modulus_j + (Scalar(1) - vj2) * young_modulus_i);
  const Scalar r_star = (radius_i * radius_j) / contact;
  const Scalar overlap = contact - distance;
  return (Scalar(4) / Scalar(3)) * e_star * tecs::detail::sqrt_(r_star) *
         tecs::detail::pow_(overlap, Scalar(3) / Scalar(2));
}
template <typename Scalar, typename Vector>
TECS_HD Vector HertzContact(const Vector& displacement, const Scalar distance, const Scalar radius_i,
                            const Scalar radius_j, const Scalar young_modulus_i = Scalar(1),
                            const Scalar young_modulus_j = Scalar(1), const Scalar poisson_ratio_i = Scalar(0),
                            const Scalar poisson_ratio_j = Scalar(0)) {
  if (distance == Scalar(0)) return Vector{Scalar(0)};
  const Scalar F = HertzContactPotential(distance, radius_i, radius_j, young_modulus_i, young_modulus_j,
                                         poisson_ratio_i, poisson_ratio_j);
  return displacement * F / distance;
}

// Built-in pairwise force laws.  A pair at distance d < cutoff gets
// displacement * F(d) / d (zero at d == 0) with
//   F(d) = k_rep * max(r_rep - d, 0) - k_adh * max(d - r_adh, 0),
// the two-radius spring of the spheroid and ensemble workloads; with r_rep ==
// r_adh it is forces::PiecewiseLinear / forces::Spring's linear spring
// (include/forces/predefined.hpp:60-144).
struct Spring2R {
  float k_rep = 2.0f, r_rep = 0.7f, k_adh = 0.5f, r_adh = 0.8f;
  static constexpr bool is_link = false;
  static constexpr int force_id = TECS_FORCE_SPRING2R;
  static constexpr bool needs_polarity = false;
  float k_pol_value() const { return 0.0f; }
};

// Spring2R plus k_pol * (Polarity_::bending_force + bidirectional alignment)
// on a (position, polarity) config, as the epithelium examples write it
// (include/types/polarity.hpp:131-198).
struct PolaritySpring {
  float k_rep = 2.0f, r_rep = 0.7f, k_adh = 0.5f, r_adh = 0.8f, k_pol = 0.2f;
  static constexpr bool is_link = false;
  static constexpr int force_id = TECS_FORCE_POLARITY;
  static constexpr bool needs_polarity = true;
  float k_pol_value() const { return k_pol; }
};

// Pairs found, no deltas: the neighbour-counting use of main.cpp.
struct NoForce {
  float k_rep = 0.0f, r_rep = 0.0f, k_adh = 0.0f, r_adh = 0.0f;
  static constexpr bool is_link = false;
  static constexpr int force_id = TECS_FORCE_NONE;
  static constexpr bool needs_polarity = false;
  float k_pol_value() const { return 0.0f; }
};
// The link law of the reference's protrusion examples
// (examples/intercalation.cpp:65-71): along every link (a, b), cell a gets
// strength * (x_b - x_a) / |x_b - x_a| and cell b its negative, after the
// pairwise forces and in link order.
struct LinkPull {
  float strength = 0.0f;
  static constexpr bool is_link = true;
};
}  // namespace forces

// A connection between two agents (include/types/link.hpp).
struct Link {
  static constexpr unsigned int dimensions = 2;
  unsigned int a = 0;
  unsigned int b = 0;
  constexpr Link() = default;
  TECS_HD constexpr Link(unsigned int a_, unsigned int b_) : a(a_), b(b_) {}
};
static_assert(sizeof(Link) == 8, "links upload as (a, b) pairs");

namespace io {
// The reference's no-op writer (include/io/dummy.hpp).
template <typename... Ts>
struct Dummy {
  static constexpr bool writes = false;
  struct Settings {};
  Dummy(const std::string&, const Settings& = {}) {}
  template <typename... A>
  void write(A&&...) {}
  template <typename... A>
  void write_static(A&&...) {}
};
}  // namespace io

}  // namespace tecs

#endif  // TECS_CXX_COMPONENTS_HPP
