// tecs/grid.hpp -- the standalone bin grid of the C++20 drop-in layer:
// tecs::acceleration::Grid with the reference's nearest / random-neighbour
// queries (include/utils/grid.hpp:29-638) and tecs::utils::get_bounds
// (utils/functions.hpp:205-220).  The drop-in layer runs update functions on
// the host, so this grid lives on the host: it bins the view's host array.
// Bins are cubes of bin_size from min_bounds, ceil((max - min) / bin_size)
// per axis, x fastest; a point's bin truncates and clamps into the grid;
// each bin lists its points in ascending index (Kokkos BinSort's binning
// order); the queries visit the (2r+1)^d bins around the point in the
// reference's task order (x fastest) and draw from the caller's generator as
// the reference does.  The GPU form of the same grid is tecs_grid_* of the
// C ABI.
#ifndef TECS_CXX_GRID_HPP
#define TECS_CXX_GRID_HPP

#include <cmath>
#include <limits>
#include <string>
#include <vector>

#include "view.hpp"

namespace tecs {
namespace utils {

template <typename Vector>
struct Bounds {
  Vector min;
  Vector max;
};

// per-dimension minimum and maximum over the view's extent (its capacity, as
// the reference's reduction runs over points_view.extent(0))
template <typename Vector, typename PointsView = View<Vector>>
Bounds<Vector> get_bounds(const PointsView& points_view) {
  using Scalar = typename Vector::value_type;
  Bounds<Vector> b{Vector(std::numeric_limits<Scalar>::max()), Vector(std::numeric_limits<Scalar>::lowest())};
  const std::size_t n = points_view.extent(0);
  for (std::size_t i = 0; i < n; ++i) {
    const Vector p = points_view.access(static_cast<int>(i));
    for (int d = 0; d < Vector::size(); ++d) {
      if (p[d] < b.min[d]) b.min[d] = p[d];
      if (p[d] > b.max[d]) b.max[d] = p[d];
    }
  }
  return b;
}

}  // namespace utils

namespace acceleration {

template <typename Vector, typename ViewType = View<Vector>>
class Grid {
 public:
  using Scalar = typename Vector::value_type;
  static constexpr int dimensions = Vector::size();
  using VectorI = VectorN<int, dimensions>;

  // the edge for about agents_per_bin points per bin (grid.hpp:43-58)
  static Scalar get_bin_size(const Vector& min_bounds_, const Vector& max_bounds_, unsigned agent_count_,
                             unsigned agents_per_bin_ = 1) {
    if (agent_count_ == 0) return Scalar(1);
    Scalar volume = 1;
    for (int d = 0; d < dimensions; ++d) volume *= (max_bounds_[d] - min_bounds_[d]);
    return static_cast<Scalar>(
        std::pow((static_cast<Scalar>(agents_per_bin_) * volume) / static_cast<Scalar>(agent_count_), 1.0 / dimensions));
  }

  Grid(const ViewType& data_view_, unsigned agent_count_, const Vector& min_bounds_, const Vector& max_bounds_,
       Scalar bin_size_)
      : data_view(data_view_), agent_count(agent_count_), min_bounds(min_bounds_), max_bounds(max_bounds_),
        bin_size(bin_size_) {
    for (int d = 0; d < dimensions; ++d) {
      // a grid of no extent (bin size 0) has no bins: its queries find nothing
      const double e = std::ceil(double(max_bounds[d] - min_bounds[d]) / double(bin_size));
      bin_extents[d] = std::isfinite(e) && e > 0 ? static_cast<int>(e) : 0;
    }
    bin_count = 1;
    for (int d = 0; d < dimensions; ++d) bin_count *= bin_extents[d];
  }
  Grid(const ViewType& data_view_, unsigned agent_count_, const utils::Bounds<Vector>& bounds,
       unsigned agents_per_bin_ = 1)
      : Grid(data_view_, agent_count_, bounds.min, bounds.max,
             get_bin_size(bounds.min, bounds.max, agent_count_, agents_per_bin_)) {}
  Grid(const ViewType& data_view_, unsigned agent_count_, unsigned agents_per_bin_ = 1)
      : Grid(data_view_, agent_count_, utils::get_bounds<Vector, ViewType>(data_view_), agents_per_bin_) {}
  explicit Grid(const ViewType& data_view_, unsigned agents_per_bin_ = 1)
      : Grid(data_view_, static_cast<unsigned>(data_view_.extent(0)), agents_per_bin_) {}
  Grid() = default;

  ViewType data_view;
  unsigned agent_count = 0;
  Vector min_bounds{};
  Vector max_bounds{};
  Scalar bin_size = 0;
  VectorI bin_extents{};
  int bin_count = 0;

  Vector get_min_bounds() const { return min_bounds; }
  Vector get_max_bounds() const { return max_bounds; }
  Scalar get_bin_size() const { return bin_size; }
  VectorI get_bin_extents() const { return bin_extents; }
  int get_bin_count() const { return bin_count; }
  const std::vector<unsigned>& get_permute_vector() const { return perm_; }
  const std::vector<unsigned>& get_bin_offsets() const { return offsets_; }
  int get_agent_count_for_bin(int b) const { return static_cast<int>(offsets_[b + 1] - offsets_[b]); }

  // the point's bin: truncation, clamped into the grid (grid.hpp:222-230)
  VectorI calc_bin_coords_from_point(const Vector& point) const {
    VectorI r;
    for (int d = 0; d < dimensions; ++d) {
      const int v = static_cast<int>((point[d] - min_bounds[d]) / bin_size);
      r[d] = std::max(0, std::min(v, bin_extents[d] - 1));
    }
    return r;
  }
  int flatten_bin_index(const VectorI& c) const {
    int b = 0, stride = 1;
    for (int d = 0; d < dimensions; ++d) {
      b += c[d] * stride;
      stride *= bin_extents[d];
    }
    return b;
  }
  int calc_bin_index_from_point(const Vector& point) const { return flatten_bin_index(calc_bin_coords_from_point(point)); }

  // bin every active point, then list each bin's points in ascending index
  // (grid.hpp:389-401)
  void rebuild() {
    offsets_.assign(std::size_t(bin_count) + 1, 0u);
    perm_.assign(agent_count, 0u);
    if (bin_count == 0) return;
    std::vector<int> key(agent_count);
    for (unsigned i = 0; i < agent_count; ++i) {
      key[i] = calc_bin_index_from_point(data_view.access(static_cast<int>(i)));
      ++offsets_[std::size_t(key[i]) + 1];
    }
    for (int b = 0; b < bin_count; ++b) offsets_[std::size_t(b) + 1] += offsets_[b];
    std::vector<unsigned> fill(offsets_.begin(), offsets_.end() - 1);
    for (unsigned i = 0; i < agent_count; ++i) perm_[fill[key[i]]++] = i;
  }

  // nearest point in the (2r+1)^d bins around the point, the first of equals
  // (grid.hpp:413-441)
  int get_nearest_point_index(const Vector& point, int search_radius = 1) const {
    int best = -1;
    Scalar best_d2 = std::numeric_limits<Scalar>::max();
    each_bin(point, search_radius, [&](int b) {
      for (unsigned k = offsets_[b]; k < offsets_[b + 1]; ++k) {
        const int j = static_cast<int>(perm_[k]);
        const Scalar d2 = point.distance_to_squared(data_view.access(j));
        if (d2 < best_d2) {
          best = j;
          best_d2 = d2;
        }
      }
    });
    return best;
  }

  // a point of the (2r+1)^d bins, uniformly: the rng.rand(0, total)-th in
  // task order (grid.hpp:453-492; the draw happens even when there is none)
  template <typename Random>
  int get_random_point_index_in_neighbourhood_bins(const Vector& point, int radius_bins, Random& rng) const {
    int total = 0;
    each_bin(point, radius_bins, [&](int b) { total += get_agent_count_for_bin(b); });
    const int target = rng.rand(0, total);
    int seen = 0, found = -1;
    each_bin(point, radius_bins, [&](int b) {
      const int count = get_agent_count_for_bin(b);
      if (found >= 0 || count == 0) return;
      if (target < seen + count) found = static_cast<int>(perm_[offsets_[b] + unsigned(target - seen)]);
      seen += count;
    });
    return found;
  }

  // a point within the radius, uniformly: the rng.urand(total)-th in task
  // order, -1 (and no draw) when there is none (grid.hpp:505-556)
  template <typename Random>
  int get_random_point_index_in_neighbourhood(const Vector& point, Scalar search_radius, Random& rng) const {
    return random_within(point, search_radius, rng, [](int) { return true; });
  }
  // the same among the points the filter accepts (grid.hpp:579-637)
  template <typename Random, typename FilterFunc>
  int get_random_point_index_in_neighbourhood(const Vector& point, Scalar search_radius, Random& rng,
                                              const FilterFunc& filter) const {
    return random_within(point, search_radius, rng, filter);
  }

 private:
  // f(bin) for every bin of the (2r+1)^d block around the point that lies in
  // the grid, in task order: x fastest (grid.hpp:264-373)
  template <typename F>
  void each_bin(const Vector& point, int r, F&& f) const {
    if (bin_count == 0) return;
    const VectorI c = calc_bin_coords_from_point(point);
    const int side = 2 * r + 1;
    int tasks = 1;
    for (int d = 0; d < dimensions; ++d) tasks *= side;
    for (int t = 0; t < tasks; ++t) {
      VectorI nb;
      int rest = t;
      bool outside = false;
      for (int d = 0; d < dimensions; ++d) {
        nb[d] = c[d] + (rest % side) - r;
        rest /= side;
        outside = outside || nb[d] < 0 || nb[d] >= bin_extents[d];
      }
      if (!outside) f(flatten_bin_index(nb));
    }
  }
  template <typename Random, typename FilterFunc>
  int random_within(const Vector& point, Scalar search_radius, Random& rng, const FilterFunc& filter) const {
    const int r = std::max(1, static_cast<int>(std::ceil(search_radius / bin_size)));
    const Scalar r2 = search_radius * search_radius;
    int total = 0;
    each_bin(point, r, [&](int b) {
      for (unsigned k = offsets_[b]; k < offsets_[b + 1]; ++k) {
        const int j = static_cast<int>(perm_[k]);
        if (point.distance_to_squared(data_view.access(j)) <= r2 && filter(j)) ++total;
      }
    });
    if (total == 0) return -1;
    const int target = static_cast<int>(rng.urand(static_cast<unsigned>(total)));
    int seen = 0, found = -1;
    each_bin(point, r, [&](int b) {
      for (unsigned k = offsets_[b]; k < offsets_[b + 1] && found < 0; ++k) {
        const int j = static_cast<int>(perm_[k]);
        if (point.distance_to_squared(data_view.access(j)) <= r2 && filter(j)) {
          if (seen == target) found = j;
          ++seen;
        }
      }
    });
    return found;
  }

  std::vector<unsigned> offsets_;
  std::vector<unsigned> perm_;
};

}  // namespace acceleration
}  // namespace tecs

#endif  // TECS_CXX_GRID_HPP
