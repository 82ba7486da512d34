// tecs/simulation.hpp -- Simulation<Config> of the C++20 drop-in layer.
//
// Keeps the reference's Simulation interface for the per-timestep path
// (include/simulation.hpp:76-153 constructors and Settings, :231-332 views,
// counts and links, :338-546 initialisers and init, :548-556 take_step,
// :600-667 write) and runs every step in the CUDA library through the C ABI
// of include/tecs_gpu.h.  The library holds the state between steps; a
// field's View (tecs/view.hpp) mirrors it on the host and on the device.
// The views are refreshed from the library when they are read or synchronised
// after steps, and their changes -- written on the host, or by device code --
// go back to the library before the next step: the DualView protocol of
// include/types/view.hpp:47-266, with the library as the view's source.
//
// Initialisers and init functions (INIT_FUNC, UPDATE_FUNC through init) run
// on the host in cell order from one generator state, seeded from
// Settings::seed -- the order in which the reference's Serial backend hands
// its pool state from cell to cell -- so a program's initial state is
// reproducible; the steps run on the GPU.
//
// Errors: every C-ABI failure throws tecs::Error with tecs_last_error().
#ifndef TECS_CXX_SIMULATION_HPP
#define TECS_CXX_SIMULATION_HPP

#include <cmath>
#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "../tecs_gpu.h"
#include "components.hpp"
#include "config.hpp"
#include "hdf5_writer.hpp"
#include "kokkos_compat.hpp"
#include "random.hpp"
#include "vector.hpp"
#include "view.hpp"

namespace tecs {

struct Error : std::runtime_error {
  using std::runtime_error::runtime_error;
};

inline void check(int rc) {
  if (rc != 0) throw Error(tecs_last_error());
}

namespace detail {
// the tags of user laws: PAIRWISE_FORCE / GENERIC_FORCE lambdas and their _OP functors
// (include/utils/utils.hpp:181-276), defined with tecs/pairwise.cuh
struct PairwiseForceTag {};
struct GenericForceTag {};
struct UpdateFuncTag {};
struct LinkForceTag {};

// PAIRWISE_FORCE's, GENERIC_FORCE's and UPDATE_FUNC's values: the lambda with
// its tag (utils.hpp:181-184)
template <typename L, typename Tag>
struct TaggedForce {
  using tag = Tag;
  L f;
  template <typename... A>
  TECS_HD void operator()(A&&... a) const {
    f(static_cast<A&&>(a)...);
  }
};
template <typename Tag>
struct TaggedForceMaker {
  template <typename L>
  TaggedForce<L, Tag> operator|(L f) const {
    return TaggedForce<L, Tag>{f};
  }
};
inline constexpr TaggedForceMaker<PairwiseForceTag> pairwise_force{};
inline constexpr TaggedForceMaker<GenericForceTag> generic_force{};
inline constexpr TaggedForceMaker<UpdateFuncTag> update_func{};
inline constexpr TaggedForceMaker<LinkForceTag> link_force{};
template <typename F, typename Tag>
concept TaggedLaw = requires { typename F::tag; } && std::is_same_v<typename F::tag, Tag>;
template <typename F>
concept UserPairLaw = TaggedLaw<F, PairwiseForceTag>;
template <typename F>
concept UserGenericLaw = TaggedLaw<F, GenericForceTag>;
template <typename F>
concept UserUpdateFunc = TaggedLaw<F, UpdateFuncTag>;
template <typename F>
concept UserLinkLaw = TaggedLaw<F, LinkForceTag>;
template <typename F>
constexpr bool is_link_law() {
  if constexpr (requires { F::is_link; }) return F::is_link;
  else return UserLinkLaw<F>;
}
// no law of that kind in the step
struct NoLaw {};
// A force argument as a step uses it.  PAIRWISE_FORCE(...) and its kin are
// factories (utils.hpp:237-255); the reference's take_step takes a factory
// or its result, so a factory is called here.
template <typename F>
decltype(auto) resolve_force(const F& f) {
  if constexpr (requires { typename F::tag; } || requires { F::force_id; } || is_link_law<F>()) {
    return (f);
  } else if constexpr (std::is_invocable_v<const F&>) {
    return f();
  } else {
    return (f);
  }
}
// Hands a step's user laws (generic G, pairwise P; NoLaw where absent) to a
// simulation's library handle; defined by tecs/pairwise.cuh.
template <typename Config, typename G, typename P, typename L>
struct PairLawBinding;
}  // namespace detail

// Cell division after each step (the pattern of examples/growth_w_wall.cpp:119-136,
// done on the device): each active cell divides with this probability per step;
// its daughter is placed at offset * a random unit vector and appended.
struct DivisionSettings {
  double probability = 0.0;
  float offset = 0.25f;
};

template <typename Config>
class Simulation {
 public:
  using Scalar = typename Config::Scalar;
  static constexpr int dimensions = Config::dimensions;
  using Vector = VectorN<Scalar, dimensions>;
  using Polarity = Polarity_<Scalar>;
  using Fields = typename Config::Fields;
  using PairFinder = typename Config::template PairFinderT<Config>;
  using Integrator = typename Config::template IntegratorT<Config>;
  using ComFixer = typename Config::template ComFixerT<Config>;
  using Writer = typename Config::template WriterT<Config>;

  static_assert(std::is_same_v<Scalar, float>, "the GB300 path computes in float");
  static_assert(dimensions == 2 || dimensions == 3, "2 or 3 dimensions");

 private:
  // the fields as the library holds them (tecs/config.hpp: FieldLayout)
  using Layout = detail::FieldLayout<Fields>;
  static_assert(std::is_same_v<typename Layout::template type<0>, Vector>, "the first field must be a Vector");
  static_assert(Layout::extra <= 8, "at most 8 float components of extra fields");
  template <std::size_t K>
  using FieldType = typename Layout::template type<K>;
  // one view per field; the position's and the polarity's are positions_ and
  // polarity_, the other fields' live here (their slots in this tuple for the
  // position and the polarity stay empty)
  using FieldViews = decltype([]<std::size_t... K>(std::index_sequence<K...>) {
    return std::tuple<View<FieldType<K>>...>{};
  }(std::make_index_sequence<Layout::n>{}));
  template <typename F, std::size_t... K>
  void each_extra(F&& f, std::index_sequence<K...>) {
    (
        [&] {
          if constexpr (Layout::role(K) == 2) f(std::integral_constant<std::size_t, K>{}, std::get<K>(extras_));
        }(),
        ...);
  }
  // f(index, view) for every extra field
  template <typename F>
  void each_extra(F&& f) {
    each_extra(static_cast<F&&>(f), std::make_index_sequence<Layout::n>{});
  }
  template <typename Field, std::size_t... K>
  static constexpr std::size_t index_of(std::index_sequence<K...>) {
    std::size_t at = Layout::n;
    ((at = std::is_same_v<Field, std::tuple_element_t<K, typename FieldListTuple<Fields>::type>> ? K : at), ...);
    return at;
  }
  template <typename L>
  struct FieldListTuple;
  template <typename... Fs>
  struct FieldListTuple<detail::FieldList<Fs...>> {
    using type = std::tuple<Fs...>;
  };

 public:
  static constexpr bool has_polarity = Layout::has_polarity;

  struct Settings {
    Settings(unsigned agent_count_, const std::string& output_path_)
        : agent_count(agent_count_), output_path(output_path_), capacity(agent_count_) {}
    unsigned agent_count;
    std::string output_path;
    unsigned capacity;
    Scalar cutoff_distance = Scalar(1'000'000);
    std::uint64_t seed = 2807;
    typename PairFinder::Settings pair_finder_settings = {};
    typename Writer::Settings writer_settings = {};
    // extension: device-side cell division after every step
    DivisionSettings division = {};
    int device = 0;
    /// Allocate space for links between agents (0 = no links), and how many are active.
    unsigned int link_capacity = 0;
    unsigned int link_active_count = 0;
  };

  // legacy positional constructor (include/simulation.hpp:110-126)
  Simulation(unsigned agent_count, const std::string& output_path, Scalar cutoff_distance = Scalar(1'000'000),
             const typename PairFinder::Settings& pair_finder_settings = {}, std::uint64_t seed = 2807)
      : Simulation(make_settings(agent_count, output_path, cutoff_distance, pair_finder_settings, seed)) {}

  explicit Simulation(const Settings& s)
      : agent_count(s.agent_count), capacity(s.capacity), settings_(s), writer_(s.output_path, s.writer_settings),
        pool_(s.seed) {
    if (s.capacity < s.agent_count) throw Error("capacity must be >= agent_count");
    tecs_sim_desc d{};
    check(tecs_sim_desc_default(&d));
    d.dims = dimensions;
    d.finder = PairFinder::finder_id;
    d.symmetric = PairFinder::symmetric ? 1 : 0;
    d.cutoff = s.cutoff_distance;
    apply_finder_settings(d, s.pair_finder_settings);
    d.integrator = Integrator::integrator_id;
    d.com_fix = ComFixer::com_fix;
    d.force = TECS_FORCE_NONE;
    d.has_polarity = has_polarity ? 1 : 0;
    d.capacity = s.capacity;
    d.division_probability = s.division.probability;
    d.division_offset = s.division.offset;
    d.seed = s.seed;
    d.device = s.device;
    delaunay_for_capacity(d);
    check(tecs_sim_create(&d, &handle_));
    desc_ = d;
    positions_ = View<Vector>(std::string(field_name<0>()), s.agent_count, s.capacity);
    if constexpr (has_polarity) polarity_ = View<Polarity>("polarity", s.agent_count, s.capacity);
    links_ = View<Link>("links", s.link_active_count, s.link_capacity);
    // zero-initialised views are the first state, as Kokkos views are
    positions_.set_host_modified(true);
    auto refresh = [this]() { refresh_host(); };
    positions_.set_refresh(refresh);
    if constexpr (has_polarity) polarity_.set_refresh(refresh);
    if constexpr (Layout::extra > 0) {
      check(tecs_sim_set_extra_fields(handle_, Layout::extra, Layout::double_mask()));
      each_extra([&](auto k, auto& v) {
        v = View<FieldType<k>>(std::string(field_name<k>()), s.agent_count, s.capacity);
        v.set_refresh(refresh);
      });
    }
  }

  Simulation(const Simulation&) = delete;
  Simulation& operator=(const Simulation&) = delete;
  ~Simulation() {
    positions_.set_refresh(nullptr);
    if constexpr (has_polarity) polarity_.set_refresh(nullptr);
    each_extra([&](auto, auto& v) { v.set_refresh(nullptr); });
    if (handle_) tecs_sim_destroy(handle_);
  }

  // -- views ----------------------------------------------------------------
  // A field's view (simulation.hpp:231-256): current on the host when read
  // there, and sent to the library before the next step if written.
  template <typename Field>
  View<typename Field::value_type>& get_view() {
    return view_of<Field>();
  }
  template <typename Field>
  const View<typename Field::value_type>& get_view() const {
    return const_cast<Simulation*>(this)->template view_of<Field>();
  }
  View<Vector>& get_positions_view() { return positions_; }

  // The links (include/simulation.hpp:317-332): link_capacity entries, the
  // first get_active_count() in use, written on the host or by device code;
  // they reach the library with the next step that passes a link law.
  View<Link>& get_links() {
    links_dirty_ = true;
    return links_;
  }
  const View<Link>& get_links() const { return links_; }
  // the links view's capacity, as the reference's (simulation.hpp:330-333)
  unsigned get_link_count() const { return static_cast<unsigned>(links_.extent(0)); }

  // The integrator's old velocities (include/simulation.hpp:312-314,
  // integrators/base.hpp:74): each step's velocity per cell, which user
  // pairwise laws that set drag read.  The library keeps them once a step
  // has run a user pairwise law or this was called (zero until the next
  // step); the view returned is a copy of them as they are now.
  View<Vector> get_old_velocities_view_from_integrator() {
    keep_old_velocities();
    View<Vector> v("integrator_base_old_velocities", capacity);
    std::vector<float> buf(std::size_t(capacity) * dimensions);
    unsigned n = 0;
    check(tecs_sim_old_velocities(handle_, buf.data(), &n));
    for (unsigned c = 0; c < n; ++c)
      for (int d = 0; d < dimensions; ++d) v.host_array()[c][d] = buf[std::size_t(c) * dimensions + d];
    v.copy_to_device();
    return v;
  }

  unsigned get_capacity() const { return capacity; }
  unsigned get_agent_count() const {
    if (lib_newer_host_ || lib_newer_dev_) {
      unsigned n = 0;
      check(tecs_sim_count(handle_, &n));
      const_cast<Simulation*>(this)->agent_count = n;
    }
    return agent_count;
  }
  // Simulation::set_agent_count (include/simulation.hpp:295-302): the next
  // step starts from the first n cells and resets the finder's counter
  // A new capacity (include/simulation.hpp:266-281): the field views, the
  // library's state and the integrator's old velocities keep their first
  // values; extra views passed along are resized too.  The library's
  // simulation is made anew at the new size and the state sent to it, so user
  // laws bind again at the next step.
  void set_capacity(unsigned value) {
    if (value < agent_count) throw Error("capacity below the agent count");
    sync_to_library();
    refresh_host();
    std::vector<float> ov;
    if (old_velocities_kept_ && agent_count) {
      ov.resize(std::size_t(agent_count) * dimensions);
      unsigned n = 0;
      check(tecs_sim_old_velocities(handle_, ov.data(), &n));
    }
    tecs_sim_desc d = desc_;
    d.capacity = value;
    delaunay_for_capacity(d);
    tecs_sim* next = nullptr;
    check(tecs_sim_create(&d, &next));
    check(tecs_sim_set_pair_law(handle_, nullptr, nullptr));
    tecs_sim_destroy(handle_);
    handle_ = next;
    desc_ = d;
    law_holder_.reset();
    law_fn_ = nullptr;
    links_on_device_ = 0;
    links_dirty_ = true;
    capacity = value;
    positions_.resize(value);
    if constexpr (has_polarity) polarity_.resize(value);
    each_extra([&](auto, auto& v) { v.resize(value); });
    if constexpr (Layout::extra > 0) check(tecs_sim_set_extra_fields(handle_, Layout::extra, Layout::double_mask()));
    set_count(agent_count);
    mark_fields_host_modified();
    lib_newer_dev_ = lib_newer_host_ = false;
    if (old_velocities_kept_) {
      old_velocities_kept_ = false;
      keep_old_velocities();
      if (!ov.empty()) check(tecs_sim_set_old_velocities(handle_, ov.data(), agent_count));
    }
  }
  template <typename V0, typename... Vs>
  void set_capacity(unsigned value, V0& view0, Vs&... views) {
    set_capacity(value);
    view0.resize(value);
    (views.resize(value), ...);
  }

  void set_agent_count(unsigned n) {
    if (n > capacity) throw Error("agent count exceeds capacity");
    refresh_host();
    agent_count = n;
    positions_.set_active_count(n);
    if constexpr (has_polarity) polarity_.set_active_count(n);
    positions_.set_host_modified(true);
  }
  // the same, and the active count of extra views (simulation.hpp:305-309)
  template <typename V0, typename... Vs>
  void set_agent_count(unsigned n, V0& view0, Vs&... views) {
    set_agent_count(n);
    view0.set_active_count(n);
    (views.set_active_count(n), ...);
  }

  // -- stepping ---------------------------------------------------------------
  // take_step(dt, forces...): one integrator step with at most one pairwise
  // law (built-in, or a user law of tecs/pairwise.cuh), at most one generic
  // law and at most one link law, in any order (the reference fuses forces by
  // kind, kernel_fuser.hpp:148-156).  A PAIRWISE_FORCE(...) factory may be
  // passed itself or called, as the reference accepts both.
  template <typename... Forces>
  void take_step(double dt, const Forces&... forces) {
    take_steps(dt, 1, forces...);
  }
  // n steps queued at once (one graph replay each)
  template <typename... Forces>
  void take_steps(double dt, int n, const Forces&... forces) {
    take_steps_impl(dt, n, detail::resolve_force(forces)...);
  }

  // One full-step force evaluation of the current state without moving it:
  // per-cell deltas and the directed (self, other) pairs found.
  template <typename Force>
  std::vector<std::pair<unsigned, unsigned>> evaluate(const Force& force, std::vector<Vector>* deltas = nullptr) {
    const auto& f = detail::resolve_force(force);
    apply_pair_law(f);
    apply_link_law(f);
    sync_to_library();
    const unsigned n = get_agent_count();
    std::vector<Vector> dx(n ? n : 1);
    std::vector<std::uint32_t> raw(2 * std::size_t(64) * (n ? n : 1));
    std::size_t count = 0;
    for (;;) {
      check(tecs_sim_evaluate(handle_, reinterpret_cast<float*>(dx.data()), nullptr, raw.data(), raw.size() / 2,
                              &count));
      if (count <= raw.size() / 2) break;
      raw.resize(2 * count);
    }
    if (deltas) deltas->assign(dx.begin(), dx.begin() + n);
    std::vector<std::pair<unsigned, unsigned>> pairs(count);
    for (std::size_t k = 0; k < count; ++k) pairs[k] = {raw[2 * k], raw[2 * k + 1]};
    return pairs;
  }

  void synchronize() { check(tecs_sim_synchronize(handle_)); }

  // -- initialisers (include/initializers, simulation.hpp:348-546) -----------
  // Each places the agents, then applies the given init functions, all on the
  // host in cell order from the simulation's generator (see the file comment).
  template <typename... InitFuncs>
  void init_random_filled_sphere(Scalar radius, InitFuncs&&... init_functions) {
    static_assert(dimensions >= 3, "a random filled sphere needs 3 dimensions");
    init(
        [&](unsigned i, Random& g) {
          // initializers/spheres.hpp:56-75
          const Scalar r = radius * Kokkos::cbrt(static_cast<Scalar>(g.drand()));
          const Scalar z = static_cast<Scalar>(g.drand(0.0, 2.0)) - Scalar(1.0);
          const Scalar theta = static_cast<Scalar>(g.drand(0.0, 2.0 * Kokkos::numbers::pi_v<double>));
          const Scalar rxy = Kokkos::sqrt(Scalar(1.0) - z * z) * r;
          positions_(i)[0] = rxy * Kokkos::cos(theta);
          positions_(i)[1] = rxy * Kokkos::sin(theta);
          positions_(i)[2] = z * r;
        },
        static_cast<InitFuncs&&>(init_functions)...);
  }
  template <typename... InitFuncs>
  void init_random_hollow_sphere(Scalar radius, InitFuncs&&... init_functions) {
    static_assert(dimensions >= 3, "a random hollow sphere needs 3 dimensions");
    init(
        [&](unsigned i, Random& g) {
          // initializers/spheres.hpp:24-41
          const Scalar u = static_cast<Scalar>(g.drand());
          const Scalar v = static_cast<Scalar>(g.drand());
          const Scalar z = Scalar(2.0) * u - Scalar(1.0);
          const Scalar theta = Scalar(2.0) * Scalar(Kokkos::numbers::pi_v<Scalar>) * v;
          const Scalar rxy = Kokkos::sqrt(Scalar(1.0) - z * z) * radius;
          positions_(i)[0] = rxy * Kokkos::cos(theta);
          positions_(i)[1] = rxy * Kokkos::sin(theta);
          positions_(i)[2] = z * radius;
        },
        static_cast<InitFuncs&&>(init_functions)...);
  }
  // A random filled sphere relaxed by `steps` steps (default 2000) of dt 0.1
  // with the piecewise-linear law at distance 0.8 (repulsion 2, adhesion 1;
  // initializers/spheres.hpp:86-106, relax_force.hpp:17-30), then the init
  // functions.  The relax law is the built-in spring of the same arithmetic.
  template <typename... Args>
  void init_relaxed_sphere(Scalar radius, Args&&... args) {
    if constexpr (sizeof...(Args) > 0 && (std::is_integral_v<std::decay_t<Args>> || ...)) {
      init_relaxed_sphere_n(radius, static_cast<Args&&>(args)...);
    } else {
      init_relaxed_sphere_n(radius, 2000u, static_cast<Args&&>(args)...);
    }
  }

  // agents on a line: every component of cell i at i * distance (initializers/line.hpp)
  template <typename... InitFuncs>
  void init_line(Scalar distance, InitFuncs&&... init_functions) {
    init([&](unsigned i, Random&) { positions_(i) = Vector(Scalar(i) * distance); },
         static_cast<InitFuncs&&>(init_functions)...);
  }
  // uniform in [min, max) per component (initializers/cuboid.hpp:19-44)
  template <typename... InitFuncs>
  void init_random_cuboid(const Vector& min, const Vector& max, InitFuncs&&... init_functions) {
    const Vector extent = max - min;
    init(
        [&](unsigned i, Random& g) {
          for (int d = 0; d < dimensions; ++d) positions_(i)[d] = min[d] + g.drand(0.0, extent[d]);
        },
        static_cast<InitFuncs&&>(init_functions)...);
  }
  // a random cuboid relaxed by `steps` steps (default 2000), then the init
  // functions (initializers/cuboid.hpp:50-85, simulation.hpp:452-506)
  template <typename... Args>
  void init_relaxed_cuboid(const Vector& min, const Vector& max, Args&&... args) {
    if constexpr (sizeof...(Args) > 0 && (std::is_integral_v<std::decay_t<Args>> || ...)) {
      init_relaxed_cuboid_n(min, max, static_cast<Args&&>(args)...);
    } else {
      init_relaxed_cuboid_n(min, max, 2000u, static_cast<Args&&>(args)...);
    }
  }
  // rings of a hexagonal lattice around cell 0 (initializers/hexagon.hpp:21-64):
  // cell i > 0 on ring k, side s, step t, linearly between the ring's corners
  template <typename... InitFuncs>
  void init_regular_hexagon(Scalar distance_to_neighbour, InitFuncs&&... init_functions) {
    static_assert(dimensions >= 2, "a hexagon needs 2 dimensions");
    init(
        [&](unsigned i, Random&) {
          if (i == 0) return;
          unsigned remaining = i - 1, ring = 1;
          while (remaining >= 6 * ring) {
            remaining -= 6 * ring;
            ++ring;
          }
          const Scalar beta = Scalar(Kokkos::numbers::pi_v<Scalar>) / Scalar(3);
          const unsigned side = remaining / ring, step = remaining % ring;
          const Scalar radius = distance_to_neighbour * Scalar(ring);
          const Scalar t = Scalar(step) / Scalar(ring);
          const Scalar s0 = -radius * Kokkos::sin(beta * Scalar(side));
          const Scalar c0 = radius * Kokkos::cos(beta * Scalar(side));
          const Scalar s1 = -radius * Kokkos::sin(beta * Scalar(side + 1));
          const Scalar c1 = radius * Kokkos::cos(beta * Scalar(side + 1));
          Vector p{Scalar(0)};
          p[0] = s0 + (s1 - s0) * t;
          p[1] = c0 + (c1 - c0) * t;
          positions_(i) = p;
        },
        static_cast<InitFuncs&&>(init_functions)...);
  }
  // rows of nx cells, every other row shifted by half a spacing
  // (initializers/rectangle.hpp:21-50)
  template <typename... InitFuncs>
  void init_regular_rectangle(Scalar distance_to_neighbour, unsigned nx, InitFuncs&&... init_functions) {
    static_assert(dimensions >= 2, "a rectangle needs 2 dimensions");
    init(
        [&](unsigned i, Random&) {
          const unsigned row = i / nx, col = i % nx;
          const Scalar row_height = distance_to_neighbour * Scalar(0.5) * Kokkos::sqrt(Scalar(3.0));
          const Scalar row_offset = (row % 2 != 0) ? (distance_to_neighbour * Scalar(0.5)) : Scalar(0.0);
          positions_(i)[0] = row_offset + Scalar(col) * distance_to_neighbour;
          positions_(i)[1] = Scalar(row) * row_height;
        },
        static_cast<InitFuncs&&>(init_functions)...);
  }
  // uniform in a disk of radius sqrt(capacity) * spacing / 2
  // (initializers/disk.hpp:20-41: the view's extent is its capacity)
  template <typename... InitFuncs>
  void init_random_disk(Scalar distance_to_neighbour, InitFuncs&&... init_functions) {
    static_assert(dimensions >= 2, "a disk needs 2 dimensions");
    const Scalar r_max = Kokkos::sqrt(static_cast<Scalar>(positions_.extent(0))) * distance_to_neighbour / Scalar(2.0);
    init(
        [&](unsigned i, Random& g) {
          const Scalar r = r_max * Kokkos::sqrt(static_cast<Scalar>(g.drand()));
          const Scalar phi = static_cast<Scalar>(g.drand()) * Scalar(2.0) * Kokkos::numbers::pi_v<Scalar>;
          positions_(i)[0] = r * Kokkos::sin(phi);
          positions_(i)[1] = r * Kokkos::cos(phi);
        },
        static_cast<InitFuncs&&>(init_functions)...);
  }
  // rejection sampling of the heart surface's inside in [-2, 2)^3, scaled
  // (initializers/heart.hpp:22-55)
  template <typename... InitFuncs>
  void init_random_heart(Scalar scale, InitFuncs&&... init_functions) {
    static_assert(dimensions >= 3, "a heart needs 3 dimensions");
    auto outside = [](Scalar x, Scalar y, Scalar z) {
      return Kokkos::pow(x * x + 9.0 / 4.0 * y * y + z * z - 1.0, 3) - x * x * z * z * z -
             9.0 / 80.0 * y * y * z * z * z;
    };
    init(
        [&](unsigned i, Random& g) {
          Scalar x, y, z;
          do {
            x = static_cast<Scalar>(g.drand(-2.0, 2.0));
            y = static_cast<Scalar>(g.drand(-2.0, 2.0));
            z = static_cast<Scalar>(g.drand(-2.0, 2.0));
          } while (outside(x, y, z) > Scalar(0.0));
          positions_(i)[0] = x * scale;
          positions_(i)[1] = y * scale;
          positions_(i)[2] = z * scale;
        },
        static_cast<InitFuncs&&>(init_functions)...);
  }

  // init(f, fs...) (simulation.hpp:519-537): f(i, rng) for every agent in
  // cell order, then the next function
  template <typename Initializer, typename... InitFuncs>
  void init(Initializer&& initializer, InitFuncs&&... init_functions) {
    refresh_host();
    const unsigned n = agent_count;
    for (unsigned i = 0; i < n; ++i) {
      Random g = pool_.get_state();
      initializer(i, g);
      pool_.free_state(g);
    }
    mark_fields_host_modified();
    if constexpr (sizeof...(init_functions) > 0) init(static_cast<InitFuncs&&>(init_functions)...);
  }

  // run_custom(count, f...) (include/simulation.hpp:566-598): f(i, rng) for
  // i in [0, count).  Several functions are fused per index as the
  // reference's kernel fuser does (kernel_fuser.hpp:42-48): for each i every
  // function in turn, with the same generator.  Like init, on the host in
  // index order from the reference's generator stream; the views and the
  // links the functions may write are sent to the library before the next
  // step.
  template <typename... Funcs>
  void run_custom(unsigned count, Funcs&&... functions) {
    refresh_host();
    for (unsigned i = 0; i < count; ++i) {
      Random g = pool_.get_state();
      (functions(i, g), ...);
      pool_.free_state(g);
    }
    mark_fields_host_modified();
    links_dirty_ = true;
  }
  // over the agents, and over the active links
  template <typename... Funcs>
  void run(Funcs&&... functions) {
    run_custom(agent_count, static_cast<Funcs&&>(functions)...);
  }
  template <typename... Funcs>
  void run_links(Funcs&&... functions) {
    run_custom(links_.get_active_count(), static_cast<Funcs&&>(functions)...);
  }

  // -- output (include/simulation.hpp:600-667) --------------------------------
  // One snapshot of every field, the given extra views and the links, in
  // group "t<current_step>"; current_step counts the writes.  The config's
  // writer decides the format (io::HDF5_Writer: "<output_path>.h5";
  // io::Dummy: nothing).
  void write(double time) { write_all(time); }
  template <typename T0, typename... Ts>
  void write(double time, const View<T0>& extra0, const View<Ts>&... extra) {
    write_all(time, extra0, extra...);
  }
  void write() { write(last_dt * current_step); }
  template <typename T0, typename... Ts>
  void write(const View<T0>& extra0, const View<Ts>&... extra) {
    write(last_dt * current_step, extra0, extra...);
  }
  template <typename... Ts>
  void write_static(const View<Ts>&... views) {
    writer_.write_static(views...);
  }

  tecs_sim* handle() const { return handle_; }

  unsigned agent_count;
  unsigned capacity;
  unsigned current_step = 0;
  double last_dt = 0.0;

 private:
  using Random = XorShiftRandom;

  static Settings make_settings(unsigned n, const std::string& path, Scalar cutoff,
                                const typename PairFinder::Settings& pfs, std::uint64_t seed) {
    Settings s(n, path);
    s.cutoff_distance = cutoff;
    s.pair_finder_settings = pfs;
    s.seed = seed;
    return s;
  }

  template <typename... InitFuncs>
  void init_relaxed_sphere_n(Scalar radius, unsigned steps, InitFuncs&&... init_functions) {
    init_random_filled_sphere(radius);
    relax(steps);
    if constexpr (sizeof...(init_functions) > 0) init(static_cast<InitFuncs&&>(init_functions)...);
  }
  template <typename... InitFuncs>
  void init_relaxed_cuboid_n(const Vector& min, const Vector& max, unsigned steps, InitFuncs&&... init_functions) {
    init_random_cuboid(min, max);
    relax(steps);
    if constexpr (sizeof...(init_functions) > 0) init(static_cast<InitFuncs&&>(init_functions)...);
  }
  // `steps` steps of dt 0.1 with the piecewise-linear law at distance 0.8,
  // repulsion 2, adhesion 1 (initializers/relax_force.hpp:17-30: the
  // built-in two-radius spring of the same arithmetic)
  void relax(unsigned steps) {
    for (unsigned k = 0; k < steps; ++k) take_step(0.1, forces::Spring2R{2.0f, 0.8f, 1.0f, 0.8f});
  }

  template <typename... Forces>
  void take_steps_impl(double dt, int n, const Forces&... forces) {
    static_assert((0 + ... + (detail::is_link_law<Forces>() || detail::UserGenericLaw<Forces> ? 0 : 1)) <= 1,
                  "one pairwise law per step");
    static_assert((0 + ... + (detail::is_link_law<Forces>() ? 1 : 0)) <= 1, "one link law per step");
    static_assert((0 + ... + (detail::UserGenericLaw<Forces> ? 1 : 0)) <= 1, "one generic law per step");
    static_assert(!(false || ... || detail::UserUpdateFunc<Forces>),
                  "UPDATE_FUNC functions run through Simulation::init, not take_step");
    constexpr bool user = (false || ... ||
                           (detail::UserGenericLaw<Forces> || detail::UserPairLaw<Forces> || detail::UserLinkLaw<Forces>));
    apply_pair_law(forces...);
    apply_link_law(forces...);
    sync_to_library();
    if constexpr (user) {
      // user code may read and write views and device values on the device
      refresh_device();
      detail::push_device_vars();
    }
    check(tecs_sim_step(handle_, dt, n));
    mark_library_newer();
    if constexpr (user) {
      detail::device_ran_user_code();
      user_code_ran_ = true;
    }
    last_dt = dt;
  }

  // the first force of type kind in the pack, or NoLaw{}
  template <template <typename> class Is, typename F0, typename... Fs>
  static const auto& first_of(const F0& f0, const Fs&... fs) {
    if constexpr (Is<F0>::value) return f0;
    else return first_of<Is>(fs...);
  }
  template <template <typename> class Is>
  static const detail::NoLaw& first_of() {
    static const detail::NoLaw none{};
    return none;
  }
  template <typename F>
  struct IsGeneric : std::bool_constant<detail::UserGenericLaw<F>> {};
  template <typename F>
  struct IsUserPair : std::bool_constant<detail::UserPairLaw<F>> {};
  template <typename F>
  struct IsUserLink : std::bool_constant<detail::UserLinkLaw<F>> {};

  // the pairwise law of this step (none: pairs only, no deltas); user laws
  // (a PAIRWISE_FORCE, a GENERIC_FORCE and a LINK_FORCE law, any of them)
  // replace the built-in one until a step passes a built-in law again
  template <typename... Forces>
  void apply_pair_law(const Forces&... forces) {
    int id = TECS_FORCE_NONE;
    float k[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
    constexpr bool generic = (false || ... || detail::UserGenericLaw<Forces>);
    constexpr bool user_pair = (false || ... || detail::UserPairLaw<Forces>);
    constexpr bool user_link = (false || ... || detail::UserLinkLaw<Forces>);
    constexpr bool user = generic || user_pair || user_link;
    auto one = [&](const auto& f) {
      using F = std::decay_t<decltype(f)>;
      if constexpr (!detail::UserPairLaw<F> && !detail::UserGenericLaw<F> && !detail::is_link_law<F>()) {
        static_assert(!user || sizeof(F) == 0,
                      "GENERIC_FORCE and LINK_FORCE laws combine with a PAIRWISE_FORCE law, not a built-in one");
        static_assert(!F::needs_polarity || has_polarity, "this force needs a (Polarity, polarity) field");
        id = F::force_id;
        k[0] = f.k_rep; k[1] = f.r_rep; k[2] = f.k_adh; k[3] = f.r_adh; k[4] = f.k_pol_value();
      }
    };
    (one(forces), ...);
    // a pairwise law may set drag, which reads the old velocities
    if constexpr (user_pair) keep_old_velocities();
    if constexpr (user) {
      const auto& g = first_of<IsGeneric>(forces...);
      const auto& p = first_of<IsUserPair>(forces...);
      const auto& l = first_of<IsUserLink>(forces...);
      detail::PairLawBinding<Config, std::decay_t<decltype(g)>, std::decay_t<decltype(p)>,
                             std::decay_t<decltype(l)>>::bind(handle_, settings_.device, g, p, l, law_holder_,
                                                              law_fn_);
    }
    if (!user && law_fn_) {
      check(tecs_sim_set_pair_law(handle_, nullptr, nullptr));
      law_holder_.reset();
      law_fn_ = nullptr;
    }
    check(tecs_sim_set_force(handle_, id, k[0], k[1], k[2], k[3], k[4]));
  }

  // the link law of this step: links act only in steps that pass one.  The
  // reference evaluates every link of the view's capacity
  // (integrators/base.hpp:196-233, links.extent(0)); unused slots hold
  // (0, 0), which it skips as a self link.
  template <typename... Forces>
  void apply_link_law(const Forces&... forces) {
    bool has = false;
    float strength = 0.f;
    auto one = [&](const auto& f) {
      using F = std::decay_t<decltype(f)>;
      if constexpr (detail::UserLinkLaw<F>) {
        has = true;
      } else if constexpr (detail::is_link_law<F>()) {
        has = true;
        strength = f.strength;
      }
    };
    (one(forces), ...);
    const unsigned want = has ? static_cast<unsigned>(links_.extent(0)) : 0u;
    if (!links_dirty_ && want == links_on_device_ && (!has || strength == link_strength_)) return;
    if (want) links_.sync_host();  // links written by device code
    check(tecs_sim_set_links(handle_, want ? reinterpret_cast<const uint32_t*>(links_.data()) : nullptr, want,
                             strength));
    links_on_device_ = want;
    link_strength_ = strength;
    links_dirty_ = false;
  }

  template <typename PFS>
  static void apply_finder_settings(tecs_sim_desc& d, const PFS& p) {
    if constexpr (requires { p.gabriel_coefficient; }) d.gabriel_coefficient = p.gabriel_coefficient;
    if constexpr (requires { p.min_bounds; }) {
      for (int k = 0; k < 3; ++k) {
        d.min_bounds[k] = k < dimensions ? p.min_bounds[k] : 0.0f;
        d.max_bounds[k] = k < dimensions ? p.max_bounds[k] : 0.0f;
      }
    }
    if constexpr (requires { p.bin_size_scale; }) d.bin_size_scale = p.bin_size_scale;
    if constexpr (requires { p.rebuild_every_n; }) d.rebuild_every_n = p.rebuild_every_n;
  }

  template <std::size_t K>
  static constexpr std::string_view field_name() {
    return std::tuple_element_t<K, typename FieldListTuple<Fields>::type>::name;
  }
  template <std::size_t K>
  View<FieldType<K>>& view_at() {
    if constexpr (Layout::role(K) == 0) return positions_;
    else if constexpr (Layout::role(K) == 1) return polarity_;
    else return std::get<K>(extras_);
  }
  template <typename Field>
  View<typename Field::value_type>& view_of() {
    constexpr std::size_t K = index_of<Field>(std::make_index_sequence<Layout::n>{});
    static_assert(K < Layout::n, "no such field in this config");
    return view_at<K>();
  }

  // every field in the config's order, then the extra views, then the links
  // (the reference writes get_views() first, simulation.hpp:600-667)
  template <typename... Ts>
  void write_all(double time, const View<Ts>&... extra) {
    refresh_host();
    const unsigned step = current_step++;
    [&]<std::size_t... K>(std::index_sequence<K...>) {
      writer_.write(time, step, view_at<K>()..., extra..., links_);
    }(std::make_index_sequence<Layout::n>{});
  }

  // The library's state after steps is newer than both arrays of the field views.
  void mark_library_newer() {
    lib_newer_dev_ = lib_newer_host_ = true;
    positions_.set_stale(true);
    if constexpr (has_polarity) polarity_.set_stale(true);
    each_extra([&](auto, auto& v) { v.set_stale(true); });
  }
  template <std::size_t K>
  static constexpr unsigned width_of() {
    return detail::FieldWidth<FieldType<K>>::value;
  }
  // library -> the field views' device arrays (cell-id order, on the device)
  void refresh_device() {
    if (!lib_newer_dev_) return;
    unsigned n = 0;
    check(tecs_sim_download_device(handle_, reinterpret_cast<float*>(positions_.device_data()),
                                   has_polarity ? reinterpret_cast<float*>(polarity_.device_data()) : nullptr, &n));
    set_count(n);
    each_extra([&](auto k, auto& v) {
      unsigned m = 0;
      check(tecs_sim_download_extra(handle_, Layout::offset(k), width_of<k>(), reinterpret_cast<float*>(v.device_data()),
                                    &m));
      v.clear_device_flag();
    });
    lib_newer_dev_ = false;
    positions_.clear_device_flag();
    if constexpr (has_polarity) polarity_.clear_device_flag();
  }
  // library -> the field views' host arrays (through their device arrays)
  void refresh_host() {
    if (!lib_newer_host_) return;
    refresh_device();
    positions_.copy_to_host();
    if constexpr (has_polarity) polarity_.copy_to_host();
    positions_.set_stale(false);
    if constexpr (has_polarity) polarity_.set_stale(false);
    positions_.set_host_modified(false);
    if constexpr (has_polarity) polarity_.set_host_modified(false);
    each_extra([&](auto, auto& v) {
      v.copy_to_host();
      v.set_stale(false);
      v.set_host_modified(false);
    });
    lib_newer_host_ = false;
  }
  void set_count(unsigned n) {
    agent_count = n;
    positions_.set_active_count(n);
    if constexpr (has_polarity) polarity_.set_active_count(n);
    each_extra([&](auto, auto& v) { v.set_active_count(n); });
  }
  void mark_fields_host_modified() {
    positions_.set_host_modified(true);
    if constexpr (has_polarity) polarity_.set_host_modified(true);
    each_extra([&](auto, auto& v) { v.set_host_modified(true); });
  }
  // field views written since the library last read them -> the library: the
  // host arrays when host code wrote them, else the device arrays when
  // device code did
  void sync_to_library() {
    const bool host = positions_.host_modified() || (has_polarity && polarity_.host_modified());
    bool host_extra = false;
    each_extra([&](auto, auto& v) { host_extra = host_extra || v.host_modified(); });
    if (host || host_extra) {
      // the position upload keeps the library's extra fields (by cell id)
      if (host) {
        check(tecs_sim_upload(handle_, reinterpret_cast<const float*>(positions_.host_array()),
                              has_polarity ? reinterpret_cast<const float*>(polarity_.host_array()) : nullptr,
                              agent_count));
        positions_.set_host_modified(false);
        if constexpr (has_polarity) polarity_.set_host_modified(false);
      }
      each_extra([&](auto k, auto& v) {
        if (!v.host_modified()) return;
        check(tecs_sim_upload_extra(handle_, Layout::offset(k), width_of<k>(),
                                    reinterpret_cast<const float*>(v.host_array()), agent_count));
        v.set_host_modified(false);
      });
      // the device arrays did not see these writes
      lib_newer_dev_ = true;
      return;
    }
    if (!user_code_ran_) return;
    user_code_ran_ = false;
    if (lib_newer_dev_) return;
    const bool dev = positions_.device_flag() || (has_polarity && polarity_.device_flag());
    bool changed = false;
    if (dev) {
      check(tecs_sim_upload_device(handle_, reinterpret_cast<const float*>(positions_.device_data()),
                                   has_polarity ? reinterpret_cast<const float*>(polarity_.device_data()) : nullptr,
                                   agent_count));
      positions_.clear_device_flag();
      if constexpr (has_polarity) polarity_.clear_device_flag();
      changed = true;
    }
    each_extra([&](auto k, auto& v) {
      if (!v.device_flag()) return;
      check(tecs_sim_upload_extra(handle_, Layout::offset(k), width_of<k>(),
                                  reinterpret_cast<const float*>(v.device_data()), agent_count));
      v.clear_device_flag();
      changed = true;
    });
    if (changed) {
      lib_newer_host_ = true;
      positions_.set_stale(true);
      if constexpr (has_polarity) polarity_.set_stale(true);
      each_extra([&](auto, auto& v) { v.set_stale(true); });
    }
  }

  Settings settings_;
  Writer writer_;
  XorShiftPool pool_;
  // the bound user pairwise law (its launcher and the law object it launches with); destroyed after handle_
  std::shared_ptr<void> law_holder_;
  tecs_pair_law_fn law_fn_ = nullptr;
  tecs_sim* handle_ = nullptr;
  View<Vector> positions_;
  View<Polarity> polarity_;
  FieldViews extras_;
  View<Link> links_;
  bool links_dirty_ = false;        // the host links may differ from the device's
  unsigned links_on_device_ = 0;    // links active in the library
  float link_strength_ = 0.f;
  bool lib_newer_dev_ = false;      // the library's state is newer than the views' device arrays
  bool lib_newer_host_ = false;     // ... than their host arrays
  bool user_code_ran_ = false;      // user code ran on the device since the views were last checked
  bool old_velocities_kept_ = false;
  tecs_sim_desc desc_{};
  // NaiveDelaunay takes the library's Delaunay finder of any capacity past
  // the naive finder's 4096 cells (the same multiplicities in 2-D; the
  // Delaunay tetrahedra in 3-D), and the naive one below
  static void delaunay_for_capacity(tecs_sim_desc& d) {
    if (PairFinder::finder_id != TECS_FINDER_NAIVE_DELAUNAY) return;
    d.finder = d.capacity > 4096u ? TECS_FINDER_DELAUNAY : TECS_FINDER_NAIVE_DELAUNAY;
  }

  void keep_old_velocities() {
    if (old_velocities_kept_) return;
    check(tecs_sim_keep_old_velocities(handle_, 1));
    old_velocities_kept_ = true;
  }
};

}  // namespace tecs

// Init and update functions (utils.hpp:217, 249, 279-306): f(i, rng) per
// agent, run by Simulation::init and the initialisers.
#if defined(__CUDACC__)
#define TECS_CXX_LAMBDA [=] __host__ __device__
#else
#define TECS_CXX_LAMBDA [=]
#endif
#define INIT_FUNC(...) \
  [&]() { return TECS_CXX_LAMBDA([[maybe_unused]] const unsigned int i, [[maybe_unused]] Random& rng) { __VA_ARGS__ }; }
#define INIT_OP TECS_HD void operator()([[maybe_unused]] const unsigned int i, [[maybe_unused]] Random& generator) const
#define UPDATE_FUNC_PARAMETERS [[maybe_unused]] const unsigned int i, [[maybe_unused]] Random &rng
#define UPDATE_FUNC(...) \
  [&]() { return tecs::detail::update_func | TECS_CXX_LAMBDA(UPDATE_FUNC_PARAMETERS) { __VA_ARGS__ }; }
#define UPDATE_FUNC_OP                    \
  using tag = tecs::detail::UpdateFuncTag; \
  TECS_HD void operator()(UPDATE_FUNC_PARAMETERS) const

#endif  // TECS_CXX_SIMULATION_HPP
