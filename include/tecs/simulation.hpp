// tecs/simulation.hpp -- Simulation<Config> of the C++20 drop-in layer.
//
// Keeps the reference's Simulation interface for the per-timestep path
// (include/simulation.hpp:76-153 constructors and Settings, :231-302 views and
// counts, :548-556 take_step) and runs every step in the CUDA library through
// the C ABI of include/tecs_gpu.h.  The device holds the state; a field's
// View is a host mirror that is refreshed from the device when the program
// asks for it after steps and uploaded again before the next step if the
// program may have written it -- the DualView modified-flag protocol of
// include/types/view.hpp:47-266, with the host side explicit.
//
// Errors: every C-ABI failure throws tecs::Error with tecs_last_error().
#ifndef TECS_CXX_SIMULATION_HPP
#define TECS_CXX_SIMULATION_HPP

#include <cmath>
#include <cstdint>
#include <memory>
#include <random>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "../tecs_gpu.h"
#include "components.hpp"
#include "config.hpp"
#include "hdf5_writer.hpp"
#include "vector.hpp"

namespace tecs {

struct Error : std::runtime_error {
  using std::runtime_error::runtime_error;
};

inline void check(int rc) {
  if (rc != 0) throw Error(tecs_last_error());
}

// A field's values for the active agents, on the host.
template <typename T>
class View {
 public:
  using value_type = T;
  using non_const_value_type = std::remove_const_t<T>;

  View() = default;
  View(const std::string& label, std::size_t n) : label_(label), data_(n), active_(static_cast<unsigned>(n)) {}

  T& operator()(std::size_t i) { return data_[i]; }
  const T& operator()(std::size_t i) const { return data_[i]; }
  std::size_t extent(int) const { return data_.size(); }
  T* data() { return data_.data(); }
  const T* data() const { return data_.data(); }
  unsigned get_active_count() const { return active_; }
  void set_active_count(unsigned n) { active_ = n; }
  const std::string& label() const { return label_; }

  void resize(std::size_t n) { data_.resize(n); }

 private:
  std::string label_;
  std::vector<T> data_;
  unsigned active_ = 0;
};

namespace detail {
// the tags of user laws: PAIRWISE_FORCE / GENERIC_FORCE lambdas and their _OP functors
// (include/utils/utils.hpp:181-276), defined with tecs/pairwise.cuh
struct PairwiseForceTag {};
struct GenericForceTag {};
template <typename F, typename Tag>
concept TaggedLaw = requires { typename F::tag; } && std::is_same_v<typename F::tag, Tag>;
template <typename F>
concept UserPairLaw = TaggedLaw<F, PairwiseForceTag>;
template <typename F>
concept UserGenericLaw = TaggedLaw<F, GenericForceTag>;
template <typename F>
constexpr bool is_link_law() {
  if constexpr (requires { F::is_link; }) return F::is_link;
  else return false;
}
// no law of that kind in the step
struct NoLaw {};
// Hands a step's user laws (generic G, pairwise P; NoLaw where absent) to a
// simulation's library handle; defined by tecs/pairwise.cuh.
template <typename Config, typename G, typename P>
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
  template <typename F>
  static constexpr bool is_position_field = std::is_same_v<typename F::value_type, Vector> && F::name == "position";
  template <typename F>
  static constexpr bool is_polarity_field = std::is_same_v<typename F::value_type, Polarity> && F::name == "polarity";

  template <typename L>
  struct FieldShape;
  template <typename F0, typename... Fs>
  struct FieldShape<detail::FieldList<F0, Fs...>> {
    static constexpr int n = 1 + static_cast<int>(sizeof...(Fs));
    static constexpr bool first_is_position = is_position_field<F0>;
    static constexpr bool polarity = (false || ... || is_polarity_field<Fs>);
    static constexpr bool only_known = (true && ... && is_polarity_field<Fs>);
  };
  using Shape = FieldShape<Fields>;
  static_assert(Shape::first_is_position, "the first field must be (Vector, position)");
  static_assert(Shape::only_known && Shape::n <= 2,
                "the GB300 path carries a (Vector, position) field and an optional (Polarity, polarity) field");

 public:
  static constexpr bool has_polarity = Shape::polarity;

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
      : agent_count(s.agent_count), capacity(s.capacity), settings_(s), writer_(s.output_path, s.writer_settings) {
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
    check(tecs_sim_create(&d, &handle_));
    positions_ = View<Vector>("position", s.capacity);
    positions_.set_active_count(s.agent_count);
    if constexpr (has_polarity) {
      polarity_ = View<Polarity>("polarity", s.capacity);
      polarity_.set_active_count(s.agent_count);
    }
    host_valid_ = true;  // zero-initialised, as Kokkos views are
    host_dirty_ = true;
    links_ = View<Link>("links", s.link_capacity);
    links_.set_active_count(s.link_active_count);
  }

  Simulation(const Simulation&) = delete;
  Simulation& operator=(const Simulation&) = delete;
  ~Simulation() {
    if (handle_) tecs_sim_destroy(handle_);
  }

  // -- views ----------------------------------------------------------------
  // The returned view may be written: it is uploaded before the next step.
  template <typename Field>
  View<typename Field::value_type>& get_view() {
    refresh_host();
    host_dirty_ = true;
    return view_of<Field>();
  }
  template <typename Field>
  const View<typename Field::value_type>& get_view() const {
    const_cast<Simulation*>(this)->refresh_host();
    return const_cast<Simulation*>(this)->template view_of<Field>();
  }
  View<Vector>& get_positions_view() { return get_view<FIELD(Vector, position)>(); }

  // The links (include/simulation.hpp:317-332): a host view of link_capacity
  // entries, the first get_active_count() in use; written links reach the
  // device with the next step that passes a link law.
  View<Link>& get_links() {
    links_dirty_ = true;
    return links_;
  }
  const View<Link>& get_links() const { return links_; }
  unsigned get_link_count() const { return links_.get_active_count(); }

  unsigned get_capacity() const { return capacity; }
  unsigned get_agent_count() const {
    if (!host_valid_) {
      unsigned n = 0;
      check(tecs_sim_count(handle_, &n));
      const_cast<Simulation*>(this)->agent_count = n;
    }
    return agent_count;
  }
  // Simulation::set_agent_count (include/simulation.hpp:295-302): the next
  // step starts from the first n host values and resets the finder's counter
  void set_agent_count(unsigned n) {
    if (n > capacity) throw Error("agent count exceeds capacity");
    refresh_host();
    agent_count = n;
    positions_.set_active_count(n);
    if constexpr (has_polarity) polarity_.set_active_count(n);
    host_dirty_ = true;
  }

  // -- stepping ---------------------------------------------------------------
  // take_step(dt, forces...): one integrator step with at most one pairwise
  // law (built-in, or a user law of tecs/pairwise.cuh) and at most one link
  // law, in any order (the reference fuses forces by kind and evaluates
  // pairwise before link forces)
  template <typename... Forces>
  void take_step(double dt, const Forces&... forces) {
    take_steps(dt, 1, forces...);
  }
  // n steps queued at once (one graph replay each)
  template <typename... Forces>
  void take_steps(double dt, int n, const Forces&... forces) {
    static_assert((0 + ... + (detail::is_link_law<Forces>() || detail::UserGenericLaw<Forces> ? 0 : 1)) <= 1,
                  "one pairwise law per step");
    static_assert((0 + ... + (detail::is_link_law<Forces>() ? 1 : 0)) <= 1, "one link law per step");
    static_assert((0 + ... + (detail::UserGenericLaw<Forces> ? 1 : 0)) <= 1, "one generic law per step");
    apply_pair_law(forces...);
    apply_link_law(forces...);
    upload_if_dirty();
    check(tecs_sim_step(handle_, dt, n));
    host_valid_ = false;
    last_dt = dt;
  }

  // One full-step force evaluation of the current state without moving it:
  // per-cell deltas and the directed (self, other) pairs found.
  template <typename Force>
  std::vector<std::pair<unsigned, unsigned>> evaluate(const Force& force, std::vector<Vector>* deltas = nullptr) {
    apply_pair_law(force);
    apply_link_law(force);
    upload_if_dirty();
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

  // -- initialisers (subset of include/initializers) -------------------------
  // Uniform in a ball of the given radius (initializers/spheres.hpp's
  // random filled sphere; the stream is this library's own).
  void init_random_filled_sphere(Scalar radius) {
    std::mt19937_64 rng(settings_.seed);
    std::uniform_real_distribution<double> u(-1.0, 1.0);
    refresh_host();
    for (unsigned i = 0; i < agent_count; ++i) {
      double p[3] = {0, 0, 0}, r2;
      do {
        r2 = 0;
        for (int d = 0; d < dimensions; ++d) { p[d] = u(rng); r2 += p[d] * p[d]; }
      } while (r2 > 1.0);
      for (int d = 0; d < dimensions; ++d) positions_(i)[d] = static_cast<Scalar>(p[d] * radius);
    }
    host_dirty_ = true;
  }
  // Uniform on a sphere surface of the given radius (random hollow sphere).
  void init_random_hollow_sphere(Scalar radius) {
    std::mt19937_64 rng(settings_.seed);
    std::normal_distribution<double> g(0.0, 1.0);
    refresh_host();
    for (unsigned i = 0; i < agent_count; ++i) {
      double p[3] = {0, 0, 0}, r2 = 0;
      for (int d = 0; d < dimensions; ++d) { p[d] = g(rng); r2 += p[d] * p[d]; }
      const double s = radius / std::sqrt(r2);
      for (int d = 0; d < dimensions; ++d) positions_(i)[d] = static_cast<Scalar>(p[d] * s);
    }
    host_dirty_ = true;
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
  static Settings make_settings(unsigned n, const std::string& path, Scalar cutoff,
                                const typename PairFinder::Settings& pfs, std::uint64_t seed) {
    Settings s(n, path);
    s.cutoff_distance = cutoff;
    s.pair_finder_settings = pfs;
    s.seed = seed;
    return s;
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

  // the pairwise law of this step (none: pairs only, no deltas); user laws
  // (a PAIRWISE_FORCE law, a GENERIC_FORCE law, or both) replace the built-in
  // one until a step passes a built-in law again
  template <typename... Forces>
  void apply_pair_law(const Forces&... forces) {
    int id = TECS_FORCE_NONE;
    float k[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
    constexpr bool generic = (false || ... || detail::UserGenericLaw<Forces>);
    constexpr bool user_pair = (false || ... || detail::UserPairLaw<Forces>);
    constexpr bool user = generic || user_pair;
    auto one = [&](const auto& f) {
      using F = std::decay_t<decltype(f)>;
      if constexpr (!detail::UserPairLaw<F> && !detail::UserGenericLaw<F> && !detail::is_link_law<F>()) {
        static_assert(!user || sizeof(F) == 0,
                      "a GENERIC_FORCE law combines with a PAIRWISE_FORCE law, not a built-in one");
        static_assert(!F::needs_polarity || has_polarity, "this force needs a (Polarity, polarity) field");
        id = F::force_id;
        k[0] = f.k_rep; k[1] = f.r_rep; k[2] = f.k_adh; k[3] = f.r_adh; k[4] = f.k_pol_value();
      }
    };
    (one(forces), ...);
    if constexpr (user) {
      const auto& g = first_of<IsGeneric>(forces...);
      const auto& p = first_of<IsUserPair>(forces...);
      detail::PairLawBinding<Config, std::decay_t<decltype(g)>, std::decay_t<decltype(p)>>::bind(
          handle_, settings_.device, g, p, law_holder_, law_fn_);
    }
    if (!user && law_fn_) {
      check(tecs_sim_set_pair_law(handle_, nullptr, nullptr));
      law_holder_.reset();
      law_fn_ = nullptr;
    }
    check(tecs_sim_set_force(handle_, id, k[0], k[1], k[2], k[3], k[4]));
  }

  // the link law of this step: links act only in steps that pass one
  template <typename... Forces>
  void apply_link_law(const Forces&... forces) {
    bool has = false;
    float strength = 0.f;
    auto one = [&](const auto& f) {
      using F = std::decay_t<decltype(f)>;
      if constexpr (detail::is_link_law<F>()) {
        has = true;
        strength = f.strength;
      }
    };
    (one(forces), ...);
    const unsigned want = has ? links_.get_active_count() : 0u;
    if (!links_dirty_ && want == links_on_device_ && (!has || strength == link_strength_)) return;
    if (want > links_.extent(0)) throw Error("link active count exceeds link_capacity");
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

  template <typename Field>
  View<typename Field::value_type>& view_of() {
    if constexpr (is_position_field<Field>) {
      return positions_;
    } else {
      static_assert(has_polarity && is_polarity_field<Field>, "no such field in this config");
      return polarity_;
    }
  }

  template <typename... Ts>
  void write_all(double time, const View<Ts>&... extra) {
    refresh_host();
    const unsigned step = current_step++;
    if constexpr (has_polarity) writer_.write(time, step, positions_, polarity_, extra..., links_);
    else writer_.write(time, step, positions_, extra..., links_);
  }

  void refresh_host() {
    if (host_valid_) return;
    unsigned n = 0;
    check(tecs_sim_download(handle_, reinterpret_cast<float*>(positions_.data()),
                            has_polarity ? reinterpret_cast<float*>(polarity_.data()) : nullptr, &n));
    agent_count = n;
    positions_.set_active_count(n);
    if constexpr (has_polarity) polarity_.set_active_count(n);
    host_valid_ = true;
    host_dirty_ = false;
  }

  void upload_if_dirty() {
    if (!host_dirty_) return;
    check(tecs_sim_upload(handle_, reinterpret_cast<const float*>(positions_.data()),
                          has_polarity ? reinterpret_cast<const float*>(polarity_.data()) : nullptr, agent_count));
    host_dirty_ = false;
  }

  Settings settings_;
  Writer writer_;
  // the bound user pairwise law (its launcher and the law object it launches with); destroyed after handle_
  std::shared_ptr<void> law_holder_;
  tecs_pair_law_fn law_fn_ = nullptr;
  tecs_sim* handle_ = nullptr;
  View<Vector> positions_;
  View<Polarity> polarity_;
  View<Link> links_;
  bool links_dirty_ = false;        // the host links may differ from the device's
  unsigned links_on_device_ = 0;    // links active in the library
  float link_strength_ = 0.f;
  bool host_valid_ = false;  // the host mirror holds the device state
  bool host_dirty_ = false;  // the host mirror may differ from the device state
};

}  // namespace tecs

#endif  // TECS_CXX_SIMULATION_HPP
