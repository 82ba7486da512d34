// config_checks.cpp -- compile-time checks of the C++20 drop-in layer's
// config machinery and defaults against the reference's
// (include/simulation_config.hpp:356-372, include/pair_finders/*.hpp Settings,
// include/simulation.hpp:76-98).  Compiling this file is the test.
#include <type_traits>

#include "tecs/tecs.hpp"

using namespace tecs;

// the default config: 3-D float, NaiveAllPairs, NoComFixer, Heun, one position field
static_assert(DefaultSimulationConfig::dimensions == 3);
static_assert(std::is_same_v<DefaultSimulationConfig::Scalar, float>);
static_assert(DefaultSimulationConfig::PairFinderT<DefaultSimulationConfig>::finder_id == TECS_FINDER_NAIVE_ALL_PAIRS);
static_assert(DefaultSimulationConfig::IntegratorT<DefaultSimulationConfig>::integrator_id == TECS_HEUN);
static_assert(DefaultSimulationConfig::ComFixerT<DefaultSimulationConfig>::com_fix == 0);
static_assert(DefaultSimulationConfig::Fields::size == 1);

// overrides in any order before RESOLVE_TECS_CONFIG(); the field types follow the final dimensions
struct TwoD : public DefaultSimulationConfig {
  CONFIG_FIELDS((Vector, position))
  CONFIG_PAIR_FINDER(pair_finders::BinnedGabrielSymmetric)
  CONFIG_DIMENSIONS(2)
  RESOLVE_TECS_CONFIG()
};
static_assert(std::is_same_v<TwoD::Vector, VectorN<float, 2>>);
using TwoDFinder = TwoD::PairFinderT<TwoD>;
static_assert(TwoDFinder::symmetric && TwoDFinder::binned && TwoDFinder::gabriel);

CREATE_SIMULATION_CONFIG(Sheet, CONFIG_PAIR_FINDER(pair_finders::BinnedGabriel)
                                    CONFIG_COM_FIXER(com_fixers::GlobalComFixer)
                                    CONFIG_FIELDS((Vector, position), (Polarity, polarity)))
static_assert(Simulation<Sheet>::has_polarity);
static_assert(!Simulation<DefaultSimulationConfig>::has_polarity);
static_assert(Sheet::ComFixerT<Sheet>::com_fix == 1);

EXTRACT_ALL_FROM_SIMULATION_CONFIG(Sheet)
static_assert(std::is_same_v<PairFinder, pair_finders::BinnedGabriel<View<Vector>, float, 3>>);
static_assert(std::is_same_v<typename PairFinder::positions_view_type, View<Vector>>);

// Settings defaults: binned_gabriel.hpp:20-26, binned_all_pairs.hpp:20-25, naive_gabriel.hpp
constexpr PairFinder::Settings gabriel_defaults{};
static_assert(gabriel_defaults.gabriel_coefficient == 0.8f);
static_assert(gabriel_defaults.min_bounds == Vector(-20.0f) && gabriel_defaults.max_bounds == Vector(20.0f));
static_assert(gabriel_defaults.bin_size_scale == 1.0f && gabriel_defaults.rebuild_every_n == 0);
constexpr pair_finders::BinnedAllPairs<View<Vector>, float, 3>::Settings all_pairs_defaults{};
static_assert(all_pairs_defaults.min_bounds == Vector(-20.0f) && all_pairs_defaults.rebuild_every_n == 0);
static_assert(pair_finders::NaiveGabriel<View<Vector>, float, 3>::Settings{}.gabriel_coefficient == 0.8f);
static_assert(std::is_empty_v<pair_finders::NaiveDelaunay<View<Vector>, float, 3>::Settings>);

// the host value types match the C ABI's AoS layout
static_assert(sizeof(Vector) == 12 && sizeof(Polarity) == 8);
static_assert(Vector(1.0f, 2.0f, 2.0f).length_squared() == 9.0f);

int main() {
  // Simulation::Settings defaults (simulation.hpp:76-98)
  Simulation<Sheet>::Settings s(10, "out");
  return (s.capacity == 10 && s.cutoff_distance == 1'000'000.0f && s.seed == 2807) ? 0 : 1;
}
