// example_programs.cu -- five experiments of the reference's example programs
// (examples/springs.cpp, epithelium.cpp, polarization.cpp, growth_w_wall.cpp,
// delaunay_spheroid.cpp), set up with the same settings, initialisers, force
// laws, init and update functions, device values, steps and writes, through
// the drop-in layer's API.  tests/test_reference_examples.py runs each on a
// GB300 and compares the HDF5 output with the reference programs' own.
//
//   example_programs <springs|epithelium|polarization|growth_w_wall|delaunay_spheroid>
//
// writes ./output/<name>.h5 (and .xmf); the directory must exist.
#include <cstdio>
#include <cstring>
#include <string>

#include "tecs.hpp"

using namespace tecs;

namespace springs_run {
EXTRACT_TYPES_FROM_SIMULATION_CONFIG(DefaultSimulationConfig)
// 800 bodies in a ball of radius 3, all pairs joined by springs of rest length 0.5
int run() {
  const Scalar rest = 0.5f;
  Simulation<DefaultSimulationConfig> sim(800, "./output/springs");
  sim.init_random_filled_sphere(3.0);
  sim.write(0.0);
  auto law = PAIRWISE_FORCE(ctx.position.delta += forces::Spring(displacement, distance, rest););
  for (int k = 1; k <= 100; ++k) {
    sim.take_step(0.001, law());
    sim.write(k * 0.001);
  }
  return 0;
}
}  // namespace springs_run

CREATE_SIMULATION_CONFIG(PolarConfig, CONFIG_FIELDS((Vector, position), (Polarity, polarity)))

namespace epithelium_run {
EXTRACT_TYPES_FROM_SIMULATION_CONFIG(PolarConfig)
// 250 cells relaxed in a sphere, polarities pointing outward, then 101 steps of
// the piecewise-linear law with apical-basal bending
int run() {
  Simulation<PolarConfig> sim(250, "./output/epithelium", Scalar(1.0));
  auto& x = sim.get_view<FIELD(Vector, position)>();
  auto& p = sim.get_view<FIELD(Polarity, polarity)>();
  auto outward = INIT_FUNC(p(i) = Polarity(x(i)););
  sim.init_relaxed_sphere(0.8, outward());
  auto law = PAIRWISE_FORCE(
    ctx.position.delta += forces::PiecewiseLinear(displacement, distance, 0.7f, 0.8f, 1.0f);
    const auto bend = ctx.polarity.self.bending_force(displacement, ctx.polarity.other, distance);
    ctx.position.delta += bend.vector;
    ctx.polarity.delta += bend.polarity;);
  for (int k = 0; k <= 100; ++k) {
    sim.take_step(0.05, law());
    sim.write(k * 0.05);
  }
  return 0;
}
}  // namespace epithelium_run

namespace polarization_run {
EXTRACT_TYPES_FROM_SIMULATION_CONFIG(PolarConfig)
// 200 cells in a ball of radius 1.5 with random polarities, a two-radius
// polynomial law and bidirectional alignment, 300 steps
int run() {
  const Scalar far = 1.0f, near = 0.6f;
  Simulation<PolarConfig> sim(200, "./output/polarization", far);
  auto& p = sim.get_view<FIELD(Polarity, polarity)>();
  auto random_direction = INIT_FUNC(
    p(i) = Polarity{Kokkos::acos(2.0 * rng.drand(0.0, 1.0) - 1.0),
                    2.0 * Kokkos::numbers::pi_v<Scalar> * rng.drand(0.0, 1.0)};);
  sim.init_random_filled_sphere(1.5, random_direction());
  sim.write(0.0);
  auto law = PAIRWISE_FORCE(
    Scalar F = 2.0 * (near - distance) * (far - distance) + Kokkos::pow(far - distance, 2);
    ctx.position.delta += displacement * F / distance;
    ctx.polarity.delta += ctx.polarity.self.bidirectional_polarization_force(ctx.polarity.other););
  for (int k = 1; k <= 300; ++k) {
    sim.take_step(0.025, law());
    sim.write(k * 0.025);
  }
  return 0;
}
}  // namespace polarization_run

CREATE_SIMULATION_CONFIG(WallConfig, CONFIG_PAIR_FINDER(pair_finders::BinnedGabriel))

namespace growth_run {
EXTRACT_TYPES_FROM_SIMULATION_CONFIG(WallConfig)
// 500 cells above the wall z = 0, growing by random division (rate 0.005 per
// cell and step, daughter at 0.75 / 4 in a random direction) for 500 steps
// of the piecewise-linear law and the wall's push, a write every 5 steps
int run() {
  const Scalar spacing = 0.75f, rate = 0.005f;
  Plane wall(0.0f, 0.0f, 1.0f, 0.0f);
  Simulation<WallConfig> sim(10000, "./output/growth_w_wall", Scalar(1.0));
  sim.set_agent_count(500);
  auto& x = sim.get_view<FIELD(Vector, position)>();
  auto above = INIT_FUNC(if (x(i).z() < 0.0f) x(i).z() *= -1.0f;);
  sim.init_random_filled_sphere(3.0f, above());
  sim.write(0.0);
  auto law = PAIRWISE_FORCE(ctx.position.delta += forces::PiecewiseLinear(displacement, distance, 0.7f););
  auto push = GENERIC_FORCE(
    const Scalar sd = wall.signed_distance(ctx.position.self);
    if (sd < 0.0f) ctx.position.delta += wall.normal() * (-sd * 10.0f););
  DeviceVar<int> cells = sim.get_agent_count();
  auto divide = UPDATE_FUNC(
    if (rng.drand(0.0, 1.0) > rate) return;
    const int d = Kokkos::atomic_fetch_add(cells.data(), 1);
    // the reference passes both draws to one constructor call, whose argument
    // order the compiler picks; its build drew the second argument first
    const double u_phi = rng.drand(0.0, 1.0);
    const double u_theta = rng.drand(0.0, 1.0);
    const Polarity dir(Kokkos::acos(2.0 * u_theta - 1), u_phi * 2.0 * Kokkos::numbers::pi_v<Scalar>);
    x(d) = x(i) + spacing / 4 * dir.to_vector3(););
  for (int k = 1; k <= 500; ++k) {
    sim.take_step(0.1, law(), push());
    sim.init(divide());
    sim.set_agent_count(cells);
    if (k % 5 == 0) sim.write(k * 0.1);
  }
  return 0;
}
}  // namespace growth_run

CREATE_SIMULATION_CONFIG(DelaunayConfig, CONFIG_PAIR_FINDER(pair_finders::NaiveDelaunay))

namespace delaunay_run {
EXTRACT_TYPES_FROM_SIMULATION_CONFIG(DelaunayConfig)
// 100 cells in a ball of radius 3; the Delaunay pairs of the start recorded
// as links by a pairwise law, then 300 steps of a piecewise-linear law
int run() {
  const int n = 100;
  Simulation<DelaunayConfig>::Settings settings(n, "./output/delaunay_spheroid");
  settings.cutoff_distance = 1.0f;
  settings.link_capacity = n * n * n / 2;
  Simulation<DelaunayConfig> sim(settings);
  auto& links = sim.get_links();
  sim.init_random_filled_sphere(3.0);
  DeviceVar<int> recorded = links.get_active_count();
  auto record = PAIRWISE_FORCE(
    if (!is_full_step) return;
    const int k = Kokkos::atomic_fetch_add(recorded.data(), 1);
    links(k) = Link(i, j););
  sim.take_step(0.0, record);
  links.set_active_count(recorded);
  sim.write(0.0);
  auto law = PAIRWISE_FORCE(ctx.position.delta += forces::PiecewiseLinear(displacement, distance, 0.5f) * 3.0;);
  for (int k = 1; k <= 300; ++k) {
    sim.take_step(0.001, law());
    sim.write(k * 0.001);
  }
  return 0;
}
}  // namespace delaunay_run

int main(int argc, char** argv) {
  if (argc < 2) {
    std::fprintf(stderr, "usage: %s <experiment>\n", argv[0]);
    return 2;
  }
  const std::string name = argv[1];
  try {
    if (name == "springs") return springs_run::run();
    if (name == "epithelium") return epithelium_run::run();
    if (name == "polarization") return polarization_run::run();
    if (name == "growth_w_wall") return growth_run::run();
    if (name == "delaunay_spheroid") return delaunay_run::run();
  } catch (const std::exception& e) {
    std::fprintf(stderr, "%s: %s\n", name.c_str(), e.what());
    return 1;
  }
  std::fprintf(stderr, "unknown experiment %s\n", name.c_str());
  return 2;
}
