// ref_driver.cpp -- runs the TECS reference's own headers (compiled unmodified
// against oracle/kokkos_shim) on a raw input file and writes raw outputs.
// Used only to generate the golden vectors that pin the oracle
// (tests/golden/make_golden.py); never part of the product.
//
//   ref_driver <scenario> <in.bin> <out_prefix> <steps> <dt>
//
// in.bin: uint32 n, uint32 dims, uint32 has_polarity, float32 params[16],
//         float32 positions[n*dims], float32 polarity[n*2] (if present)
// params: cutoff, gabriel_c, min_x, min_y, min_z, max_x, max_y, max_z,
//         k_rep, r_rep, k_adh, r_adh, k_pol, capacity, bin_size_scale, spare
// outputs: <out>.pairs (uint32 pairs, evaluation order), <out>.dpos, <out>.dpol
//          (one full-step pass from a fresh finder), <out>.pos / <out>.pol
//          (state after <steps> take_step calls).
// Link scenarios (names starting "lk_") read, after the polarity block,
// uint32 n_links and uint32 links[2*n_links] (a, b), take the link strength
// from params[15], step with take_step(dt, link_force, pairwise_force) and
// write <out>.pos only.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

// the reference's umbrella include order (include/tecs.hpp:1-57) minus the CLI helper
#include <utils/utils.hpp>
#include <types/vector.hpp>
#include <types/polarity.hpp>
#include <types/plane.hpp>
#include <types/link.hpp>
#include <types/view.hpp>
#include <types/device_var.hpp>
#include <integrators/base.hpp>
#include <forces/detail.hpp>
#include <forces/kernel_fuser.hpp>
#include <simulation.hpp>
#include <pair_finders/binned_all_pairs.hpp>
#include <pair_finders/binned_all_pairs_symmetric.hpp>
#include <pair_finders/binned_gabriel.hpp>
#include <pair_finders/binned_gabriel_symmetric.hpp>
#include <pair_finders/naive_all_pairs.hpp>
#include <pair_finders/naive_all_pairs_symmetric.hpp>
#include <pair_finders/naive_gabriel.hpp>
#include <pair_finders/naive_gabriel_symmetric.hpp>
#include <pair_finders/naive_delaunay.hpp>
#include <integrators/euler.hpp>
#include <integrators/heun.hpp>
#include <com_fixers/com_fixers.hpp>
#include <io/dummy.hpp>
#include <io/hdf5_writer.hpp>
#include <forces/predefined.hpp>

struct Input {
  unsigned n = 0, dims = 0, has_pol = 0;
  float prm[16] = {};
  std::vector<float> x, p;
  std::vector<unsigned> links;
};

static Input read_input(const char* path, bool with_links) {
  Input in;
  FILE* f = std::fopen(path, "rb");
  if (!f) { std::perror(path); std::exit(2); }
  unsigned hdr[3];
  if (std::fread(hdr, 4, 3, f) != 3) std::exit(2);
  in.n = hdr[0]; in.dims = hdr[1]; in.has_pol = hdr[2];
  if (std::fread(in.prm, 4, 16, f) != 16) std::exit(2);
  in.x.resize((size_t)in.n * in.dims);
  if (in.n && std::fread(in.x.data(), 4, in.x.size(), f) != in.x.size()) std::exit(2);
  if (in.has_pol) {
    in.p.resize((size_t)in.n * 2);
    if (in.n && std::fread(in.p.data(), 4, in.p.size(), f) != in.p.size()) std::exit(2);
  }
  if (with_links) {
    unsigned nl = 0;
    if (std::fread(&nl, 4, 1, f) != 1) std::exit(2);
    in.links.resize((size_t)nl * 2);
    if (nl && std::fread(in.links.data(), 4, in.links.size(), f) != in.links.size()) std::exit(2);
  }
  std::fclose(f);
  return in;
}

static void write_raw(const std::string& path, const void* data, size_t bytes) {
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) { std::perror(path.c_str()); std::exit(2); }
  if (bytes) std::fwrite(data, 1, bytes, f);
  std::fclose(f);
}

// --- force laws, written as user PAIRWISE_FORCE lambdas -------------------
// spring2r: F(d) = k_rep*max(r_rep-d,0) - k_adh*max(d-r_adh,0), zero at d == 0
#define TECS_DRIVER_SPRING                                                                              \
  if (capture) {                                                                                        \
    const int slot = Kokkos::atomic_fetch_add(counter.data(), 1);                                       \
    pairs(2 * slot) = i;                                                                                \
    pairs(2 * slot + 1) = j;                                                                            \
  }                                                                                                     \
  if (distance != Scalar(0)) {                                                                          \
    const Scalar F = k_rep * Kokkos::fmax(r_rep - distance, Scalar(0)) -                                \
                     k_adh * Kokkos::fmax(distance - r_adh, Scalar(0));                                 \
    ctx.position.delta += displacement * F / distance;                                                 \
  }

// polarity: spring2r + k_pol * (bending_force + bidirectional_polarization_force)
#define TECS_DRIVER_POLARITY                                                                            \
  TECS_DRIVER_SPRING                                                                                    \
  auto bend = ctx.polarity.self.bending_force(displacement, ctx.polarity.other, distance);             \
  ctx.position.delta += bend.vector * k_pol;                                                            \
  ctx.polarity.delta += bend.polarity * k_pol;                                                          \
  ctx.polarity.delta += ctx.polarity.self.bidirectional_polarization_force(ctx.polarity.other) * k_pol;

// --- one scenario per (finder, integrator, com fixer, fields, dims) -------
#define TECS_SCENARIO(NAME, FINDER, INTEGRATOR, COMFIXER, DIMS, POLAR)                                    \
  namespace NAME {                                                                                      \
  CREATE_SIMULATION_CONFIG(Config, CONFIG_PAIR_FINDER(FINDER) CONFIG_INTEGRATOR(INTEGRATOR)             \
                                       CONFIG_COM_FIXER(COMFIXER) CONFIG_DIMENSIONS(DIMS)                \
                                           CONFIG_WRITER(tecs::io::Dummy) TECS_FIELDS_##POLAR)           \
  EXTRACT_ALL_FROM_SIMULATION_CONFIG(Config)                                                            \
  static int run(const Input& in, const std::string& out, int steps, double dt) {                       \
    return tecs_driver_run<Config, PairFinder, Scalar, Vector, Random, PairwiseForceFields, POLAR>(     \
        in, out, steps, dt);                                                                            \
  }                                                                                                     \
  }

#define TECS_FIELDS_0 CONFIG_FIELDS((Vector, position))
#define TECS_FIELDS_1 CONFIG_FIELDS((Vector, position), (Polarity, polarity))

template <class Sim, class Settings>
static void fill_settings(Settings& s, const Input& in) {
  s.cutoff_distance = in.prm[0];
  s.capacity = (unsigned)in.prm[13] > in.n ? (unsigned)in.prm[13] : in.n;
}

template <class PFS>
static void fill_finder_settings(PFS& pfs, const Input& in) {
  if constexpr (requires { pfs.gabriel_coefficient; }) pfs.gabriel_coefficient = in.prm[1];
  if constexpr (requires { pfs.min_bounds; }) {
    for (unsigned d = 0; d < in.dims; ++d) {
      pfs.min_bounds[d] = in.prm[2 + d];
      pfs.max_bounds[d] = in.prm[5 + d];
    }
  }
  if constexpr (requires { pfs.bin_size_scale; }) pfs.bin_size_scale = in.prm[14];
}

template <class Config, class PairFinder, class Scalar, class Vector, class Random, class PairwiseForceFields,
          int POLAR>
static int tecs_driver_run(const Input& in, const std::string& out, int steps, double dt) {
  using namespace tecs;
  const Scalar k_rep = in.prm[8], r_rep = in.prm[9], k_adh = in.prm[10], r_adh = in.prm[11], k_pol = in.prm[12];
  (void)k_pol;
  const unsigned n = in.n;
  // the Delaunay finder applies a pair once per accepted triangle/tetrahedron
  const size_t per_cell = n <= 256 ? (size_t)n * n : (n < 4096 ? n : 64);
  Kokkos::View<unsigned*> pairs("pairs", 2 * (size_t)n * per_cell + 2);
  DeviceVar<int> counter = 0;
  bool capture = true;

  auto make_force = [&]() {
    if constexpr (POLAR) {
      return PAIRWISE_FORCE(TECS_DRIVER_POLARITY)();
    } else {
      return PAIRWISE_FORCE(TECS_DRIVER_SPRING)();
    }
  };

  // (1) one full-step pass with a fresh finder: PairFinder::evaluate_force
  {
    typename PairFinder::Settings pfs{};
    fill_finder_settings(pfs, in);
    PairFinder finder(n, in.prm[0], pfs);
    using PV = Kokkos::View<Vector*>;
    PV x("position", n), dx("position", n), vold("old_velocities", n);
    for (unsigned i = 0; i < n; ++i)
      for (unsigned d = 0; d < in.dims; ++d) x(i)[d] = in.x[(size_t)i * in.dims + d];
    Kokkos::Random_XorShift64_Pool<> pool(2807);
    auto force = make_force();
    if constexpr (POLAR) {
      using PolV = Kokkos::View<Polarity_<Scalar>*>;
      PolV p("polarity", n), dp("polarity", n);
      for (unsigned i = 0; i < n; ++i) { p(i)[0] = in.p[2 * i]; p(i)[1] = in.p[2 * i + 1]; }
      detail::ViewPack<PV, PolV> ip(x, p), op(dx, dp);
      finder.template evaluate_force<decltype(pool), decltype(force.force), PairwiseForceFields>(ip, op, vold, pool,
                                                                                                force.force, true);
      write_raw(out + ".dpol", dp.data(), (size_t)n * 8);
    } else {
      detail::ViewPack<PV> ip(x), op(dx);
      finder.template evaluate_force<decltype(pool), decltype(force.force), PairwiseForceFields>(ip, op, vold, pool,
                                                                                                force.force, true);
    }
    std::vector<float> flat((size_t)n * in.dims);
    for (unsigned i = 0; i < n; ++i)
      for (unsigned d = 0; d < in.dims; ++d) flat[(size_t)i * in.dims + d] = dx(i)[d];
    write_raw(out + ".dpos", flat.data(), flat.size() * 4);
    const int np = counter;
    write_raw(out + ".pairs", pairs.data(), (size_t)np * 8);
  }

  // (2) Simulation::take_step, steps times
  capture = false;
  {
    typename Simulation<Config>::Settings st(n, "unused");
    fill_settings<Simulation<Config>>(st, in);
    fill_finder_settings(st.pair_finder_settings, in);
    Simulation<Config> sim(st);
    auto& pos = sim.template get_view<FIELD(Vector, position)>();
    for (unsigned i = 0; i < n; ++i)
      for (unsigned d = 0; d < in.dims; ++d) pos(i)[d] = in.x[(size_t)i * in.dims + d];
    if constexpr (POLAR) {
      auto& pol = sim.template get_view<FIELD(Polarity_<Scalar>, polarity)>();
      for (unsigned i = 0; i < n; ++i) { pol(i)[0] = in.p[2 * i]; pol(i)[1] = in.p[2 * i + 1]; }
    }
    auto force = make_force();
    for (int s = 0; s < steps; ++s) sim.take_step(dt, force);
    std::vector<float> flat((size_t)n * in.dims);
    for (unsigned i = 0; i < n; ++i)
      for (unsigned d = 0; d < in.dims; ++d) flat[(size_t)i * in.dims + d] = pos(i)[d];
    write_raw(out + ".pos", flat.data(), flat.size() * 4);
    if constexpr (POLAR) {
      auto& pol = sim.template get_view<FIELD(Polarity_<Scalar>, polarity)>();
      std::vector<float> pf((size_t)n * 2);
      for (unsigned i = 0; i < n; ++i) { pf[2 * i] = pol(i)[0]; pf[2 * i + 1] = pol(i)[1]; }
      write_raw(out + ".pol", pf.data(), pf.size() * 4);
    }
  }
  return 0;
}

// Link scenarios: the protrusion law of examples/intercalation.cpp:65-71
// (constant pull of strength k along the link) with the spring pairwise law.
template <class Config, class Scalar, class Vector, class Random, class PairwiseForceFields, class LinkForceFields>
static int tecs_driver_run_links(const Input& in, const std::string& out, int steps, double dt) {
  using namespace tecs;
  const Scalar k_rep = in.prm[8], r_rep = in.prm[9], k_adh = in.prm[10], r_adh = in.prm[11];
  const Scalar k_link = in.prm[15];
  const unsigned n = in.n;
  Kokkos::View<unsigned*> pairs("pairs", 2);
  DeviceVar<int> counter = 0;
  const bool capture = false;
  auto make_force = [&]() { return PAIRWISE_FORCE(TECS_DRIVER_SPRING)(); };
  auto make_link_force = LINK_FORCE(
    Vector displacement = ctx.position.b - ctx.position.a;
    Scalar distance = displacement.length();
    ctx.position.delta_a += k_link * displacement / distance;
    ctx.position.delta_b += -k_link * displacement / distance;
  );
  typename Simulation<Config>::Settings st(n, "unused");
  fill_settings<Simulation<Config>>(st, in);
  fill_finder_settings(st.pair_finder_settings, in);
  const unsigned nl = (unsigned)(in.links.size() / 2);
  st.link_capacity = nl ? nl : 1;
  st.link_active_count = nl;
  Simulation<Config> sim(st);
  auto& pos = sim.template get_view<FIELD(Vector, position)>();
  for (unsigned i = 0; i < n; ++i)
    for (unsigned d = 0; d < in.dims; ++d) pos(i)[d] = in.x[(size_t)i * in.dims + d];
  auto& links = sim.get_links();
  for (unsigned l = 0; l < nl; ++l) links(l) = Link{in.links[2 * l], in.links[2 * l + 1]};
  auto force = make_force();
  auto link_force = make_link_force();
  for (int s = 0; s < steps; ++s) sim.take_step(dt, link_force, force);
  std::vector<float> flat((size_t)n * in.dims);
  for (unsigned i = 0; i < n; ++i)
    for (unsigned d = 0; d < in.dims; ++d) flat[(size_t)i * in.dims + d] = pos(i)[d];
  write_raw(out + ".pos", flat.data(), flat.size() * 4);
  return 0;
}

// Generic-force scenarios: a GENERIC_FORCE law (a pull towards the origin on
// full steps, a constant push on Heun's second evaluation) with the spring
// pairwise law, passed pairwise first: the reference evaluates the generic
// force first (kernel_fuser.hpp:148-156).  Writes <out>.pos only.
template <class Config, class Scalar, class Vector, class Random, class PairwiseForceFields, class GenericForceFields>
static int tecs_driver_run_generic(const Input& in, const std::string& out, int steps, double dt) {
  using namespace tecs;
  const Scalar k_rep = in.prm[8], r_rep = in.prm[9], k_adh = in.prm[10], r_adh = in.prm[11];
  const unsigned n = in.n;
  Kokkos::View<unsigned*> pairs("pairs", 2);
  DeviceVar<int> counter = 0;
  const bool capture = false;
  auto make_force = [&]() { return PAIRWISE_FORCE(TECS_DRIVER_SPRING)(); };
  auto make_generic = GENERIC_FORCE(
    if (is_full_step) ctx.position.delta += ctx.position.self * Scalar(-0.02);
    else ctx.position.delta += Vector(Scalar(0.001));
  );
  typename Simulation<Config>::Settings st(n, "unused");
  fill_settings<Simulation<Config>>(st, in);
  fill_finder_settings(st.pair_finder_settings, in);
  Simulation<Config> sim(st);
  auto& pos = sim.template get_view<FIELD(Vector, position)>();
  for (unsigned i = 0; i < n; ++i)
    for (unsigned d = 0; d < in.dims; ++d) pos(i)[d] = in.x[(size_t)i * in.dims + d];
  auto force = make_force();
  auto generic = make_generic();
  for (int s = 0; s < steps; ++s) sim.take_step(dt, force, generic);
  std::vector<float> flat((size_t)n * in.dims);
  for (unsigned i = 0; i < n; ++i)
    for (unsigned d = 0; d < in.dims; ++d) flat[(size_t)i * in.dims + d] = pos(i)[d];
  write_raw(out + ".pos", flat.data(), flat.size() * 4);
  return 0;
}

// A pairwise law that sets drag (the spring plus drag = 0.5 * max(1.2 - d, 0)
// + 0.1): the reference's finders add sum(drag * old velocity of j) /
// max(sum(drag), eps) to each cell's position delta, and its integrators
// write the old velocities every step.  Outputs <out>.pos and <out>.ov (the
// old velocities after the last step).
template <class Config, class Scalar, class Vector, class Random, class PairwiseForceFields>
static int tecs_driver_run_drag(const Input& in, const std::string& out, int steps, double dt) {
  using namespace tecs;
  const Scalar k_rep = in.prm[8], r_rep = in.prm[9], k_adh = in.prm[10], r_adh = in.prm[11];
  const unsigned n = in.n;
  Kokkos::View<unsigned*> pairs("pairs", 2);
  DeviceVar<int> counter = 0;
  const bool capture = false;
  auto make_force = [&]() {
    return PAIRWISE_FORCE(TECS_DRIVER_SPRING drag = Scalar(0.5) * Kokkos::fmax(Scalar(1.2) - distance, Scalar(0)) +
                                                    Scalar(0.1);)();
  };
  typename Simulation<Config>::Settings st(n, "unused");
  fill_settings<Simulation<Config>>(st, in);
  fill_finder_settings(st.pair_finder_settings, in);
  Simulation<Config> sim(st);
  auto& pos = sim.template get_view<FIELD(Vector, position)>();
  for (unsigned i = 0; i < n; ++i)
    for (unsigned d = 0; d < in.dims; ++d) pos(i)[d] = in.x[(size_t)i * in.dims + d];
  auto force = make_force();
  for (int s = 0; s < steps; ++s) sim.take_step(dt, force);
  std::vector<float> flat((size_t)n * in.dims), ov((size_t)n * in.dims);
  auto old = sim.get_old_velocities_view_from_integrator();
  for (unsigned i = 0; i < n; ++i)
    for (unsigned d = 0; d < in.dims; ++d) {
      flat[(size_t)i * in.dims + d] = pos(i)[d];
      ov[(size_t)i * in.dims + d] = old(i)[d];
    }
  write_raw(out + ".pos", flat.data(), flat.size() * 4);
  write_raw(out + ".ov", ov.data(), ov.size() * 4);
  return 0;
}

// Update functions between steps, as the reference's growth and protrusion
// programs run them: Simulation::run with two UPDATE_FUNC functions (fused per
// cell, one generator), run_links with one that rewires every link, and an
// INIT_FUNC through init; then the steps.  Outputs <out>.pos, <out>.links
// (uint32 pairs) and <out>.hits (int32: a DeviceVar counter the functions add to).
template <class Config, class Scalar, class Vector, class Random, class PairwiseForceFields>
static int tecs_driver_run_update(const Input& in, const std::string& out, int steps, double dt) {
  using namespace tecs;
  const Scalar k_rep = in.prm[8], r_rep = in.prm[9], k_adh = in.prm[10], r_adh = in.prm[11];
  const unsigned n = in.n;
  Kokkos::View<unsigned*> pairs("pairs", 2);
  DeviceVar<int> counter = 0;
  const bool capture = false;
  auto make_force = [&]() { return PAIRWISE_FORCE(TECS_DRIVER_SPRING)(); };
  typename Simulation<Config>::Settings st(n, "unused");
  fill_settings<Simulation<Config>>(st, in);
  fill_finder_settings(st.pair_finder_settings, in);
  st.link_capacity = n;
  st.link_active_count = n;
  Simulation<Config> sim(st);
  auto& pos = sim.template get_view<FIELD(Vector, position)>();
  for (unsigned i = 0; i < n; ++i)
    for (unsigned d = 0; d < in.dims; ++d) pos(i)[d] = in.x[(size_t)i * in.dims + d];
  auto& links = sim.get_links();
  DeviceVar<int> hits = 0;
  auto nudge_x = UPDATE_FUNC(pos(i)[0] += Scalar(0.01) * Scalar(rng.drand(-1.0, 1.0)););
  auto nudge_y = UPDATE_FUNC(
    pos(i)[1] += Scalar(0.01) * Scalar(rng.drand(-1.0, 1.0));
    if (rng.drand(0.0, 1.0) < 0.1) Kokkos::atomic_fetch_add(hits.data(), 1););
  auto rewire = UPDATE_FUNC(links(i) = Link{i, (unsigned)rng.urand(n)};);
  auto lift = INIT_FUNC(pos(i)[2] += Scalar(0.001) * Scalar(rng.frand(0.0f, 1.0f)););
  sim.run(nudge_x(), nudge_y());
  sim.run_links(rewire());
  sim.init(lift());
  auto force = make_force();
  for (int s = 0; s < steps; ++s) sim.take_step(dt, force);
  std::vector<float> flat((size_t)n * in.dims);
  for (unsigned i = 0; i < n; ++i)
    for (unsigned d = 0; d < in.dims; ++d) flat[(size_t)i * in.dims + d] = pos(i)[d];
  std::vector<unsigned> lk(2 * (size_t)n);
  for (unsigned l = 0; l < n; ++l) {
    lk[2 * l] = links(l).a;
    lk[2 * l + 1] = links(l).b;
  }
  const int h = hits;
  write_raw(out + ".pos", flat.data(), flat.size() * 4);
  write_raw(out + ".links", lk.data(), lk.size() * 4);
  write_raw(out + ".hits", &h, 4);
  return 0;
}

namespace upd_bg_heun_3 {
using namespace tecs;
CREATE_SIMULATION_CONFIG(Config, CONFIG_PAIR_FINDER(pair_finders::BinnedGabriel) CONFIG_INTEGRATOR(integrators::Heun)
                                     CONFIG_WRITER(tecs::io::Dummy) TECS_FIELDS_0)
EXTRACT_ALL_FROM_SIMULATION_CONFIG(Config)
static int run(const Input& in, const std::string& out, int steps, double dt) {
  return tecs_driver_run_update<Config, Scalar, Vector, Random, PairwiseForceFields>(in, out, steps, dt);
}
}  // namespace upd_bg_heun_3

// A config with fields beyond the position: a Scalar u and a Vector w.  The
// pairwise law diffuses u and w between neighbours and drives w along the
// displacement; the generic law adds to u from the position; every field is
// integrated by the reference's integrators (a Scalar field in double).
// Outputs <out>.pos, <out>.u, <out>.w.
template <class Config, class Scalar, class Vector, class Random, class PairwiseForceFields, class GenericForceFields>
static int tecs_driver_run_fields(const Input& in, const std::string& out, int steps, double dt) {
  using namespace tecs;
  const Scalar k_rep = in.prm[8], r_rep = in.prm[9], k_adh = in.prm[10], r_adh = in.prm[11];
  const unsigned n = in.n;
  Kokkos::View<unsigned*> pairs("pairs", 2);
  DeviceVar<int> counter = 0;
  const bool capture = false;
  auto make_force = [&]() {
    return PAIRWISE_FORCE(TECS_DRIVER_SPRING
                          ctx.u.delta += (ctx.u.other - ctx.u.self) * Scalar(0.2);
                          ctx.w.delta += (ctx.w.other - ctx.w.self) * Scalar(0.1) + displacement * Scalar(0.01);)();
  };
  auto make_generic = GENERIC_FORCE(ctx.u.delta += Scalar(0.05) * ctx.position.self[0];);
  typename Simulation<Config>::Settings st(n, "unused");
  fill_settings<Simulation<Config>>(st, in);
  fill_finder_settings(st.pair_finder_settings, in);
  Simulation<Config> sim(st);
  auto& pos = sim.template get_view<FIELD(Vector, position)>();
  auto& u = sim.template get_view<FIELD(Scalar, u)>();
  auto& w = sim.template get_view<FIELD(Vector, w)>();
  for (unsigned i = 0; i < n; ++i) {
    for (unsigned d = 0; d < in.dims; ++d) pos(i)[d] = in.x[(size_t)i * in.dims + d];
    u(i) = pos(i)[0] * Scalar(0.3) + Scalar(1);
    w(i) = pos(i) * Scalar(0.5);
  }
  auto force = make_force();
  auto generic = make_generic();
  for (int s = 0; s < steps; ++s) sim.take_step(dt, force, generic);
  std::vector<float> fp((size_t)n * in.dims), fu(n), fw((size_t)n * in.dims);
  for (unsigned i = 0; i < n; ++i) {
    fu[i] = u(i);
    for (unsigned d = 0; d < in.dims; ++d) {
      fp[(size_t)i * in.dims + d] = pos(i)[d];
      fw[(size_t)i * in.dims + d] = w(i)[d];
    }
  }
  write_raw(out + ".pos", fp.data(), fp.size() * 4);
  write_raw(out + ".u", fu.data(), fu.size() * 4);
  write_raw(out + ".w", fw.data(), fw.size() * 4);
  return 0;
}

#define TECS_FIELDS_SCENARIO(NAME, FINDER, INTEGRATOR, COMFIXER)                                         \
  namespace NAME {                                                                                      \
  CREATE_SIMULATION_CONFIG(Config, CONFIG_PAIR_FINDER(FINDER) CONFIG_INTEGRATOR(INTEGRATOR)             \
                                       CONFIG_COM_FIXER(COMFIXER) CONFIG_WRITER(tecs::io::Dummy)        \
                                           CONFIG_FIELDS((Vector, position), (Scalar, u), (Vector, w)))  \
  EXTRACT_ALL_FROM_SIMULATION_CONFIG(Config)                                                            \
  static int run(const Input& in, const std::string& out, int steps, double dt) {                       \
    return tecs_driver_run_fields<Config, Scalar, Vector, Random, PairwiseForceFields, GenericForceFields>( \
        in, out, steps, dt);                                                                            \
  }                                                                                                     \
  }

#define TECS_DRAG_SCENARIO(NAME, FINDER, INTEGRATOR, COMFIXER)                                          \
  namespace NAME {                                                                                      \
  CREATE_SIMULATION_CONFIG(Config, CONFIG_PAIR_FINDER(FINDER) CONFIG_INTEGRATOR(INTEGRATOR)             \
                                       CONFIG_COM_FIXER(COMFIXER) CONFIG_WRITER(tecs::io::Dummy)        \
                                           TECS_FIELDS_0)                                                \
  EXTRACT_ALL_FROM_SIMULATION_CONFIG(Config)                                                            \
  static int run(const Input& in, const std::string& out, int steps, double dt) {                       \
    return tecs_driver_run_drag<Config, Scalar, Vector, Random, PairwiseForceFields>(in, out, steps, dt); \
  }                                                                                                     \
  }

// The reference's writer on a stepped simulation: write_static, write(0), then
// take_step + write(); its XDMF sidecar <out>.xmf is the output (the HDF5
// calls go to the HighFive stand-in and write nothing).
template <class Config, class Scalar, class Vector, class Random, class PairwiseForceFields>
static int tecs_driver_run_writer(const Input& in, const std::string& out, int steps, double dt) {
  using namespace tecs;
  const Scalar k_rep = in.prm[8], r_rep = in.prm[9], k_adh = in.prm[10], r_adh = in.prm[11];
  const unsigned n = in.n;
  Kokkos::View<unsigned*> pairs("pairs", 2);
  DeviceVar<int> counter = 0;
  const bool capture = false;
  auto make_force = [&]() { return PAIRWISE_FORCE(TECS_DRIVER_SPRING)(); };
  typename Simulation<Config>::Settings st(n, out);
  fill_settings<Simulation<Config>>(st, in);
  fill_finder_settings(st.pair_finder_settings, in);
  const unsigned nl = (unsigned)(in.links.size() / 2);
  st.link_capacity = nl;
  st.link_active_count = nl;
  Simulation<Config> sim(st);
  auto& pos = sim.template get_view<FIELD(Vector, position)>();
  for (unsigned i = 0; i < n; ++i)
    for (unsigned d = 0; d < in.dims; ++d) pos(i)[d] = in.x[(size_t)i * in.dims + d];
  auto& pol = sim.template get_view<FIELD(Polarity_<Scalar>, polarity)>();
  for (unsigned i = 0; i < n; ++i) { pol(i)[0] = in.p[2 * i]; pol(i)[1] = in.p[2 * i + 1]; }
  auto& links = sim.get_links();
  for (unsigned l = 0; l < nl; ++l) links(l) = Link{in.links[2 * l], in.links[2 * l + 1]};
  View<float> cell_type("cell_type", n);
  for (unsigned i = 0; i < n; ++i) cell_type(i) = (float)(i % 3);
  sim.write_static(cell_type);
  sim.write(0.0);
  auto force = make_force();
  for (int s = 0; s < steps; ++s) {
    sim.take_step(dt, force);
    sim.write();
  }
  return 0;
}

#define TECS_LINK_SCENARIO(NAME, FINDER, INTEGRATOR, COMFIXER)                                           \
  namespace NAME {                                                                                      \
  CREATE_SIMULATION_CONFIG(Config, CONFIG_PAIR_FINDER(FINDER) CONFIG_INTEGRATOR(INTEGRATOR)             \
                                       CONFIG_COM_FIXER(COMFIXER) CONFIG_WRITER(tecs::io::Dummy)         \
                                           TECS_FIELDS_0)                                                \
  EXTRACT_ALL_FROM_SIMULATION_CONFIG(Config)                                                            \
  static int run(const Input& in, const std::string& out, int steps, double dt) {                       \
    return tecs_driver_run_links<Config, Scalar, Vector, Random, PairwiseForceFields, LinkForceFields>(  \
        in, out, steps, dt);                                                                            \
  }                                                                                                     \
  }

using namespace tecs;
TECS_SCENARIO(ba_euler_3, pair_finders::BinnedAllPairs, integrators::Euler, com_fixers::NoComFixer, 3, 0)
TECS_SCENARIO(ba_heun_com_3, pair_finders::BinnedAllPairs, integrators::Heun, com_fixers::GlobalComFixer, 3, 0)
TECS_SCENARIO(bg_heun_3, pair_finders::BinnedGabriel, integrators::Heun, com_fixers::NoComFixer, 3, 0)
TECS_SCENARIO(bg_heun_com_3, pair_finders::BinnedGabriel, integrators::Heun, com_fixers::GlobalComFixer, 3, 0)
TECS_SCENARIO(bg_euler_com_3, pair_finders::BinnedGabriel, integrators::Euler, com_fixers::GlobalComFixer, 3, 0)
TECS_SCENARIO(na_heun_3, pair_finders::NaiveAllPairs, integrators::Heun, com_fixers::NoComFixer, 3, 0)
TECS_SCENARIO(ng_heun_3, pair_finders::NaiveGabriel, integrators::Heun, com_fixers::NoComFixer, 3, 0)
TECS_SCENARIO(bgs_euler_com_3, pair_finders::BinnedGabrielSymmetric, integrators::Euler, com_fixers::GlobalComFixer,
              3, 0)
TECS_SCENARIO(bas_heun_3, pair_finders::BinnedAllPairsSymmetric, integrators::Heun, com_fixers::NoComFixer, 3, 0)
TECS_SCENARIO(ngs_euler_3, pair_finders::NaiveGabrielSymmetric, integrators::Euler, com_fixers::NoComFixer, 3, 0)
TECS_SCENARIO(nas_heun_3, pair_finders::NaiveAllPairsSymmetric, integrators::Heun, com_fixers::NoComFixer, 3, 0)
TECS_SCENARIO(bg_heun_pol_3, pair_finders::BinnedGabriel, integrators::Heun, com_fixers::NoComFixer, 3, 1)
TECS_SCENARIO(ng_euler_2, pair_finders::NaiveGabriel, integrators::Euler, com_fixers::NoComFixer, 2, 0)
TECS_SCENARIO(bg_heun_2, pair_finders::BinnedGabriel, integrators::Heun, com_fixers::NoComFixer, 2, 0)
TECS_SCENARIO(nd_euler_2, pair_finders::NaiveDelaunay, integrators::Euler, com_fixers::NoComFixer, 2, 0)
TECS_SCENARIO(nd_heun_3, pair_finders::NaiveDelaunay, integrators::Heun, com_fixers::NoComFixer, 3, 0)
TECS_LINK_SCENARIO(lk_bg_heun_3, pair_finders::BinnedGabriel, integrators::Heun, com_fixers::NoComFixer)
namespace lk_writer_3 {
CREATE_SIMULATION_CONFIG(Config, CONFIG_PAIR_FINDER(pair_finders::BinnedGabriel) CONFIG_INTEGRATOR(integrators::Heun)
                                     CONFIG_WRITER(tecs::io::HDF5_Writer) TECS_FIELDS_1)
EXTRACT_ALL_FROM_SIMULATION_CONFIG(Config)
static int run(const Input& in, const std::string& out, int steps, double dt) {
  return tecs_driver_run_writer<Config, Scalar, Vector, Random, PairwiseForceFields>(in, out, steps, dt);
}
}  // namespace lk_writer_3
TECS_LINK_SCENARIO(lk_ba_euler_com_3, pair_finders::BinnedAllPairs, integrators::Euler, com_fixers::GlobalComFixer)
namespace gen_bg_heun_3 {
CREATE_SIMULATION_CONFIG(Config, CONFIG_PAIR_FINDER(pair_finders::BinnedGabriel) CONFIG_INTEGRATOR(integrators::Heun)
                                     CONFIG_WRITER(tecs::io::Dummy) TECS_FIELDS_0)
EXTRACT_ALL_FROM_SIMULATION_CONFIG(Config)
static int run(const Input& in, const std::string& out, int steps, double dt) {
  return tecs_driver_run_generic<Config, Scalar, Vector, Random, PairwiseForceFields, GenericForceFields>(in, out,
                                                                                                        steps, dt);
}
}  // namespace gen_bg_heun_3

TECS_DRAG_SCENARIO(drag_bg_heun_3, pair_finders::BinnedGabriel, integrators::Heun, com_fixers::NoComFixer)
TECS_FIELDS_SCENARIO(fields_bg_heun_3, pair_finders::BinnedGabriel, integrators::Heun, com_fixers::NoComFixer)
TECS_FIELDS_SCENARIO(fields_ba_euler_com_3, pair_finders::BinnedAllPairs, integrators::Euler,
                     com_fixers::GlobalComFixer)
TECS_DRAG_SCENARIO(drag_ba_euler_com_3, pair_finders::BinnedAllPairs, integrators::Euler, com_fixers::GlobalComFixer)

// Grid-query scenarios (names starting "grid_"): the reference's standalone
// acceleration::Grid (utils/grid.hpp:29-638) over the input points, with bins
// of params[0] over [params[2..4], params[5..7]), rebuilt once, then queried
// at m points read after the positions (uint32 m, float32 q[m*dims], uint32
// draws[m]).  The random pickers draw from a stub generator whose rand(a, b)
// and urand(r) return a + draw % (b - a) and draw % r, so the draw decides the
// target exactly.  Outputs (int32[m] each): <out>.near1 / .near2 (nearest
// point, search radius 1 / 2 bins), .rbins (random point in the 3^d bins),
// .rrad (random point within params[1]), .rfilt (the same among indices not
// divisible by 3).
struct DrawRng {
  unsigned draw = 0;
  int rand(int a, int b) const { return b > a ? a + (int)(draw % (unsigned)(b - a)) : a; }
  unsigned urand(unsigned r) const { return r ? draw % r : 0u; }
};

template <int DIMS>
static int run_grid(const char* path, const std::string& out) {
  using Vector = tecs::VectorN<float, DIMS>;
  FILE* f = std::fopen(path, "rb");
  if (!f) return 2;
  unsigned hdr[3];
  float prm[16];
  if (std::fread(hdr, 4, 3, f) != 3 || std::fread(prm, 4, 16, f) != 16) return 2;
  const unsigned n = hdr[0];
  std::vector<float> x((size_t)n * DIMS);
  if (n && std::fread(x.data(), 4, x.size(), f) != x.size()) return 2;
  unsigned m = 0;
  if (std::fread(&m, 4, 1, f) != 1) return 2;
  std::vector<float> q((size_t)m * DIMS);
  std::vector<unsigned> draws(m);
  if (m && (std::fread(q.data(), 4, q.size(), f) != q.size() || std::fread(draws.data(), 4, m, f) != m)) return 2;
  std::fclose(f);
  tecs::View<Vector> pts("points", n);
  for (unsigned i = 0; i < n; ++i)
    for (int d = 0; d < DIMS; ++d) pts(i)[d] = x[(size_t)i * DIMS + d];
  Vector mn, mx;
  for (int d = 0; d < DIMS; ++d) { mn[d] = prm[2 + d]; mx[d] = prm[5 + d]; }
  tecs::acceleration::Grid<Vector> grid(pts, n, mn, mx, prm[0]);
  grid.rebuild();
  std::vector<int> near1(m), near2(m), rbins(m), rrad(m), rfilt(m);
  for (unsigned k = 0; k < m; ++k) {
    Vector p;
    for (int d = 0; d < DIMS; ++d) p[d] = q[(size_t)k * DIMS + d];
    DrawRng rng{draws[k]};
    near1[k] = grid.get_nearest_point_index(p, 1);
    near2[k] = grid.get_nearest_point_index(p, 2);
    rbins[k] = grid.get_random_point_index_in_neighbourhood_bins(p, 1, rng);
    rrad[k] = grid.get_random_point_index_in_neighbourhood(p, prm[1], rng);
    rfilt[k] = grid.get_random_point_index_in_neighbourhood(p, prm[1], rng, [](int j) { return j % 3 != 0; });
  }
  write_raw(out + ".near1", near1.data(), (size_t)m * 4);
  write_raw(out + ".near2", near2.data(), (size_t)m * 4);
  write_raw(out + ".rbins", rbins.data(), (size_t)m * 4);
  write_raw(out + ".rrad", rrad.data(), (size_t)m * 4);
  write_raw(out + ".rfilt", rfilt.data(), (size_t)m * 4);
  return 0;
}

// Scenario "laws": the reference's predefined force functions
// (forces/predefined.hpp:60-491) in float at m distances and displacements
// read from the input (uint32 m, float32 d[m], float32 disp[m*3]).  Output
// <out>.laws: per
// distance 7 magnitudes then 7 vectors (x, y, z), in the order Spring,
// PiecewiseLinear, PiecewiseQuadratic, Cubic, Morse, LennardJones,
// HertzContact, with the parameters written beside each call.
static int run_laws(const char* path, const std::string& out) {
  using Vector = tecs::VectorN<float, 3>;
  namespace F = tecs::forces;
  FILE* f = std::fopen(path, "rb");
  if (!f) return 2;
  unsigned m = 0;
  if (std::fread(&m, 4, 1, f) != 1) return 2;
  std::vector<float> d(m), disp((size_t)m * 3);
  if (m && (std::fread(d.data(), 4, m, f) != m || std::fread(disp.data(), 4, disp.size(), f) != disp.size()))
    return 2;
  std::fclose(f);
  std::vector<float> res((size_t)m * 28);
  for (unsigned k = 0; k < m; ++k) {
    const float r = d[k];
    const Vector v{disp[3 * k], disp[3 * k + 1], disp[3 * k + 2]};
    float* o = &res[(size_t)k * 28];
    o[0] = F::SpringPotential(r, 1.0f, 0.5f);
    o[1] = F::PiecewiseLinearPotential(r, 0.8f, 1.5f, 0.3f);
    o[2] = F::PiecewiseQuadraticPotential(r, 1.0f, 1.4f, 1.8f, 2.0f, 0.7f);
    o[3] = F::CubicPotential(r, 1.0f, 1.6f, 3.0f);
    o[4] = F::MorsePotential(r, 1.0f, 2.0f, 0.25f);
    o[5] = F::LennardJonesPotential(r, 0.9f, 1.1f, 0.5f);
    o[6] = F::HertzContactPotential(r, 0.6f, 0.7f, 2.0f, 3.0f, 0.3f, 0.4f);
    const Vector w[7] = {F::Spring(v, r, 1.0f, 0.5f),
                         F::PiecewiseLinear(v, r, 0.8f, 1.5f, 0.3f),
                         F::PiecewiseQuadratic(v, r, 1.0f, 1.4f, 1.8f, 2.0f, 0.7f),
                         F::Cubic(v, r, 1.0f, 1.6f, 3.0f),
                         F::Morse(v, r, 1.0f, 2.0f, 0.25f),
                         F::LennardJones(v, r, 0.9f, 1.1f, 0.5f),
                         F::HertzContact(v, r, 0.6f, 0.7f, 2.0f, 3.0f, 0.3f, 0.4f)};
    for (int l = 0; l < 7; ++l)
      for (int c = 0; c < 3; ++c) o[7 + 3 * l + c] = w[l][c];
  }
  write_raw(out + ".laws", res.data(), res.size() * 4);
  return 0;
}

int main(int argc, char** argv) {
  if (argc < 6) {
    std::fprintf(stderr, "usage: %s <scenario> <in.bin> <out_prefix> <steps> <dt>\n", argv[0]);
    return 2;
  }
  Kokkos::initialize();
  const std::string sc = argv[1];
  if (sc == "grid_3" || sc == "grid_2") {
    const int rc = sc == "grid_3" ? run_grid<3>(argv[2], argv[3]) : run_grid<2>(argv[2], argv[3]);
    Kokkos::finalize();
    return rc;
  }
  if (sc == "laws") {
    const int rc = run_laws(argv[2], argv[3]);
    Kokkos::finalize();
    return rc;
  }
  const Input in = read_input(argv[2], sc.rfind("lk_", 0) == 0);
  const std::string out = argv[3];
  const int steps = std::atoi(argv[4]);
  const double dt = std::atof(argv[5]);
  int rc = 3;
#define DISPATCH(NAME) \
  if (sc == #NAME) rc = NAME::run(in, out, steps, dt);
  DISPATCH(drag_bg_heun_3) DISPATCH(drag_ba_euler_com_3) DISPATCH(upd_bg_heun_3)
  DISPATCH(fields_bg_heun_3) DISPATCH(fields_ba_euler_com_3)
  DISPATCH(ba_euler_3) DISPATCH(ba_heun_com_3) DISPATCH(bg_heun_3) DISPATCH(bg_heun_com_3) DISPATCH(bg_euler_com_3)
  DISPATCH(na_heun_3) DISPATCH(ng_heun_3) DISPATCH(bgs_euler_com_3) DISPATCH(bas_heun_3) DISPATCH(ngs_euler_3)
  DISPATCH(nas_heun_3)
  DISPATCH(bg_heun_pol_3) DISPATCH(ng_euler_2) DISPATCH(bg_heun_2) DISPATCH(nd_euler_2) DISPATCH(nd_heun_3)
  DISPATCH(lk_bg_heun_3) DISPATCH(lk_ba_euler_com_3) DISPATCH(lk_writer_3) DISPATCH(gen_bg_heun_3)
#undef DISPATCH
  if (rc == 3) std::fprintf(stderr, "unknown scenario %s\n", sc.c_str());
  return rc;
}
