// drop_in_driver.cpp -- a C++20 program written against the drop-in layer
// (include/tecs/tecs.hpp) the way the reference's programs are written
// against include/tecs.hpp: a config struct, Simulation<Config>, get_view,
// take_step.  The tests compile it with g++ and run it on the inputs of the
// golden fixtures; its outputs must equal the reference's.
//
//   drop_in_driver <scenario> <in.bin> <out_prefix> <steps> <dt>
//
// in.bin: uint32 n, uint32 dims, uint32 has_polarity, float32 params[16],
//         float32 positions[n*dims], float32 polarity[n*2] (if present)
// params: cutoff, gabriel_c, min_x, min_y, min_z, max_x, max_y, max_z,
//         k_rep, r_rep, k_adh, r_adh, k_pol, capacity, bin_size_scale, spare
// outputs: <out>.pairs (uint32 directed pairs), <out>.dpos (deltas of one
//          full-step pass), <out>.pos / <out>.pol (state after the steps).
// Link scenarios ("lk_*") read, after the polarity block, uint32 n_links and
// uint32 links[2*n_links], take the link strength from params[15], step with
// take_step(dt, link_law, pairwise_law) and write <out>.pos only; "lk_writer"
// writes <out>.h5 and <out>.xmf through CONFIG_WRITER(io::HDF5_Writer).
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "tecs/tecs.hpp"

using namespace tecs;

CREATE_SIMULATION_CONFIG(BinnedAllPairsEuler,
                         CONFIG_PAIR_FINDER(pair_finders::BinnedAllPairs)
                         CONFIG_INTEGRATOR(integrators::Euler))

CREATE_SIMULATION_CONFIG(BinnedGabrielHeun,
                         CONFIG_PAIR_FINDER(pair_finders::BinnedGabriel)
                         CONFIG_INTEGRATOR(integrators::Heun))

CREATE_SIMULATION_CONFIG(BinnedGabrielHeunCom,
                         CONFIG_PAIR_FINDER(pair_finders::BinnedGabriel)
                         CONFIG_INTEGRATOR(integrators::Heun)
                         CONFIG_COM_FIXER(com_fixers::GlobalComFixer))

CREATE_SIMULATION_CONFIG(EpithelialSheet,
                         CONFIG_PAIR_FINDER(pair_finders::BinnedGabriel)
                         CONFIG_INTEGRATOR(integrators::Heun)
                         CONFIG_FIELDS((Vector, position), (Polarity, polarity)))

CREATE_SIMULATION_CONFIG(BinnedGabrielHeunH5,
                         CONFIG_PAIR_FINDER(pair_finders::BinnedGabriel)
                         CONFIG_INTEGRATOR(integrators::Heun)
                         CONFIG_WRITER(io::HDF5_Writer))

CREATE_SIMULATION_CONFIG(BinnedAllPairsEulerCom,
                         CONFIG_PAIR_FINDER(pair_finders::BinnedAllPairs)
                         CONFIG_INTEGRATOR(integrators::Euler)
                         CONFIG_COM_FIXER(com_fixers::GlobalComFixer))

CREATE_SIMULATION_CONFIG(EpithelialSheetH5,
                         CONFIG_PAIR_FINDER(pair_finders::BinnedGabriel)
                         CONFIG_INTEGRATOR(integrators::Heun)
                         CONFIG_WRITER(io::HDF5_Writer)
                         CONFIG_FIELDS((Vector, position), (Polarity, polarity)))

struct PlainDelaunay2D : public DefaultSimulationConfig {
  CONFIG_PAIR_FINDER(pair_finders::NaiveDelaunay)
  CONFIG_INTEGRATOR(integrators::Euler)
  CONFIG_DIMENSIONS(2)
  RESOLVE_TECS_CONFIG()
};

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
  in.x.resize(std::size_t(in.n) * in.dims);
  if (in.n && std::fread(in.x.data(), 4, in.x.size(), f) != in.x.size()) std::exit(2);
  if (in.has_pol) {
    in.p.resize(std::size_t(in.n) * 2);
    if (in.n && std::fread(in.p.data(), 4, in.p.size(), f) != in.p.size()) std::exit(2);
  }
  if (with_links) {
    unsigned nl = 0;
    if (std::fread(&nl, 4, 1, f) != 1) std::exit(2);
    in.links.resize(std::size_t(nl) * 2);
    if (nl && std::fread(in.links.data(), 4, in.links.size(), f) != in.links.size()) std::exit(2);
  }
  std::fclose(f);
  return in;
}

static void write_raw(const std::string& path, const void* data, std::size_t bytes) {
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) { std::perror(path.c_str()); std::exit(2); }
  if (bytes) std::fwrite(data, 1, bytes, f);
  std::fclose(f);
}

template <typename Config, typename Force>
static int run(const Input& in, const std::string& out, int steps, double dt, const Force& force) {
  using Sim = Simulation<Config>;
  using Vector = typename Sim::Vector;
  constexpr int D = Sim::dimensions;
  if (int(in.dims) != D) { std::fprintf(stderr, "input has %u dims, config %d\n", in.dims, D); return 2; }
  typename Sim::Settings settings(in.n, "unused");
  settings.cutoff_distance = in.prm[0];
  settings.capacity = unsigned(in.prm[13]) > in.n ? unsigned(in.prm[13]) : in.n;
  auto& pfs = settings.pair_finder_settings;
  if constexpr (requires { pfs.gabriel_coefficient; }) pfs.gabriel_coefficient = in.prm[1];
  if constexpr (requires { pfs.min_bounds; }) {
    for (int d = 0; d < D; ++d) {
      pfs.min_bounds[d] = in.prm[2 + d];
      pfs.max_bounds[d] = in.prm[5 + d];
    }
    pfs.bin_size_scale = in.prm[14];
  }
  Sim sim(settings);
  auto& positions = sim.template get_view<FIELD(Vector, position)>();
  for (unsigned i = 0; i < in.n; ++i)
    for (int d = 0; d < D; ++d) positions(i)[d] = in.x[std::size_t(i) * D + d];
  if constexpr (Sim::has_polarity) {
    auto& polarity = sim.template get_view<FIELD(Polarity_<float>, polarity)>();
    for (unsigned i = 0; i < in.n; ++i) polarity(i) = Polarity_<float>(in.p[2 * i], in.p[2 * i + 1]);
  }

  // one full-step force pass of the initial state
  std::vector<Vector> deltas;
  const auto pairs = sim.evaluate(force, &deltas);
  std::vector<unsigned> flat_pairs;
  for (const auto& pr : pairs) { flat_pairs.push_back(pr.first); flat_pairs.push_back(pr.second); }
  write_raw(out + ".pairs", flat_pairs.data(), flat_pairs.size() * 4);
  write_raw(out + ".dpos", deltas.data(), deltas.size() * sizeof(Vector));

  for (int s = 0; s < steps; ++s) sim.take_step(dt, force);

  const auto& final_positions = sim.template get_view<FIELD(Vector, position)>();
  write_raw(out + ".pos", final_positions.data(), std::size_t(sim.get_agent_count()) * sizeof(Vector));
  if constexpr (Sim::has_polarity) {
    const auto& final_polarity = sim.template get_view<FIELD(Polarity_<float>, polarity)>();
    write_raw(out + ".pol", final_polarity.data(), std::size_t(sim.get_agent_count()) * 8);
  }
  return 0;
}

// the reference's protrusion programs: links written through get_links(),
// stepped with a link law and a pairwise law
template <typename Config>
static int run_links(const Input& in, const std::string& out, int steps, double dt) {
  using Sim = Simulation<Config>;
  constexpr int D = Sim::dimensions;
  typename Sim::Settings settings(in.n, "unused");
  settings.cutoff_distance = in.prm[0];
  settings.capacity = unsigned(in.prm[13]) > in.n ? unsigned(in.prm[13]) : in.n;
  const unsigned nl = unsigned(in.links.size() / 2);
  settings.link_capacity = nl;
  settings.link_active_count = nl;
  for (int d = 0; d < D; ++d) {
    settings.pair_finder_settings.min_bounds[d] = in.prm[2 + d];
    settings.pair_finder_settings.max_bounds[d] = in.prm[5 + d];
  }
  Sim sim(settings);
  auto& positions = sim.get_positions_view();
  for (unsigned i = 0; i < in.n; ++i)
    for (int d = 0; d < D; ++d) positions(i)[d] = in.x[std::size_t(i) * D + d];
  auto& links = sim.get_links();
  for (unsigned l = 0; l < nl; ++l) links(l) = Link{in.links[2 * l], in.links[2 * l + 1]};
  const forces::Spring2R spring{in.prm[8], in.prm[9], in.prm[10], in.prm[11]};
  const forces::LinkPull protrusions{in.prm[15]};
  for (int s = 0; s < steps; ++s) sim.take_step(dt, protrusions, spring);
  const auto& final_positions = sim.get_positions_view();
  write_raw(out + ".pos", final_positions.data(), std::size_t(sim.get_agent_count()) * sizeof(typename Sim::Vector));
  return 0;
}

// the reference's example loop: write(0), then take_step + write each step,
// into "<out>.h5"
static int run_written(const Input& in, const std::string& out, int steps, double dt) {
  using Sim = Simulation<BinnedGabrielHeunH5>;
  Sim::Settings settings(in.n, out);
  settings.cutoff_distance = in.prm[0];
  for (int d = 0; d < 3; ++d) {
    settings.pair_finder_settings.min_bounds[d] = in.prm[2 + d];
    settings.pair_finder_settings.max_bounds[d] = in.prm[5 + d];
  }
  Sim sim(settings);
  auto& positions = sim.get_positions_view();
  for (unsigned i = 0; i < in.n; ++i)
    for (int d = 0; d < 3; ++d) positions(i)[d] = in.x[std::size_t(i) * 3 + d];
  sim.write(0.0);
  const forces::Spring2R spring{in.prm[8], in.prm[9], in.prm[10], in.prm[11]};
  for (int s = 1; s <= steps; ++s) {
    sim.take_step(dt, spring);
    sim.write(s * dt);
  }
  return 0;
}

// positions, polarity and links written with a static cell-type view:
// write_static, write(0), then take_step + write() each step, into
// "<out>.h5" and its XDMF sidecar "<out>.xmf"
static int run_written_links(const Input& in, const std::string& out, int steps, double dt) {
  using Sim = Simulation<EpithelialSheetH5>;
  Sim::Settings settings(in.n, out);
  settings.cutoff_distance = in.prm[0];
  const unsigned nl = unsigned(in.links.size() / 2);
  settings.link_capacity = nl;
  settings.link_active_count = nl;
  for (int d = 0; d < 3; ++d) {
    settings.pair_finder_settings.min_bounds[d] = in.prm[2 + d];
    settings.pair_finder_settings.max_bounds[d] = in.prm[5 + d];
  }
  Sim sim(settings);
  auto& positions = sim.get_positions_view();
  for (unsigned i = 0; i < in.n; ++i)
    for (int d = 0; d < 3; ++d) positions(i)[d] = in.x[std::size_t(i) * 3 + d];
  auto& polarity = sim.get_view<FIELD(Polarity_<float>, polarity)>();
  for (unsigned i = 0; i < in.n; ++i) polarity(i) = Polarity_<float>(in.p[2 * i], in.p[2 * i + 1]);
  auto& links = sim.get_links();
  for (unsigned l = 0; l < nl; ++l) links(l) = Link{in.links[2 * l], in.links[2 * l + 1]};
  View<float> cell_type("cell_type", in.n);
  for (unsigned i = 0; i < in.n; ++i) cell_type(i) = float(i % 3);
  sim.write_static(cell_type);
  sim.write(0.0);
  const forces::Spring2R spring{in.prm[8], in.prm[9], in.prm[10], in.prm[11]};
  for (int s = 0; s < steps; ++s) {
    sim.take_step(dt, spring);
    sim.write();
  }
  return 0;
}

// update functions between steps, as the reference's growth and protrusion
// programs run them: run with two UPDATE_FUNC functions (fused per cell),
// run_links with one that rewires every link, an INIT_FUNC through init,
// then the steps; writes <out>.pos, <out>.links and <out>.hits
static int run_update(const Input& in, const std::string& out, int steps, double dt) {
  using Sim = Simulation<BinnedGabrielHeun>;
  EXTRACT_TYPES_FROM_SIMULATION_CONFIG(BinnedGabrielHeun)
  const unsigned n = in.n;
  Sim::Settings settings(n, "unused");
  settings.cutoff_distance = in.prm[0];
  settings.pair_finder_settings.gabriel_coefficient = in.prm[1];
  for (int d = 0; d < 3; ++d) {
    settings.pair_finder_settings.min_bounds[d] = in.prm[2 + d];
    settings.pair_finder_settings.max_bounds[d] = in.prm[5 + d];
  }
  settings.pair_finder_settings.bin_size_scale = in.prm[14];
  settings.link_capacity = n;
  settings.link_active_count = n;
  Sim sim(settings);
  auto& pos = sim.get_view<FIELD(Vector, position)>();
  for (unsigned i = 0; i < n; ++i)
    for (int d = 0; d < 3; ++d) pos(i)[d] = in.x[std::size_t(i) * 3 + d];
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
  const forces::Spring2R spring{in.prm[8], in.prm[9], in.prm[10], in.prm[11]};
  for (int s = 0; s < steps; ++s) sim.take_step(dt, spring);
  const auto& x = sim.get_positions_view();
  write_raw(out + ".pos", x.data(), std::size_t(n) * sizeof(Vector));
  std::vector<unsigned> lk(2 * std::size_t(n));
  for (unsigned l = 0; l < n; ++l) {
    lk[2 * l] = links(l).a;
    lk[2 * l + 1] = links(l).b;
  }
  write_raw(out + ".links", lk.data(), lk.size() * 4);
  const int h = hits;
  write_raw(out + ".hits", &h, 4);
  return 0;
}

int main(int argc, char** argv) {
  if (argc < 6) {
    std::fprintf(stderr, "usage: %s <scenario> <in.bin> <out_prefix> <steps> <dt>\n", argv[0]);
    return 2;
  }
  const std::string sc = argv[1];
  const Input in = read_input(argv[2], sc.rfind("lk_", 0) == 0);
  const std::string out = argv[3];
  const int steps = std::atoi(argv[4]);
  const double dt = std::atof(argv[5]);
  forces::Spring2R spring{in.prm[8], in.prm[9], in.prm[10], in.prm[11]};
  forces::PolaritySpring polar{in.prm[8], in.prm[9], in.prm[10], in.prm[11], in.prm[12]};
  try {
    if (sc == "ba_euler") return run<BinnedAllPairsEuler>(in, out, steps, dt, spring);
    if (sc == "bg_heun") return run<BinnedGabrielHeun>(in, out, steps, dt, spring);
    if (sc == "bg_heun_com") return run<BinnedGabrielHeunCom>(in, out, steps, dt, spring);
    if (sc == "bg_heun_pol") return run<EpithelialSheet>(in, out, steps, dt, polar);
    if (sc == "nd_euler_2d") return run<PlainDelaunay2D>(in, out, steps, dt, spring);
    if (sc == "lk_bg_heun") return run_links<BinnedGabrielHeun>(in, out, steps, dt);
    if (sc == "bg_heun_h5") return run_written(in, out, steps, dt);
    if (sc == "lk_ba_euler_com") return run_links<BinnedAllPairsEulerCom>(in, out, steps, dt);
    if (sc == "lk_writer") return run_written_links(in, out, steps, dt);
    if (sc == "upd_bg_heun") return run_update(in, out, steps, dt);
  } catch (const tecs::Error& e) {
    std::fprintf(stderr, "tecs error: %s\n", e.what());
    return 1;
  }
  std::fprintf(stderr, "unknown scenario %s\n", sc.c_str());
  return 3;
}
