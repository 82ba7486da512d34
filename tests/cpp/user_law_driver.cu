// user_law_driver.cu -- a program whose pairwise laws are PAIRWISE_FORCE
// lambdas and PAIRWISE_FORCE_OP functors, as the reference's programs write
// them, compiled by nvcc against include/tecs/pairwise.cuh.  The law is the
// two-radius spring the reference's fixtures were made with, written with the
// same operations, so its outputs must equal the reference's bit for bit.
//
//   user_law_driver <scenario> <in.bin> <out_prefix> <steps> <dt>
//
// in.bin and the outputs are those of drop_in_driver.cpp (.pairs, .dpos,
// .pos, and .pol for "bg_heun_pol"; link scenarios read the links and write
// .pos only).  Scenario
// "rng_twice" steps two copies of the input with a law that draws from rng and
// writes <out>.a.pos and <out>.b.pos; "drag_bg_heun" / "drag_ba_euler_com"
// step with a law that sets drag and also write <out>.ov, the old velocities.
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "tecs/pairwise.cuh"

using namespace tecs;

CREATE_SIMULATION_CONFIG(NaiveAllPairsHeun,
                         CONFIG_PAIR_FINDER(pair_finders::NaiveAllPairs)
                         CONFIG_INTEGRATOR(integrators::Heun))
CREATE_SIMULATION_CONFIG(NaiveGabrielHeun,
                         CONFIG_PAIR_FINDER(pair_finders::NaiveGabriel)
                         CONFIG_INTEGRATOR(integrators::Heun))
CREATE_SIMULATION_CONFIG(BinnedAllPairsEuler,
                         CONFIG_PAIR_FINDER(pair_finders::BinnedAllPairs)
                         CONFIG_INTEGRATOR(integrators::Euler))
CREATE_SIMULATION_CONFIG(BinnedAllPairsEulerCom,
                         CONFIG_PAIR_FINDER(pair_finders::BinnedAllPairs)
                         CONFIG_INTEGRATOR(integrators::Euler)
                         CONFIG_COM_FIXER(com_fixers::GlobalComFixer))
CREATE_SIMULATION_CONFIG(FieldsGabrielHeun,
                         CONFIG_PAIR_FINDER(pair_finders::BinnedGabriel)
                         CONFIG_INTEGRATOR(integrators::Heun)
                         CONFIG_FIELDS((Vector, position), (Scalar, u), (Vector, w)))
CREATE_SIMULATION_CONFIG(FieldsAllPairsEulerCom,
                         CONFIG_PAIR_FINDER(pair_finders::BinnedAllPairs)
                         CONFIG_INTEGRATOR(integrators::Euler)
                         CONFIG_COM_FIXER(com_fixers::GlobalComFixer)
                         CONFIG_FIELDS((Vector, position), (Scalar, u), (Vector, w)))
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
struct BinnedGabrielHeun2D : public DefaultSimulationConfig {
  CONFIG_PAIR_FINDER(pair_finders::BinnedGabriel)
  CONFIG_INTEGRATOR(integrators::Heun)
  CONFIG_DIMENSIONS(2)
  RESOLVE_TECS_CONFIG()
};

struct NaiveDelaunayEuler2D : public DefaultSimulationConfig {
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

// the fixtures' law, F(d) = k_rep*max(r_rep-d,0) - k_adh*max(d-r_adh,0), as a functor
template <typename Config>
struct SpringFunctor {
  EXTRACT_TYPES_FROM_SIMULATION_CONFIG(Config)
  float k_rep, r_rep, k_adh, r_adh;
  PAIRWISE_FORCE_OP {
    if (distance != Scalar(0)) {
      const Scalar F = k_rep * fmaxf(r_rep - distance, Scalar(0)) - k_adh * fmaxf(distance - r_adh, Scalar(0));
      ctx.position.delta += displacement * F / distance;
    }
  }
};

template <typename Config>
static typename Simulation<Config>::Settings settings_of(const Input& in) {
  using Sim = Simulation<Config>;
  constexpr int D = Sim::dimensions;
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
  settings.link_capacity = unsigned(in.links.size() / 2);
  settings.link_active_count = settings.link_capacity;
  return settings;
}

template <typename Config>
static void fill(Simulation<Config>& sim, const Input& in) {
  constexpr int D = Config::dimensions;
  auto& positions = sim.get_positions_view();
  for (unsigned i = 0; i < in.n; ++i)
    for (int d = 0; d < D; ++d) positions(i)[d] = in.x[std::size_t(i) * D + d];
  auto& links = sim.get_links();
  for (unsigned l = 0; l < in.links.size() / 2; ++l) links(l) = Link{in.links[2 * l], in.links[2 * l + 1]};
  if constexpr (Simulation<Config>::has_polarity) {
    auto& polarity = sim.template get_view<FIELD(Polarity_<float>, polarity)>();
    for (unsigned i = 0; i < in.n; ++i) polarity(i) = Polarity_<float>(in.p[2 * i], in.p[2 * i + 1]);
  }
}

template <typename Config>
static int run(const Input& in, const std::string& out, int steps, double dt, bool functor) {
  EXTRACT_TYPES_FROM_SIMULATION_CONFIG(Config)
  if (int(in.dims) != dimensions) { std::fprintf(stderr, "input has %u dims\n", in.dims); return 2; }
  const Scalar k_rep = in.prm[8], r_rep = in.prm[9], k_adh = in.prm[10], r_adh = in.prm[11];
  auto spring = PAIRWISE_FORCE(
    if (distance != Scalar(0)) {
      const Scalar F = k_rep * fmaxf(r_rep - distance, Scalar(0)) - k_adh * fmaxf(distance - r_adh, Scalar(0));
      ctx.position.delta += displacement * F / distance;
    }
  );
  Simulation<Config> sim(settings_of<Config>(in));
  fill(sim, in);
  auto go = [&](const auto& law) {
    std::vector<Vector> deltas;
    const auto pairs = sim.evaluate(law, &deltas);
    std::vector<unsigned> flat;
    for (const auto& pr : pairs) { flat.push_back(pr.first); flat.push_back(pr.second); }
    write_raw(out + ".pairs", flat.data(), flat.size() * 4);
    write_raw(out + ".dpos", deltas.data(), deltas.size() * sizeof(Vector));
    for (int s = 0; s < steps; ++s) sim.take_step(dt, law);
  };
  if (functor) go(SpringFunctor<Config>{k_rep, r_rep, k_adh, r_adh});
  else go(spring());
  const auto& x = sim.get_positions_view();
  write_raw(out + ".pos", x.data(), std::size_t(sim.get_agent_count()) * sizeof(Vector));
  return 0;
}

// the epithelium law: the spring plus k_pol * (bending + bidirectional alignment), written with the
// reference's Polarity_ force functions as its polarity programs write it
static int run_polarity(const Input& in, const std::string& out, int steps, double dt) {
  EXTRACT_TYPES_FROM_SIMULATION_CONFIG(EpithelialSheet)
  const Scalar k_rep = in.prm[8], r_rep = in.prm[9], k_adh = in.prm[10], r_adh = in.prm[11], k_pol = in.prm[12];
  auto epithelium = PAIRWISE_FORCE(
    if (distance != Scalar(0)) {
      const Scalar F = k_rep * fmaxf(r_rep - distance, Scalar(0)) - k_adh * fmaxf(distance - r_adh, Scalar(0));
      ctx.position.delta += displacement * F / distance;
    }
    auto bend = ctx.polarity.self.bending_force(displacement, ctx.polarity.other, distance);
    ctx.position.delta += bend.vector * k_pol;
    ctx.polarity.delta += bend.polarity * k_pol;
    ctx.polarity.delta += ctx.polarity.self.bidirectional_polarization_force(ctx.polarity.other) * k_pol;
  );
  Simulation<EpithelialSheet> sim(settings_of<EpithelialSheet>(in));
  fill(sim, in);
  std::vector<Vector> deltas;
  const auto pairs = sim.evaluate(epithelium(), &deltas);
  std::vector<unsigned> flat;
  for (const auto& pr : pairs) { flat.push_back(pr.first); flat.push_back(pr.second); }
  write_raw(out + ".pairs", flat.data(), flat.size() * 4);
  write_raw(out + ".dpos", deltas.data(), deltas.size() * sizeof(Vector));
  for (int s = 0; s < steps; ++s) sim.take_step(dt, epithelium());
  const auto& x = sim.get_positions_view();
  write_raw(out + ".pos", x.data(), std::size_t(sim.get_agent_count()) * sizeof(Vector));
  const auto& p = sim.template get_view<FIELD(Polarity_<float>, polarity)>();
  write_raw(out + ".pol", p.data(), std::size_t(sim.get_agent_count()) * 8);
  return 0;
}

// a GENERIC_FORCE law with the spring, passed pairwise first; the generic
// force is evaluated first, as the reference fuses them.  Writes .pos only.
static int run_generic(const Input& in, const std::string& out, int steps, double dt) {
  EXTRACT_TYPES_FROM_SIMULATION_CONFIG(BinnedGabrielHeun)
  const Scalar k_rep = in.prm[8], r_rep = in.prm[9], k_adh = in.prm[10], r_adh = in.prm[11];
  auto spring = PAIRWISE_FORCE(
    if (distance != Scalar(0)) {
      const Scalar F = k_rep * fmaxf(r_rep - distance, Scalar(0)) - k_adh * fmaxf(distance - r_adh, Scalar(0));
      ctx.position.delta += displacement * F / distance;
    }
  );
  auto pull = GENERIC_FORCE(
    if (is_full_step) ctx.position.delta += ctx.position.self * Scalar(-0.02);
    else ctx.position.delta += Vector(Scalar(0.001));
  );
  Simulation<BinnedGabrielHeun> sim(settings_of<BinnedGabrielHeun>(in));
  fill(sim, in);
  for (int s = 0; s < steps; ++s) sim.take_step(dt, spring(), pull());
  const auto& x = sim.get_positions_view();
  write_raw(out + ".pos", x.data(), std::size_t(sim.get_agent_count()) * sizeof(Vector));
  return 0;
}

// links and a user law in one step, as the reference's protrusion programs
template <typename Config>
static int run_links(const Input& in, const std::string& out, int steps, double dt) {
  EXTRACT_TYPES_FROM_SIMULATION_CONFIG(Config)
  const Scalar k_rep = in.prm[8], r_rep = in.prm[9], k_adh = in.prm[10], r_adh = in.prm[11];
  auto spring = PAIRWISE_FORCE(
    if (distance != Scalar(0)) {
      const Scalar F = k_rep * fmaxf(r_rep - distance, Scalar(0)) - k_adh * fmaxf(distance - r_adh, Scalar(0));
      ctx.position.delta += displacement * F / distance;
    }
  );
  Simulation<Config> sim(settings_of<Config>(in));
  fill(sim, in);
  const forces::LinkPull protrusions{in.prm[15]};
  for (int s = 0; s < steps; ++s) sim.take_step(dt, protrusions, spring());
  const auto& x = sim.get_positions_view();
  write_raw(out + ".pos", x.data(), std::size_t(sim.get_agent_count()) * sizeof(Vector));
  return 0;
}

// the same run with the link law written as a LINK_FORCE lambda, as the
// reference's protrusion programs write it (examples/intercalation.cpp:65-71)
template <typename Config>
static int run_link_lambda(const Input& in, const std::string& out, int steps, double dt) {
  EXTRACT_TYPES_FROM_SIMULATION_CONFIG(Config)
  const Scalar k_rep = in.prm[8], r_rep = in.prm[9], k_adh = in.prm[10], r_adh = in.prm[11];
  const Scalar k_link = in.prm[15];
  auto spring = PAIRWISE_FORCE(
    if (distance != Scalar(0)) {
      const Scalar F = k_rep * fmaxf(r_rep - distance, Scalar(0)) - k_adh * fmaxf(distance - r_adh, Scalar(0));
      ctx.position.delta += displacement * F / distance;
    }
  );
  auto protrusions = LINK_FORCE(
    Vector displacement = ctx.position.b - ctx.position.a;
    Scalar distance = displacement.length();
    ctx.position.delta_a += k_link * displacement / distance;
    ctx.position.delta_b += -k_link * displacement / distance;
  );
  Simulation<Config> sim(settings_of<Config>(in));
  fill(sim, in);
  for (int s = 0; s < steps; ++s) sim.take_step(dt, protrusions(), spring());
  const auto& x = sim.get_positions_view();
  write_raw(out + ".pos", x.data(), std::size_t(sim.get_agent_count()) * sizeof(Vector));
  return 0;
}

// a config with a Scalar field u and a Vector field w beyond the position:
// the pairwise law diffuses them between neighbours and drives w along the
// displacement, the generic law adds to u from the position; writes .pos,
// .u and .w
template <typename FieldsConfig>
static int run_fields(const Input& in, const std::string& out, int steps, double dt) {
  EXTRACT_TYPES_FROM_SIMULATION_CONFIG(FieldsConfig)
  const Scalar k_rep = in.prm[8], r_rep = in.prm[9], k_adh = in.prm[10], r_adh = in.prm[11];
  auto law = PAIRWISE_FORCE(
    if (distance != Scalar(0)) {
      const Scalar F = k_rep * fmaxf(r_rep - distance, Scalar(0)) - k_adh * fmaxf(distance - r_adh, Scalar(0));
      ctx.position.delta += displacement * F / distance;
    }
    ctx.u.delta += (ctx.u.other - ctx.u.self) * Scalar(0.2);
    ctx.w.delta += (ctx.w.other - ctx.w.self) * Scalar(0.1) + displacement * Scalar(0.01);
  );
  auto generic = GENERIC_FORCE(ctx.u.delta += Scalar(0.05) * ctx.position.self[0];);
  Simulation<FieldsConfig> sim(settings_of<FieldsConfig>(in));
  auto& pos = sim.template get_view<FIELD(Vector, position)>();
  auto& u = sim.template get_view<FIELD(Scalar, u)>();
  auto& w = sim.template get_view<FIELD(Vector, w)>();
  for (unsigned i = 0; i < in.n; ++i) {
    for (int d = 0; d < 3; ++d) pos(i)[d] = in.x[std::size_t(i) * 3 + d];
    u(i) = pos(i)[0] * Scalar(0.3) + Scalar(1);
    w(i) = pos(i) * Scalar(0.5);
  }
  for (int s = 0; s < steps; ++s) sim.take_step(dt, law(), generic());
  const unsigned n = sim.get_agent_count();
  write_raw(out + ".pos", pos.data(), std::size_t(n) * sizeof(Vector));
  write_raw(out + ".u", u.data(), std::size_t(n) * sizeof(Scalar));
  write_raw(out + ".w", w.data(), std::size_t(n) * sizeof(Vector));
  return 0;
}

// a law that draws from rng: two simulations of the same input give the same run
static int run_rng_twice(const Input& in, const std::string& out, int steps, double dt) {
  EXTRACT_TYPES_FROM_SIMULATION_CONFIG(BinnedGabrielHeun)
  auto noisy = PAIRWISE_FORCE(
    if (distance != Scalar(0)) {
      const Scalar F = Scalar(2) * fmaxf(Scalar(0.7) - distance, Scalar(0)) + Scalar(0.1) * rng.frand(-1.f, 1.f);
      ctx.position.delta += displacement * F / distance;
      if (is_full_step) ctx.position.delta += Vector(Scalar(0.01) * Scalar(rng.normal()));
    }
  );
  for (const char* tag : {".a.pos", ".b.pos"}) {
    Simulation<BinnedGabrielHeun> sim(settings_of<BinnedGabrielHeun>(in));
    fill(sim, in);
    for (int s = 0; s < steps; ++s) sim.take_step(dt, noisy());
    const auto& x = sim.get_positions_view();
    write_raw(out + tag, x.data(), std::size_t(sim.get_agent_count()) * sizeof(Vector));
  }
  return 0;
}

// a law that sets drag (the spring plus drag = 0.5 * max(1.2 - d, 0) + 0.1):
// writes .pos and .ov (the integrator's old velocities after the last step)
template <typename Config>
static int run_drag(const Input& in, const std::string& out, int steps, double dt) {
  EXTRACT_TYPES_FROM_SIMULATION_CONFIG(Config)
  const Scalar k_rep = in.prm[8], r_rep = in.prm[9], k_adh = in.prm[10], r_adh = in.prm[11];
  auto dragging = PAIRWISE_FORCE(
    if (distance != Scalar(0)) {
      const Scalar F = k_rep * fmaxf(r_rep - distance, Scalar(0)) - k_adh * fmaxf(distance - r_adh, Scalar(0));
      ctx.position.delta += displacement * F / distance;
    }
    drag = Scalar(0.5) * fmaxf(Scalar(1.2) - distance, Scalar(0)) + Scalar(0.1);
  );
  Simulation<Config> sim(settings_of<Config>(in));
  fill(sim, in);
  for (int s = 0; s < steps; ++s) sim.take_step(dt, dragging());
  const auto& x = sim.get_positions_view();
  const unsigned n = sim.get_agent_count();
  write_raw(out + ".pos", x.data(), std::size_t(n) * sizeof(Vector));
  auto ov = sim.get_old_velocities_view_from_integrator();
  write_raw(out + ".ov", ov.data(), std::size_t(n) * sizeof(Vector));
  return 0;
}

int main(int argc, char** argv) {
  if (argc < 6) return 2;
  const std::string scenario = argv[1];
  const bool links = scenario.rfind("lk_", 0) == 0;  // lk_* scenarios read links
  const Input in = read_input(argv[2], links);
  const std::string out = argv[3];
  const int steps = std::atoi(argv[4]);
  const double dt = std::atof(argv[5]);
  try {
    if (scenario == "na_heun") return run<NaiveAllPairsHeun>(in, out, steps, dt, false);
    if (scenario == "ng_heun") return run<NaiveGabrielHeun>(in, out, steps, dt, false);
    if (scenario == "ba_euler") return run<BinnedAllPairsEuler>(in, out, steps, dt, false);
    if (scenario == "bg_heun") return run<BinnedGabrielHeun>(in, out, steps, dt, false);
    if (scenario == "bg_heun_functor") return run<BinnedGabrielHeun>(in, out, steps, dt, true);
    if (scenario == "bg_heun_com") return run<BinnedGabrielHeunCom>(in, out, steps, dt, false);
    if (scenario == "bg_heun_2d") return run<BinnedGabrielHeun2D>(in, out, steps, dt, false);
    // NaiveDelaunay: the naive finder up to 4096 cells of capacity, the
    // library's Delaunay finder of any capacity past that
    if (scenario == "nd_euler_2d") return run<NaiveDelaunayEuler2D>(in, out, steps, dt, false);
    if (scenario == "bg_heun_pol") return run_polarity(in, out, steps, dt);
    if (scenario == "gen_bg_heun") return run_generic(in, out, steps, dt);
    if (scenario == "lk_bg_heun") return run_links<BinnedGabrielHeun>(in, out, steps, dt);
    if (scenario == "lk_lambda_bg_heun") return run_link_lambda<BinnedGabrielHeun>(in, out, steps, dt);
    if (scenario == "lk_lambda_ba_euler_com") return run_link_lambda<BinnedAllPairsEulerCom>(in, out, steps, dt);
    if (scenario == "rng_twice") return run_rng_twice(in, out, steps, dt);
    if (scenario == "drag_bg_heun") return run_drag<BinnedGabrielHeun>(in, out, steps, dt);
    if (scenario == "fields_bg_heun") return run_fields<FieldsGabrielHeun>(in, out, steps, dt);
    if (scenario == "fields_ba_euler_com") return run_fields<FieldsAllPairsEulerCom>(in, out, steps, dt);
    if (scenario == "drag_ba_euler_com") return run_drag<BinnedAllPairsEulerCom>(in, out, steps, dt);
  } catch (const Error& e) {
    std::fprintf(stderr, "tecs error: %s\n", e.what());
    return 1;
  }
  std::fprintf(stderr, "unknown scenario %s\n", scenario.c_str());
  return 2;
}
