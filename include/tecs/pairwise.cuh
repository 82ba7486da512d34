// tecs/pairwise.cuh -- user pairwise force laws for the C++20 drop-in layer.
//
// The reference's programs write their pairwise laws as lambdas or functors
// (include/utils/utils.hpp:181-276):
//
//   auto spring = PAIRWISE_FORCE(
//     ctx.position.delta += forces::Spring(displacement, distance, L_0);
//   );
//   sim.take_step(dt, spring());
//
// Included in a program compiled by nvcc (-std=c++20 --extended-lambda,
// sm_103a), this header makes such a law run on the GPU: the library's force
// pass (tecs/device/kernels.cuh, k_pass_law) is instantiated here with the
// law in place of a built-in one, and Simulation::take_step hands the library
// a launcher for it (tecs_sim_set_pair_law).  The pass finds the same pairs in
// the same order and adds each law call to the same per-cell sums as the
// built-in laws, so a law written with a built-in law's operations gives that
// law's bits (compile with -fmad=false, as the library is, for the reference's).
//
// What a law sees, per pair (i, j) the finder accepts (PAIRWISE_FORCE_PARAMETERS):
//   is_full_step   Euler and Heun's first evaluation: true; Heun's second: false
//   i, j           the two cells' ids
//   displacement   x_i - x_j, distance its length
//   rng            a tecs::CounterRandom keyed by (seed, step, evaluation, i, j)
//   drag           the pair's drag coefficient (0 unless the law sets it): the
//                  cell's position delta gains sum(drag * old velocity of j) /
//                  max(sum(drag), FLT_EPSILON) after its pair sums.  The
//                  simulation must keep old velocities (Settings::old_velocities,
//                  tecs_sim_keep_old_velocities); without them a law that sets
//                  drag makes the next count or download fail
//   ctx            ctx.<field>.self / .other / .delta for the config's fields
// A GENERIC_FORCE law (per cell: is_full_step, i, rng, ctx.<field>.self /
// .delta) runs in the same pass, added before the pair sums as the reference
// orders it; it combines with a PAIRWISE_FORCE law or runs alone.  A
// LINK_FORCE law (per link: is_full_step, link, rng, ctx.<field>.a / .b /
// .delta_a / .delta_b) takes the place of the built-in link pull: each cell
// adds its ends' accumulators after its pair sums, in link order.
// Finders: the non-symmetric all-pairs and Gabriel finders (naive and binned).
#ifndef TECS_CXX_PAIRWISE_CUH
#define TECS_CXX_PAIRWISE_CUH

#if !defined(__CUDACC__)
#error "tecs/pairwise.cuh needs nvcc (user force laws are compiled into the program's kernels)"
#endif
#if !defined(__CUDACC_EXTENDED_LAMBDA__)
#error "tecs/pairwise.cuh needs nvcc --extended-lambda (PAIRWISE_FORCE makes __host__ __device__ lambdas)"
#endif

#include <cstring>
#include <memory>

#include "device/kernels.cuh"
#include "tecs.hpp"

namespace tecs {
namespace detail {

// The laws in the form k_pass_law calls them: the values as the config's
// types, the running sums as the deltas, the law, the sums back.  G: the
// GENERIC_FORCE law or NoLaw; P: the PAIRWISE_FORCE law or NoLaw.
template <typename Config, typename G, typename P, typename L = NoLaw>
struct PairLaw {
  static constexpr bool kGeneric = !std::is_same_v<G, NoLaw>;
  static constexpr bool kPairwise = !std::is_same_v<P, NoLaw>;
  static constexpr bool kLink = !std::is_same_v<L, NoLaw>;
  G gen;
  P law;
  L link;

  // One of the cell's links (entry e of its link list) through the LINK_FORCE
  // law: the reference calls the law once per link with zeroed accumulators
  // for both ends and adds each end's accumulator to that end's delta, in
  // link order (integrators/base.hpp:196-233).  Here each end evaluates the
  // link and adds its own accumulator, so the law runs twice per link with
  // the same inputs and the same generator draws (keyed by the link's index).
  template <int D>
  __device__ void add(const PassArgs& a, unsigned n, unsigned id, const float* xs, float2 ps, unsigned e, float* s,
                      float* sp) const {
    if constexpr (kLink) {
      using Vector = VectorN<float, D>;
      using Fields = typename Config::template ForceFields<LinkFieldRef>;
      const uint2 le = a.link_ent[e];
      const bool b_end = (le.y & 1u) != 0u;
      // the other end's value: an id beyond the active cells reads an unused
      // view slot's zero
      float xo[3] = {0.f, 0.f, 0.f};
      float2 po = make_float2(0.f, 0.f);
      if (le.x < n) {
        const unsigned so = a.slot_of ? a.slot_of[le.x] : le.x;
        const float4 v = a.X[so];
        xo[0] = v.x; xo[1] = v.y; xo[2] = v.z;
        if (a.P) po = a.P[so];
      }
      Vector self, other, da, db;
      for (int d = 0; d < D; ++d) {
        self[d] = xs[d];
        other[d] = xo[d];
        da[d] = 0.f;
        db[d] = 0.f;
      }
      const Link lk{b_end ? le.x : id, b_end ? id : le.x};
      XorShiftRandom rng = XorShiftRandom::for_call(a.seed, a.ctr->step, a.full_step ? 5u : 6u, le.y >> 1, 0u);
      const Vector& va = b_end ? other : self;
      const Vector& vb = b_end ? self : other;
      if constexpr (Simulation<Config>::has_polarity) {
        const Polarity_<float> pself(ps.x, ps.y), pother(po.x, po.y);
        Polarity_<float> qa(0.f, 0.f), qb(0.f, 0.f);
        const Fields ctx{{va, vb, da, db}, {b_end ? pother : pself, b_end ? pself : pother, qa, qb}};
        link(a.full_step != 0, lk, rng, ctx);
        const Polarity_<float>& q = b_end ? qb : qa;
        sp[0] = sp[0] + q[0];
        sp[1] = sp[1] + q[1];
      } else {
        const Fields ctx{{va, vb, da, db}};
        link(a.full_step != 0, lk, rng, ctx);
      }
      const Vector& mine = b_end ? db : da;
      for (int d = 0; d < D; ++d) s[d] = s[d] + mine[d];
    }
  }

  __device__ void generic(const PassArgs& a, unsigned idi, const float* xi, float2 pi, Acc& acc) const {
    if constexpr (kGeneric) {
      constexpr int D = Config::dimensions;
      using Vector = VectorN<float, D>;
      using Fields = typename Config::template ForceFields<GenericFieldRef>;
      Vector self, delta;
      for (int d = 0; d < D; ++d) {
        self[d] = xi[d];
        delta[d] = acc.x[d];
      }
      XorShiftRandom rng = XorShiftRandom::for_call(a.seed, a.ctr->step, a.full_step ? 3u : 4u, idi, idi);
      if constexpr (Simulation<Config>::has_polarity) {
        const Polarity_<float> ps(pi.x, pi.y);
        Polarity_<float> pd(acc.p[0], acc.p[1]);
        const Fields ctx{{self, delta}, {ps, pd}};
        gen(a.full_step != 0, idi, rng, ctx);
        acc.p[0] = pd[0];
        acc.p[1] = pd[1];
      } else {
        const Fields ctx{{self, delta}};
        gen(a.full_step != 0, idi, rng, ctx);
      }
      for (int d = 0; d < D; ++d) acc.x[d] = delta[d];
    }
  }

  __device__ void operator()(const PassArgs& a, unsigned idi, unsigned idj, const float* xi, const float4& vj,
                             const float* disp, float dist, float2 pi, float2 pj, Acc& acc, DragAcc& dacc) const {
    if constexpr (!std::is_same_v<P, NoLaw>) {
      constexpr int D = Config::dimensions;
      using Vector = VectorN<float, D>;
      using Fields = typename Config::template ForceFields<PairwiseFieldRef>;
      Vector self, other, displacement, delta;
      const float xj[3] = {vj.x, vj.y, vj.z};
      for (int d = 0; d < D; ++d) {
        self[d] = xi[d];
        other[d] = xj[d];
        displacement[d] = disp[d];
        delta[d] = acc.x[d];
      }
      float drag = 0.f;
      XorShiftRandom rng = XorShiftRandom::for_call(a.seed, a.ctr->step, a.full_step ? 1u : 2u, idi, idj);
      if constexpr (Simulation<Config>::has_polarity) {
        const Polarity_<float> ps(pi.x, pi.y), po(pj.x, pj.y);
        Polarity_<float> pd(acc.p[0], acc.p[1]);
        const Fields ctx{{self, other, delta}, {ps, po, pd}};
        law(a.full_step != 0, idi, idj, displacement, dist, rng, drag, ctx);
        acc.p[0] = pd[0];
        acc.p[1] = pd[1];
      } else {
        const Fields ctx{{self, other, delta}};
        law(a.full_step != 0, idi, idj, displacement, dist, rng, drag, ctx);
      }
      for (int d = 0; d < D; ++d) acc.x[d] = delta[d];
      // total_drag += drag; total_velocity += drag * old_velocities(j)
      // (binned_gabriel.hpp:225-226); a simulation that keeps no old
      // velocities fails its next count or download when a law sets drag
      if (a.old_vel) {
        const float4 ov = a.old_vel[idj];
        const float o[3] = {ov.x, ov.y, ov.z};
        dacc.drag = dacc.drag + drag;
        for (int d = 0; d < D; ++d) dacc.v[d] = dacc.v[d] + drag * o[d];
      } else if (drag != 0.f) {
        atomicOr(&a.ctr->error, 2u);
      }
    }
  }
};

template <typename Config>
using FinderOf = typename Config::template PairFinderT<Config>;

// the launcher the library calls for every force evaluation; user is the
// binding, which holds the laws in device memory
template <typename Config, typename Law>
struct LawOnDevice {
  Law* dev = nullptr;
  alignas(Law) unsigned char host[sizeof(Law)] = {};
  bool valid = false;
  ~LawOnDevice() {
    if (dev) cudaFree(dev);
  }
};
template <typename Config, typename Law>
int pair_law_launcher(void* user, const void* call, void* stream) {
  static_assert(!FinderOf<Config>::symmetric && FinderOf<Config>::finder_id <= TECS_FINDER_NAIVE_DELAUNAY,
                "user laws run with the non-symmetric all-pairs, Gabriel and Delaunay finders");
  return launch_user_pass<Config::dimensions, FinderOf<Config>::finder_id>(
      static_cast<const UserPassCall*>(call), static_cast<cudaStream_t>(stream),
      static_cast<const LawOnDevice<Config, Law>*>(user)->dev);
}

template <typename Config, typename G, typename P, typename L>
struct PairLawBinding {
  using Law = PairLaw<Config, G, P, L>;
  using Bound = LawOnDevice<Config, Law>;
  // The step's graph launches the pass with a pointer to the laws in device
  // memory, so laws of the same types rebind by copying their values there
  // on the simulation's stream (ordered before its next step) -- no new
  // graph.  Values that compare equal byte for byte are not copied again.
  static void bind(tecs_sim* handle, int device, const G& g, const P& p, const L& l, std::shared_ptr<void>& holder,
                   tecs_pair_law_fn& bound) {
    const tecs_pair_law_fn fn = &pair_law_launcher<Config, Law>;
    const Law law{g, p, l};
    Bound* b = (holder && bound == fn) ? static_cast<Bound*>(holder.get()) : nullptr;
    if (!b) {
      if (prepare_user_pass<Config::dimensions, FinderOf<Config>::finder_id, Law>(device))
        throw Error("cannot load the user laws' pass on the device");
      auto next = std::make_shared<Bound>();
      if (cudaMalloc(reinterpret_cast<void**>(&next->dev), sizeof(Law)) != cudaSuccess)
        throw Error("cannot allocate the user laws on the device");
      check(tecs_sim_set_pair_law(handle, fn, next.get()));
      holder = next;
      bound = fn;
      b = next.get();
    }
    if (!b->valid || std::memcmp(b->host, &law, sizeof(Law)) != 0) {
      std::memcpy(b->host, &law, sizeof(Law));
      b->valid = true;
      if (cudaMemcpyAsync(b->dev, b->host, sizeof(Law), cudaMemcpyHostToDevice,
                          static_cast<cudaStream_t>(tecs_sim_stream(handle))) != cudaSuccess)
        throw Error("cannot copy the user laws to the device");
    }
  }
};

}  // namespace detail
}  // namespace tecs

// the reference's parameter list (utils.hpp:206-209); a law need not use them all
#define PAIRWISE_FORCE_PARAMETERS                                                                              \
  [[maybe_unused]] const bool is_full_step, [[maybe_unused]] const unsigned int i,                             \
      [[maybe_unused]] const unsigned int j, [[maybe_unused]] const Vector &displacement,                      \
      [[maybe_unused]] const Scalar distance, [[maybe_unused]] Random &rng, [[maybe_unused]] Scalar &drag,     \
      [[maybe_unused]] const PairwiseForceFields &ctx
#define PAIRWISE_REF(TYPE, NAME) tecs::detail::PairwiseFieldRef<TYPE> NAME

// a lambda factory, as the reference's: PAIRWISE_FORCE(body)() is the law
#define PAIRWISE_FORCE(...)                                                                                \
  [&]() {                                                                                                  \
    return tecs::detail::pairwise_force | [=] __host__ __device__(PAIRWISE_FORCE_PARAMETERS) { __VA_ARGS__ }; \
  }

// a functor's call operator: struct Law { PAIRWISE_FORCE_OP { body } };
#define PAIRWISE_FORCE_OP                     \
  using tag = tecs::detail::PairwiseForceTag; \
  __host__ __device__ void operator()(PAIRWISE_FORCE_PARAMETERS) const

// per-cell laws (integrators/base.hpp:116-142): ctx.<field>.self / .delta
#define GENERIC_FORCE_PARAMETERS                                                                   \
  [[maybe_unused]] const bool is_full_step, [[maybe_unused]] const unsigned int i,                 \
      [[maybe_unused]] Random &rng, [[maybe_unused]] const GenericForceFields &ctx
#define GENERIC_REF(TYPE, NAME) tecs::detail::GenericFieldRef<TYPE> NAME
#define GENERIC_FORCE(...)                                                                                \
  [&]() {                                                                                                 \
    return tecs::detail::generic_force | [=] __host__ __device__(GENERIC_FORCE_PARAMETERS) { __VA_ARGS__ }; \
  }
#define GENERIC_FORCE_OP                     \
  using tag = tecs::detail::GenericForceTag; \
  __host__ __device__ void operator()(GENERIC_FORCE_PARAMETERS) const

// per-link laws (utils.hpp:219-226): the link (a, b) and ctx.<field>.a / .b /
// .delta_a / .delta_b
#define LINK_FORCE_PARAMETERS                                                                        \
  [[maybe_unused]] const bool is_full_step, [[maybe_unused]] const tecs::Link &link,                 \
      [[maybe_unused]] Random &rng, [[maybe_unused]] const LinkForceFields &ctx
#define LINK_FORCE(...)                                                                                \
  [&]() {                                                                                              \
    return tecs::detail::link_force | [=] __host__ __device__(LINK_FORCE_PARAMETERS) { __VA_ARGS__ }; \
  }
#define LINK_FORCE_OP                     \
  using tag = tecs::detail::LinkForceTag; \
  __host__ __device__ void operator()(LINK_FORCE_PARAMETERS) const

#endif  // TECS_CXX_PAIRWISE_CUH
