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
#include <new>
#include <memory>
#include <utility>

#include "device/kernels.cuh"
#include "tecs.hpp"

namespace tecs {
namespace detail {

// A tuple usable in device code: one value per field.
template <std::size_t I, typename T>
struct TupLeaf {
  T v;
};
template <typename Seq, typename... T>
struct TupImpl;
template <std::size_t... I, typename... T>
struct TupImpl<std::index_sequence<I...>, T...> : TupLeaf<I, T>... {};
template <std::size_t I, typename T>
__host__ __device__ T& tget(TupLeaf<I, T>& leaf) {
  return leaf.v;
}
template <typename Layout, typename Seq>
struct ValuesOf;
template <typename Layout, std::size_t... I>
struct ValuesOf<Layout, std::index_sequence<I...>> {
  using type = TupImpl<std::index_sequence<I...>, typename Layout::template type<I>...>;
};

// The laws in the form k_pass_law calls them: the values as the config's
// types, the running sums as the deltas, the law, the sums back.  G: the
// GENERIC_FORCE law, P: the PAIRWISE_FORCE law, L: the LINK_FORCE law (NoLaw
// where absent).  Every field of the config is built from where the library
// holds it (FieldLayout: the position, the polarity, or the cell's extra
// block) into a value of the field's type, the law gets references to those,
// and the deltas go back.
template <typename Config, typename G, typename P, typename L = NoLaw>
struct PairLaw {
  static constexpr bool kGeneric = !std::is_same_v<G, NoLaw>;
  static constexpr bool kPairwise = !std::is_same_v<P, NoLaw>;
  static constexpr bool kLink = !std::is_same_v<L, NoLaw>;
  static constexpr int D = Config::dimensions;
  using Layout = FieldLayout<typename Config::Fields>;
  static constexpr unsigned kExtra = Layout::extra;
  static_assert(kExtra <= kMaxExtra, "at most 8 float components of extra fields");
  using Cell = LawCell<kExtra>;
  using Values = typename ValuesOf<Layout, std::make_index_sequence<Layout::n>>::type;
  G gen;
  P law;
  L link;

  // field k of one cell from the library's arrays: its position (xyz), its
  // polarity (p) or its extra components (ex)
  template <std::size_t K>
  __device__ static void load(typename Layout::template type<K>& v, const float* xyz, float2 p, const float* ex) {
    if constexpr (Layout::role(K) == 0) {
      for (int d = 0; d < D; ++d) v[d] = xyz[d];
    } else if constexpr (Layout::role(K) == 1) {
      v[0] = p.x;
      v[1] = p.y;
    } else {
      constexpr unsigned o = Layout::offset(K);
      if constexpr (FieldWidth<typename Layout::template type<K>>::scalar) v = ex[o];
      else
        for (unsigned c = 0; c < FieldWidth<typename Layout::template type<K>>::value; ++c) v[c] = ex[o + c];
    }
  }
  // field k's delta back into the sums
  template <std::size_t K>
  __device__ static void store(const typename Layout::template type<K>& v, float* x, float* p, float* ex) {
    if constexpr (Layout::role(K) == 0) {
      for (int d = 0; d < D; ++d) x[d] = v[d];
    } else if constexpr (Layout::role(K) == 1) {
      p[0] = v[0];
      p[1] = v[1];
    } else {
      constexpr unsigned o = Layout::offset(K);
      if constexpr (FieldWidth<typename Layout::template type<K>>::scalar) ex[o] = v;
      else
        for (unsigned c = 0; c < FieldWidth<typename Layout::template type<K>>::value; ++c) ex[o + c] = v[c];
    }
  }
  template <typename F, std::size_t... I>
  __device__ static void each(F&& f, std::index_sequence<I...>) {
    (f(std::integral_constant<std::size_t, I>{}), ...);
  }
  template <typename F>
  __device__ static void each(F&& f) {
    each(static_cast<F&&>(f), std::make_index_sequence<Layout::n>{});
  }
  // the extra components of slot j of the pass's input
  __device__ static void load_extra(const PassArgs& a, unsigned j, float* ex) {
    if constexpr (kExtra > 0)
      for (unsigned k = 0; k < kExtra; ++k) ex[k] = a.EX[k * (size_t)a.capacity + j];
  }

  __device__ void generic(const PassArgs& a, unsigned idi, const float* xi, float2 pi, Acc& acc, const float* exi,
                          float* exd) const {
    if constexpr (kGeneric) {
      using Fields = typename Config::template ForceFields<GenericFieldRef>;
      Values self{}, delta{};
      each([&](auto k) {
        load<k>(tget<k>(self), xi, pi, exi);
        load<k>(tget<k>(delta), acc.x, make_float2(acc.p[0], acc.p[1]), exd);
      });
      XorShiftRandom rng = XorShiftRandom::for_call(a.seed, a.ctr->step, a.full_step ? 3u : 4u, idi, idi);
      [&]<std::size_t... I>(std::index_sequence<I...>) {
        const Fields ctx{GenericFieldRef<typename Layout::template type<I>>{tget<I>(self), tget<I>(delta)}...};
        gen(a.full_step != 0, idi, rng, ctx);
      }(std::make_index_sequence<Layout::n>{});
      each([&](auto k) { store<k>(tget<k>(delta), acc.x, acc.p, exd); });
    }
  }

  __device__ void operator()(const PassArgs& a, unsigned idi, unsigned idj, unsigned j, const float* xi,
                             const float4& vj, const float* disp, float dist, float2 pi, float2 pj, Acc& acc,
                             Cell& cell) const {
    if constexpr (kPairwise) {
      using Fields = typename Config::template ForceFields<PairwiseFieldRef>;
      using Vector = VectorN<float, D>;
      Values self{}, other{}, delta{};
      const float xj[3] = {vj.x, vj.y, vj.z};
      float exj[kExtra > 0 ? kExtra : 1];
      load_extra(a, j, exj);
      each([&](auto k) {
        load<k>(tget<k>(self), xi, pi, cell.ex_self);
        load<k>(tget<k>(other), xj, pj, exj);
        load<k>(tget<k>(delta), acc.x, make_float2(acc.p[0], acc.p[1]), cell.ex_delta);
      });
      Vector displacement;
      for (int d = 0; d < D; ++d) displacement[d] = disp[d];
      float drag = 0.f;
      XorShiftRandom rng = XorShiftRandom::for_call(a.seed, a.ctr->step, a.full_step ? 1u : 2u, idi, idj);
      [&]<std::size_t... I>(std::index_sequence<I...>) {
        const Fields ctx{PairwiseFieldRef<typename Layout::template type<I>>{tget<I>(self), tget<I>(other),
                                                                             tget<I>(delta)}...};
        law(a.full_step != 0, idi, idj, displacement, dist, rng, drag, ctx);
      }(std::make_index_sequence<Layout::n>{});
      each([&](auto k) { store<k>(tget<k>(delta), acc.x, acc.p, cell.ex_delta); });
      // total_drag += drag; total_velocity += drag * old_velocities(j)
      // (binned_gabriel.hpp:225-226); a simulation that keeps no old
      // velocities fails its next count or download when a law sets drag
      if (a.old_vel) {
        const float4 ov = a.old_vel[idj];
        const float o[3] = {ov.x, ov.y, ov.z};
        cell.drag = cell.drag + drag;
        for (int d = 0; d < D; ++d) cell.v[d] = cell.v[d] + drag * o[d];
      } else if (drag != 0.f) {
        atomicOr(&a.ctr->error, 2u);
      }
    }
  }

  // One of the cell's links (entry e of its link list) through the LINK_FORCE
  // law: the reference calls the law once per link with zeroed accumulators
  // for both ends and adds each end's accumulator to that end's delta, in
  // link order (integrators/base.hpp:196-233).  Here each end evaluates the
  // link and adds its own accumulator, so the law runs twice per link with
  // the same inputs and the same generator draws (keyed by the link's index).
  template <int DD>
  __device__ void add(const PassArgs& a, unsigned n, unsigned id, const float* xs, float2 ps, unsigned e, float* s,
                      float* sp, float* se) const {
    if constexpr (kLink) {
      using Fields = typename Config::template ForceFields<LinkFieldRef>;
      const uint2 le = a.link_ent[e];
      const bool b_end = (le.y & 1u) != 0u;
      // the other end's values: an id beyond the active cells reads an unused
      // view slot's zero
      float xo[3] = {0.f, 0.f, 0.f};
      float2 po = make_float2(0.f, 0.f);
      float exo[kExtra > 0 ? kExtra : 1] = {};
      float exs[kExtra > 0 ? kExtra : 1] = {};
      const unsigned self_slot = a.slot_of ? a.slot_of[id] : id;
      load_extra(a, self_slot, exs);
      if (le.x < n) {
        const unsigned so = a.slot_of ? a.slot_of[le.x] : le.x;
        const float4 v = a.X[so];
        xo[0] = v.x; xo[1] = v.y; xo[2] = v.z;
        if (a.P) po = a.P[so];
        load_extra(a, so, exo);
      }
      Values va{}, vb{}, da{}, db{};
      const float zeros[3 + kMaxExtra] = {};
      each([&](auto k) {
        load<k>(tget<k>(va), b_end ? xo : xs, b_end ? po : ps, b_end ? exo : exs);
        load<k>(tget<k>(vb), b_end ? xs : xo, b_end ? ps : po, b_end ? exs : exo);
        load<k>(tget<k>(da), zeros, make_float2(0.f, 0.f), zeros);
        load<k>(tget<k>(db), zeros, make_float2(0.f, 0.f), zeros);
      });
      const Link lk{b_end ? le.x : id, b_end ? id : le.x};
      XorShiftRandom rng = XorShiftRandom::for_call(a.seed, a.ctr->step, a.full_step ? 5u : 6u, le.y >> 1, 0u);
      [&]<std::size_t... I>(std::index_sequence<I...>) {
        const Fields ctx{LinkFieldRef<typename Layout::template type<I>>{tget<I>(va), tget<I>(vb),
                                                                         tget<I>(da), tget<I>(db)}...};
        link(a.full_step != 0, lk, rng, ctx);
      }(std::make_index_sequence<Layout::n>{});
      // this end's accumulator added to its sums, in link order
      float mx[3] = {0.f, 0.f, 0.f}, mp[2] = {0.f, 0.f}, me[kExtra > 0 ? kExtra : 1] = {};
      each([&](auto k) { store<k>(b_end ? tget<k>(db) : tget<k>(da), mx, mp, me); });
      for (int d = 0; d < DD; ++d) s[d] = s[d] + mx[d];
      if (a.P) {
        sp[0] = sp[0] + mp[0];
        sp[1] = sp[1] + mp[1];
      }
      if constexpr (kExtra > 0)
        for (unsigned k = 0; k < kExtra; ++k) se[k] = se[k] + me[k];
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
    // built in zeroed storage, so that padding between the members compares
    // equal from one step to the next (padding inside the captured closures
    // is copied as it is; unequal padding only costs one more copy)
    alignas(Law) unsigned char storage[sizeof(Law)];
    std::memset(storage, 0, sizeof(Law));
    struct Built {
      Law* p;
      ~Built() { p->~Law(); }
    } built{::new (static_cast<void*>(storage)) Law{g, p, l}};
    const Law& law = *built.p;
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
