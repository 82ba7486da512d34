// tecs/config.hpp -- simulation configs for the C++20 drop-in layer.
//
// A config is a struct deriving from DefaultSimulationConfig that overrides
// members through the reference's CONFIG_* macros and ends with
// RESOLVE_TECS_CONFIG(), or is made in one go with CREATE_SIMULATION_CONFIG;
// user programs name them, so the macro names and what they declare
// (Scalar, dimensions, PairFinderT, IntegratorT, ComFixerT, WriterT, Fields,
// Vector, Polarity) follow include/simulation_config.hpp:212-379 and
// include/utils/utils.hpp:319-344.  The field list is resolved against the
// final Scalar and dimensions when RESOLVE_TECS_CONFIG() runs, so overrides
// may come in any order before it.
#ifndef TECS_CXX_CONFIG_HPP
#define TECS_CXX_CONFIG_HPP

#include <cstddef>
#include <string_view>
#include <tuple>
#include <type_traits>

#include "components.hpp"
#include "hdf5_writer.hpp"
#include "plane.hpp"
#include "random.hpp"
#include "vector.hpp"

namespace tecs {

template <typename T>
class View;

namespace detail {

// a string literal usable as a template argument (the field's name)
template <std::size_t N>
struct FixedString {
  char text[N] = {};
  constexpr FixedString(const char (&s)[N]) {
    for (std::size_t k = 0; k < N; ++k) text[k] = s[k];
  }
  constexpr std::string_view view() const { return {text, N - 1}; }
};

template <typename T, FixedString Name>
struct Field {
  using value_type = T;
  static constexpr std::string_view name = Name.view();
};

template <typename... Fs>
struct FieldList {
  static constexpr std::size_t size = sizeof...(Fs);
};

// What a force law sees of one field (include/forces/detail.hpp:185-206): a
// config's ForceFields<Ref> has one such member per field, named as the field.
template <typename T>
struct GenericFieldRef {
  const T& self;  // the agent's value
  T& delta;       // its delta, written by the law
};
template <typename T>
struct PairwiseFieldRef {
  const T& self;   // agent i's value
  const T& other;  // agent j's value
  T& delta;        // i's delta, written by the law
};
// a link's two ends (forces/detail.hpp: LinkFieldRef)
template <typename T>
struct LinkFieldRef {
  const T& a;
  const T& b;
  T& delta_a;
  T& delta_b;
};

// How the library holds a config's fields: the first field is the position
// (a Vector); a (Polarity, polarity) field is the library's polarity (the
// built-in polarity law reads it); every other field is an extra field, its
// float components packed one after another (Scalar 1, Polarity 2, Vector D)
// into the cell's extra block.  role: 0 position, 1 polarity, 2 extra.
template <typename T>
struct FieldWidth;
template <typename S, int D>
struct FieldWidth<VectorN<S, D>> {
  static constexpr unsigned value = D;
  static constexpr bool scalar = false;
};
template <typename S>
struct FieldWidth<Polarity_<S>> {
  static constexpr unsigned value = 2;
  static constexpr bool scalar = false;
};
template <>
struct FieldWidth<float> {
  static constexpr unsigned value = 1;
  static constexpr bool scalar = true;  // updated in double by the reference's integrators
};

template <typename List>
struct FieldLayout;
template <typename... Fs>
struct FieldLayout<FieldList<Fs...>> {
  static constexpr std::size_t n = sizeof...(Fs);
  template <std::size_t I>
  using type = typename std::tuple_element_t<I, std::tuple<Fs...>>::value_type;

 private:
  static constexpr bool is_pol[n] = {(std::is_same_v<typename Fs::value_type, Polarity_<float>> &&
                                      Fs::name == "polarity")...};
  static constexpr unsigned width[n] = {FieldWidth<typename Fs::value_type>::value...};
  static constexpr bool scalar[n] = {FieldWidth<typename Fs::value_type>::scalar...};
  TECS_HD static constexpr std::size_t first_polarity() {
    for (std::size_t k = 1; k < n; ++k)
      if (is_pol[k]) return k;
    return n;
  }

 public:
  static constexpr std::size_t polarity_index = first_polarity();  // n: none
  static constexpr bool has_polarity = polarity_index < n;
  TECS_HD static constexpr int role(std::size_t k) { return k == 0 ? 0 : k == polarity_index ? 1 : 2; }
  // the field's first component in the extra block (extra fields only)
  TECS_HD static constexpr unsigned offset(std::size_t k) {
    unsigned o = 0;
    for (std::size_t q = 0; q < k; ++q)
      if (role(q) == 2) o += width[q];
    return o;
  }
  static constexpr unsigned extra = offset(n);
  TECS_HD static constexpr unsigned double_mask() {
    unsigned m = 0;
    for (std::size_t q = 0; q < n; ++q)
      if (role(q) == 2 && scalar[q]) m |= 1u << offset(q);
    return m;
  }
};

// bind a finder template to the config's position view, scalar and dimensions
template <template <typename, typename, int> class Finder, typename Config>
using pair_finder_t =
    Finder<View<VectorN<typename Config::Scalar, Config::dimensions>>, typename Config::Scalar, Config::dimensions>;

}  // namespace detail
}  // namespace tecs

#define FIELD(TYPE, NAME) tecs::detail::Field<TYPE, #NAME>

#define CONFIG_SCALAR(S) using Scalar = S;
#define CONFIG_DIMENSIONS(D) static constexpr int dimensions = D;
// the drop-in layer's generator (tecs::XorShiftPool) serves every config
#define CONFIG_RANDOM_POOL(POOL)
#define CONFIG_INTEGRATOR(I) \
  template <typename SimulationConfig_> \
  using IntegratorT = I<SimulationConfig_>;
#define CONFIG_PAIR_FINDER(F) \
  template <typename SimulationConfig_> \
  using PairFinderT = tecs::detail::pair_finder_t<F, SimulationConfig_>;
#define CONFIG_COM_FIXER(C) \
  template <typename SimulationConfig_> \
  using ComFixerT = C<SimulationConfig_>;
#define CONFIG_WRITER(W) \
  template <typename SimulationConfig_> \
  using WriterT = W<SimulationConfig_>;

// (Type, name) pairs; Type is Vector, Polarity or Scalar of the final config
#define TECS_CXX_CAT(a, b) TECS_CXX_CAT_(a, b)
#define TECS_CXX_CAT_(a, b) a##b
#define TECS_CXX_NARG(...) TECS_CXX_NARG_(__VA_ARGS__, 4, 3, 2, 1, 0)
#define TECS_CXX_NARG_(a, b, c, d, n, ...) n
#define TECS_CXX_TYPE_Vector(S, D) tecs::VectorN<S, D>
#define TECS_CXX_TYPE_Polarity(S, D) tecs::Polarity_<S>
#define TECS_CXX_TYPE_Scalar(S, D) S
#define TECS_CXX_FIELD_OF(T, N) tecs::detail::Field<TECS_CXX_TYPE_##T(TecsScalar_, TecsDims_), #N>
#define TECS_CXX_APPLY(P) TECS_CXX_FIELD_OF P
#define TECS_CXX_LIST_1(a) TECS_CXX_APPLY(a)
#define TECS_CXX_LIST_2(a, b) TECS_CXX_APPLY(a), TECS_CXX_APPLY(b)
#define TECS_CXX_LIST_3(a, b, c) TECS_CXX_APPLY(a), TECS_CXX_APPLY(b), TECS_CXX_APPLY(c)
#define TECS_CXX_LIST_4(a, b, c, d) TECS_CXX_APPLY(a), TECS_CXX_APPLY(b), TECS_CXX_APPLY(c), TECS_CXX_APPLY(d)
// one member per field of a ForceFields<Ref> struct
#define TECS_CXX_REF_OF(T, N) TecsRef_<TECS_CXX_TYPE_##T(TecsScalar_, TecsDims_)> N;
#define TECS_CXX_REF_APPLY(P) TECS_CXX_REF_OF P
#define TECS_CXX_REFS_1(a) TECS_CXX_REF_APPLY(a)
#define TECS_CXX_REFS_2(a, b) TECS_CXX_REF_APPLY(a) TECS_CXX_REF_APPLY(b)
#define TECS_CXX_REFS_3(a, b, c) TECS_CXX_REF_APPLY(a) TECS_CXX_REF_APPLY(b) TECS_CXX_REF_APPLY(c)
#define TECS_CXX_REFS_4(a, b, c, d) TECS_CXX_REF_APPLY(a) TECS_CXX_REF_APPLY(b) TECS_CXX_REF_APPLY(c) TECS_CXX_REF_APPLY(d)

#define CONFIG_FIELDS(...)                                                                            \
  template <typename TecsScalar_, int TecsDims_>                                                      \
  struct TecsFieldsOf_ {                                                                              \
    using type = tecs::detail::FieldList<TECS_CXX_CAT(TECS_CXX_LIST_, TECS_CXX_NARG(__VA_ARGS__))(__VA_ARGS__)>; \
    template <template <typename> class TecsRef_>                                                     \
    struct ForceFields {                                                                              \
      TECS_CXX_CAT(TECS_CXX_REFS_, TECS_CXX_NARG(__VA_ARGS__))(__VA_ARGS__)                            \
    };                                                                                                \
  };

#define RESOLVE_TECS_CONFIG()                                                                \
  using Vector = tecs::VectorN<Scalar, dimensions>;                                          \
  using Polarity = tecs::Polarity_<Scalar>;                                                  \
  using VectorView = tecs::View<Vector>;                                                     \
  using Fields = typename TecsFieldsOf_<Scalar, dimensions>::type;                           \
  template <template <typename> class TecsRef_>                                              \
  using ForceFields = typename TecsFieldsOf_<Scalar, dimensions>::template ForceFields<TecsRef_>;

namespace tecs {

struct DefaultSimulationConfig {
  CONFIG_DIMENSIONS(3)
  CONFIG_SCALAR(float)
  CONFIG_PAIR_FINDER(tecs::pair_finders::NaiveAllPairs)
  CONFIG_COM_FIXER(tecs::com_fixers::NoComFixer)
  CONFIG_INTEGRATOR(tecs::integrators::Heun)
  CONFIG_WRITER(tecs::io::HDF5_Writer)
  CONFIG_FIELDS((Vector, position))
  RESOLVE_TECS_CONFIG()
};

}  // namespace tecs

#define CREATE_SIMULATION_CONFIG(NAME, ...)                \
  struct NAME : public tecs::DefaultSimulationConfig {     \
    __VA_ARGS__                                            \
    RESOLVE_TECS_CONFIG()                                  \
  };

#define EXTRACT_TYPES_FROM_SIMULATION_CONFIG(C)                                                                  \
  using Scalar [[maybe_unused]] = typename C::Scalar;                                                            \
  [[maybe_unused]] static constexpr int dimensions = C::dimensions;                                              \
  using Vector [[maybe_unused]] = tecs::VectorN<Scalar, dimensions>;                                             \
  using VectorI [[maybe_unused]] = tecs::VectorN<int, dimensions>;                                               \
  using VectorView [[maybe_unused]] = tecs::View<Vector>;                                                        \
  using Polarity [[maybe_unused]] = tecs::Polarity_<Scalar>;                                                     \
  using Plane [[maybe_unused]] = tecs::PlaneN<Scalar, dimensions>;                                               \
  using RandomPool [[maybe_unused]] = tecs::XorShiftPool;                                                        \
  using Random [[maybe_unused]] = tecs::XorShiftRandom;                                                          \
  using GenericForceFields [[maybe_unused]] = typename C::template ForceFields<tecs::detail::GenericFieldRef>;   \
  using PairwiseForceFields [[maybe_unused]] = typename C::template ForceFields<tecs::detail::PairwiseFieldRef>; \
  using LinkForceFields [[maybe_unused]] = typename C::template ForceFields<tecs::detail::LinkFieldRef>;

#define EXTRACT_ALL_FROM_SIMULATION_CONFIG(C)                                                                    \
  EXTRACT_TYPES_FROM_SIMULATION_CONFIG(C)                                                                        \
  using Fields [[maybe_unused]] = typename C::Fields;                                                            \
  using Integrator [[maybe_unused]] = typename C::template IntegratorT<C>;                                       \
  using PairFinder [[maybe_unused]] = typename C::template PairFinderT<C>;                                       \
  using ComFixer [[maybe_unused]] = typename C::template ComFixerT<C>;                                           \
  using Writer [[maybe_unused]] = typename C::template WriterT<C>;

#endif  // TECS_CXX_CONFIG_HPP
