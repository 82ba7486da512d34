// tecs/random.hpp -- the Random generator handed to user force laws.
//
// The reference passes each force call a Kokkos Random_XorShift64 state taken
// from a pool (include/utils/utils.hpp:208-209, pair_finders/*.hpp
// random_pool.get_state / free_state), so its draws depend on which pool
// state a thread happens to get.  Here every call gets a generator keyed by
// (seed, step, pass, cell ids): the draws are reproducible from run to run
// and independent of the launch shape.  The member functions are those the
// reference's programs call on it (urand, rand, drand, frand, normal).
//
// The stream is SplitMix64 (Steele, Lea and Flood, "Fast splittable
// pseudorandom number generators", OOPSLA 2014): a Weyl sequence with step
// 0x9e3779b97f4a7c15 through the variant-13 finaliser of MurmurHash3.
#ifndef TECS_CXX_RANDOM_HPP
#define TECS_CXX_RANDOM_HPP

#include <cmath>
#include <cstdint>

#include "vector.hpp"

namespace tecs {

class CounterRandom {
 public:
  TECS_HD explicit CounterRandom(std::uint64_t key) : state_(key) {}
  // a generator for (seed, step, pass, i, j): the key mixes each part through the finaliser
  TECS_HD static CounterRandom for_call(std::uint64_t seed, std::uint64_t step, unsigned pass, unsigned i,
                                        unsigned j) {
    std::uint64_t k = mix(seed ^ 0x243f6a8885a308d3ull);
    k = mix(k ^ step);
    k = mix(k ^ ((std::uint64_t(pass) << 32) | i));
    k = mix(k ^ j);
    return CounterRandom(k);
  }

  TECS_HD std::uint64_t urand64() {
    state_ += 0x9e3779b97f4a7c15ull;
    return mix(state_);
  }
  TECS_HD std::uint32_t urand() { return static_cast<std::uint32_t>(urand64() >> 32); }
  TECS_HD std::uint32_t urand(std::uint32_t range) { return range ? urand() % range : 0u; }
  TECS_HD std::uint32_t urand(std::uint32_t start, std::uint32_t end) { return start + urand(end - start); }
  TECS_HD int rand() { return static_cast<int>(urand() >> 1); }
  TECS_HD int rand(int range) { return range > 0 ? rand() % range : 0; }
  TECS_HD int rand(int start, int end) { return start + rand(end - start); }
  // uniform in [0, 1): the top 53 (double) or 24 (float) bits
  TECS_HD double drand() { return static_cast<double>(urand64() >> 11) * (1.0 / 9007199254740992.0); }
  TECS_HD double drand(double range) { return range * drand(); }
  TECS_HD double drand(double start, double end) { return start + (end - start) * drand(); }
  TECS_HD float frand() { return static_cast<float>(urand() >> 8) * (1.0f / 16777216.0f); }
  TECS_HD float frand(float range) { return range * frand(); }
  TECS_HD float frand(float start, float end) { return start + (end - start) * frand(); }
  // standard normal by the Box-Muller transform, one value per two uniforms
  TECS_HD double normal() {
    const double u1 = 1.0 - drand();  // (0, 1]
    const double u2 = drand();
    return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
  }
  TECS_HD double normal(double mean, double std_dev) { return mean + std_dev * normal(); }

 private:
  TECS_HD static std::uint64_t mix(std::uint64_t z) {
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
  }
  std::uint64_t state_;
};

// The Random of the drop-in layer's configs (the reference's programs take
// `Random& rng` in their laws and initialisers): Marsaglia's xorshift
// generator with Vigna's multiplicative output (xorshift64*, "An experimental
// exploration of Marsaglia's xorshift generators, scrambled", 2016), with the
// draws of Kokkos's generator interface (urand, rand, drand, frand, normal).
// The initialisers run on the host in cell order from one pool state, seeded
// from Settings::seed -- the order in which the reference's Serial backend
// hands its pool state from cell to cell -- and a law on the device gets a
// generator keyed by (seed, step, evaluation, i, j).
class XorShiftRandom {
 public:
  TECS_HD explicit XorShiftRandom(std::uint64_t state = 1) : state_(state ? state : 0x9E3779B97F4A7C15ull) {}
  TECS_HD static XorShiftRandom for_call(std::uint64_t seed, std::uint64_t step, unsigned pass, unsigned i,
                                         unsigned j) {
    CounterRandom c = CounterRandom::for_call(seed, step, pass, i, j);
    return XorShiftRandom(c.urand64());
  }
  TECS_HD std::uint64_t urand64() {
    state_ ^= state_ >> 12;
    state_ ^= state_ << 25;
    state_ ^= state_ >> 27;
    return state_ * 0x2545F4914F6CDD1Dull;
  }
  TECS_HD std::uint32_t urand() { return static_cast<std::uint32_t>(urand64() >> 32); }
  TECS_HD std::uint32_t urand(std::uint32_t range) { return range ? urand() % range : 0u; }
  TECS_HD std::uint32_t urand(std::uint32_t start, std::uint32_t end) { return start + urand(end - start); }
  TECS_HD int rand() { return static_cast<int>(urand() >> 1); }
  TECS_HD int rand(int range) { return range > 0 ? rand() % range : 0; }
  TECS_HD int rand(int start, int end) { return start + rand(end - start); }
  // uniform in [0, 1): the top 53 bits
  TECS_HD double drand() { return static_cast<double>(urand64() >> 11) * (1.0 / 9007199254740992.0); }
  TECS_HD double drand(double range) { return drand() * range; }
  TECS_HD double drand(double start, double end) { return start + drand() * (end - start); }
  TECS_HD float frand() { return static_cast<float>(drand()); }
  TECS_HD float frand(float range) { return frand() * range; }
  TECS_HD float frand(float start, float end) { return start + frand() * (end - start); }
  // standard normal by the Box-Muller transform
  TECS_HD double normal() {
    double u1 = drand();
    const double u2 = drand();
    if (u1 < 1e-300) u1 = 1e-300;
    return sqrt(-2.0 * log(u1)) * cos(2.0 * 3.14159265358979323846 * u2);
  }
  TECS_HD double normal(double mean, double std_dev) { return mean + std_dev * normal(); }

 private:
  std::uint64_t state_;
};

// The pool a config's RandomPool names: one state, handed out and taken back
// in turn (Kokkos::Random_XorShift64_Pool's interface, single-threaded).
class XorShiftPool {
 public:
  using generator_type = XorShiftRandom;
  XorShiftPool() = default;
  explicit XorShiftPool(std::uint64_t seed) : gen_(seed * 0x9E3779B97F4A7C15ull + 1ull) {}
  generator_type get_state() const { return gen_; }
  void free_state(const generator_type& g) const { gen_ = g; }

 private:
  mutable generator_type gen_{1};
};

}  // namespace tecs

#endif  // TECS_CXX_RANDOM_HPP
