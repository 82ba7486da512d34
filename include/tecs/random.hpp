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

}  // namespace tecs

#endif  // TECS_CXX_RANDOM_HPP
