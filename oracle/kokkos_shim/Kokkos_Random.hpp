// Kokkos_Random.hpp -- Random_XorShift64_Pool stand-in for the oracle's Kokkos
// shim.  The generator is Marsaglia's xorshift64* (one state per pool in this
// single-threaded shim); its stream is not Kokkos's, which the reference's
// results do not depend on except through initialisers and division, both of
// which the oracle replaces with its own counter-based RNG.
#pragma once
#include <cmath>
#include <cstdint>
#include <memory>

#include "Kokkos_Core.hpp"

namespace Kokkos {
template <class Device = Serial>
class Random_XorShift64 {
 public:
  explicit Random_XorShift64(uint64_t s = 1) : state_(s ? s : 0x9E3779B97F4A7C15ull) {}
  uint64_t urand64() {
    state_ ^= state_ >> 12;
    state_ ^= state_ << 25;
    state_ ^= state_ >> 27;
    return state_ * 0x2545F4914F6CDD1Dull;
  }
  uint32_t urand() { return (uint32_t)(urand64() >> 32); }
  uint32_t urand(uint32_t range) { return range ? urand() % range : 0u; }
  uint32_t urand(uint32_t a, uint32_t b) { return a + urand(b - a); }
  int rand() { return (int)(urand() >> 1); }
  int rand(int range) { return range > 0 ? rand() % range : 0; }
  int rand(int a, int b) { return a + rand(b - a); }
  double drand() { return (double)(urand64() >> 11) * (1.0 / 9007199254740992.0); }
  double drand(double range) { return drand() * range; }
  double drand(double a, double b) { return a + drand() * (b - a); }
  float frand() { return (float)drand(); }
  float frand(float range) { return frand() * range; }
  float frand(float a, float b) { return a + frand() * (b - a); }
  double normal() {
    double u1 = drand(), u2 = drand();
    if (u1 < 1e-300) u1 = 1e-300;
    return std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * 3.14159265358979323846 * u2);
  }
  double normal(double mean, double std_dev) { return mean + std_dev * normal(); }

 private:
  uint64_t state_;
};

// Copies of a pool share its state, as Kokkos's pools (which hold their
// generator states in a View) do: the reference's kernels capture the pool by
// value (KOKKOS_LAMBDA), and a state freed inside one must be the state the
// next kernel gets.
template <class Device = Serial>
class Random_XorShift64_Pool {
 public:
  using generator_type = Random_XorShift64<Device>;
  using device_type = Device;
  Random_XorShift64_Pool() : gen_(std::make_shared<generator_type>(1)) {}
  explicit Random_XorShift64_Pool(uint64_t seed)
      : gen_(std::make_shared<generator_type>(seed * 0x9E3779B97F4A7C15ull + 1ull)) {}
  generator_type get_state() const { return *gen_; }
  void free_state(const generator_type& g) const { *gen_ = g; }

 private:
  std::shared_ptr<generator_type> gen_;
};
}  // namespace Kokkos
