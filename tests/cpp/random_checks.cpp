// random_checks.cpp -- tecs::CounterRandom, the generator user laws get: the
// same key gives the same draws, keys that differ in any part give different
// streams, and the draws have the moments of their distributions.  Exits 0
// when every check holds, else prints the failing check.
#include <cmath>
#include <cstdio>
#include <set>

#include "tecs/random.hpp"

using tecs::CounterRandom;

static int fails = 0;
static void expect(bool ok, const char* what) {
  if (!ok) {
    std::printf("FAILED: %s\n", what);
    ++fails;
  }
}

int main() {
  {  // reproducible
    CounterRandom a = CounterRandom::for_call(2807, 12, 1, 5, 9), b = CounterRandom::for_call(2807, 12, 1, 5, 9);
    bool same = true;
    for (int k = 0; k < 1000; ++k) same = same && a.urand64() == b.urand64();
    expect(same, "the same key gives the same stream");
  }
  {  // every part of the key matters, and (i, j) is ordered
    std::set<unsigned long long> first;
    const unsigned long long keys[][5] = {{2807, 12, 1, 5, 9}, {2808, 12, 1, 5, 9}, {2807, 13, 1, 5, 9},
                                          {2807, 12, 2, 5, 9}, {2807, 12, 1, 6, 9}, {2807, 12, 1, 5, 10},
                                          {2807, 12, 1, 9, 5}};
    for (const auto& k : keys)
      first.insert(CounterRandom::for_call(k[0], k[1], unsigned(k[2]), unsigned(k[3]), unsigned(k[4])).urand64());
    expect(first.size() == 7, "keys that differ in one part start different streams");
  }
  {  // ranges and moments
    CounterRandom r(42);
    const int n = 200000;
    double sd = 0, sdd = 0, sf = 0, sn = 0, snn = 0, sn4 = 0;
    bool in_range = true;
    int counts[10] = {};
    for (int k = 0; k < n; ++k) {
      const double d = r.drand();
      const float f = r.frand();
      const double g = r.normal();
      const unsigned u = r.urand(10u);
      in_range = in_range && d >= 0.0 && d < 1.0 && f >= 0.0f && f < 1.0f && u < 10u;
      const double e = r.drand(-2.0, 3.0);
      in_range = in_range && e >= -2.0 && e < 3.0;
      sd += d; sdd += d * d; sf += f; sn += g; snn += g * g; sn4 += g * g * g * g;
      ++counts[u];
    }
    expect(in_range, "draws stay in their ranges");
    expect(std::fabs(sd / n - 0.5) < 0.005 && std::fabs(sdd / n - 1.0 / 3.0) < 0.005, "drand is uniform on [0, 1)");
    expect(std::fabs(sf / n - 0.5) < 0.005, "frand is uniform on [0, 1)");
    expect(std::fabs(sn / n) < 0.01 && std::fabs(snn / n - 1.0) < 0.02 && std::fabs(sn4 / n - 3.0) < 0.1,
           "normal has mean 0, variance 1 and kurtosis 3");
    bool flat = true;
    for (int c : counts) flat = flat && std::abs(c - n / 10) < n / 100;
    expect(flat, "urand(10) hits every value equally often");
    const double m = [&] {
      CounterRandom q(7);
      double s = 0;
      for (int k = 0; k < n; ++k) s += q.normal(2.0, 0.5);
      return s / n;
    }();
    expect(std::fabs(m - 2.0) < 0.01, "normal(mean, std_dev) shifts and scales");
  }
  return fails ? 1 : 0;
}
