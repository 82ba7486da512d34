// The Delaunay star finder (tecs/device/delaunay_star.cuh) compiled for the
// host, for the tests: reads "n dims cutoff" and n rows of x y z from stdin,
// bins the points as the device does, and prints one line "i j reps" per
// applied pair (ascending i, then j), then "err <bits>" with the OR of every
// cell's error bits (and "cellerr i bits" for every cell with some).
#include <cstdio>
#include <vector>

#include "tecs/device/delaunay_star.cuh"

using namespace tecs::dl;

template <int D>
static int run(unsigned n, float cutoff, std::vector<Pt>& P) {
  Grid g{};
  double mn[3] = {0, 0, 0}, mx[3] = {0, 0, 0};
  for (int d = 0; d < D; ++d) {
    mn[d] = 1e300;
    mx[d] = -1e300;
  }
  for (unsigned i = 0; i < n; ++i) {
    const double q[3] = {P[i].x, P[i].y, P[i].z};
    for (int d = 0; d < D; ++d) {
      if (q[d] < mn[d]) mn[d] = q[d];
      if (q[d] > mx[d]) mx[d] = q[d];
    }
  }
  if (n == 0)
    for (int d = 0; d < D; ++d) mn[d] = mx[d] = 0.0;
  plan_grid<D>(g, mn, mx, n, n + 64u);
  std::vector<unsigned> cnt(g.nbins + 1, 0u), key(n), idx(n);
  for (unsigned i = 0; i < n; ++i) {
    const double q[3] = {P[i].x, P[i].y, P[i].z};
    int b[3];
    bin_of<D>(g, q, b);
    key[i] = flat(g, b[0], b[1], b[2]);
    cnt[key[i]] += 1u;
  }
  std::vector<unsigned> off(g.nbins + 1, 0u);
  for (unsigned b = 0; b < g.nbins; ++b) off[b + 1] = off[b] + cnt[b];
  std::vector<unsigned> cur(off.begin(), off.end() - 1);
  std::vector<Pt> sp(n);
  for (unsigned i = 0; i < n; ++i) {
    const unsigned at = cur[key[i]]++;
    idx[at] = i;
    sp[at] = P[i];
  }
  g.off = off.data();
  g.idx = idx.data();
  g.sp = sp.data();
  g.P = P.data();
  g.n = n;
  g.rc2 = cutoff * cutoff;
  static Scratch sc;
  unsigned oj[64], orr[64], err_all = 0;
  for (unsigned i = 0; i < n; ++i) {
    unsigned err = 0;
    const unsigned len = cell_mult<D>(Solo{}, g, i, oj, orr, 64, &err, sc);
    err_all |= err;
    if (err) std::printf("cellerr %u %u\n", i, err);
    for (unsigned t = 0; t < len; ++t) std::printf("%u %u %u\n", i, oj[t], orr[t]);
  }
  std::printf("err %u\n", err_all);
  return 0;
}

int main() {
  unsigned n = 0;
  int dims = 0;
  float cutoff = 0.f;
  if (std::scanf("%u %d %f", &n, &dims, &cutoff) != 3) return 2;
  std::vector<Pt> P(n);
  for (unsigned i = 0; i < n; ++i) {
    float x, y, z;
    if (std::scanf("%f %f %f", &x, &y, &z) != 3) return 2;
    P[i] = Pt{x, y, z, 0.f};
  }
  return dims == 2 ? run<2>(n, cutoff, P) : run<3>(n, cutoff, P);
}
