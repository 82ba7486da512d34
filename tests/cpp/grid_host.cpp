// grid_host.cpp -- tecs::acceleration::Grid of the drop-in layer (host) on a
// grid-query fixture's inputs, with the fixture's stub generator: rand(a, b)
// = a + draw % (b - a), urand(r) = draw % r, so a draw picks its target
// exactly.  Writes the five query results as int32 rows.
//
//   grid_host <dims> <in.bin> <out.bin>
//   in:  uint32 n, uint32 m, float32 prm[16] (bin size, radius, min[3], max[3]),
//        float32 x[n*dims], float32 q[m*dims], uint32 draws[m]
//   out: int32 [m][5]: nearest (1 bin), nearest (2 bins), random in the 3^d
//        bins, random within the radius, the same among indices not divisible by 3
#include <cstdio>
#include <vector>

#include "tecs/tecs.hpp"

using namespace tecs;

struct DrawRng {
  unsigned draw = 0;
  int rand(int a, int b) const { return b > a ? a + static_cast<int>(draw % unsigned(b - a)) : a; }
  unsigned urand(unsigned r) const { return r ? draw % r : 0u; }
};

template <int D>
static int run(const char* in_path, const char* out_path) {
  using Vector = VectorN<float, D>;
  FILE* f = std::fopen(in_path, "rb");
  if (!f) return 2;
  unsigned nm[2];
  float prm[16];
  if (std::fread(nm, 4, 2, f) != 2 || std::fread(prm, 4, 16, f) != 16) return 2;
  const unsigned n = nm[0], m = nm[1];
  std::vector<float> x(std::size_t(n) * D), q(std::size_t(m) * D);
  std::vector<unsigned> draws(m);
  if (std::fread(x.data(), 4, x.size(), f) != x.size() || std::fread(q.data(), 4, q.size(), f) != q.size() ||
      std::fread(draws.data(), 4, m, f) != m)
    return 2;
  std::fclose(f);
  View<Vector> pts("points", n);
  for (unsigned i = 0; i < n; ++i)
    for (int d = 0; d < D; ++d) pts(i)[d] = x[std::size_t(i) * D + d];
  Vector mn, mx;
  for (int d = 0; d < D; ++d) {
    mn[d] = prm[2 + d];
    mx[d] = prm[5 + d];
  }
  acceleration::Grid<Vector> grid(pts, n, mn, mx, prm[0]);
  grid.rebuild();
  std::vector<int> out(std::size_t(m) * 5);
  for (unsigned k = 0; k < m; ++k) {
    Vector p;
    for (int d = 0; d < D; ++d) p[d] = q[std::size_t(k) * D + d];
    DrawRng rng{draws[k]};
    int* o = &out[std::size_t(k) * 5];
    o[0] = grid.get_nearest_point_index(p, 1);
    o[1] = grid.get_nearest_point_index(p, 2);
    o[2] = grid.get_random_point_index_in_neighbourhood_bins(p, 1, rng);
    o[3] = grid.get_random_point_index_in_neighbourhood(p, prm[1], rng);
    o[4] = grid.get_random_point_index_in_neighbourhood(p, prm[1], rng, [](int j) { return j % 3 != 0; });
  }
  FILE* g = std::fopen(out_path, "wb");
  if (!g) return 2;
  std::fwrite(out.data(), 4, out.size(), g);
  std::fclose(g);
  return 0;
}

int main(int argc, char** argv) {
  if (argc < 4) return 2;
  return argv[1][0] == '2' ? run<2>(argv[2], argv[3]) : run<3>(argv[2], argv[3]);
}
