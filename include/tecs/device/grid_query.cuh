// grid_query.cuh -- device-side queries of a uniform bin grid (sm_103a).
//
// The counterpart of acceleration::Grid's query functions
// (include/utils/grid.hpp:413-637): over points sorted by (bin, index) --
// B holds the sorted positions, Bid their indices, off the bin offsets
// (off[nbins] = the point count) -- the bins of a (2r+1)^d block around a
// point's bin are visited in the reference's task order (x fastest,
// grid.hpp:307-340), skipping bins outside the grid (:346-373), and each bin's
// points in ascending index, as the reference's BinSort lists them.  Distances
// are VectorN::distance_to_squared (vector.hpp:336-343).  A random pick takes
// the target-th eligible point, target = draw mod (number of eligible points),
// where the reference draws rng.rand(0, total) / rng.urand(total); a caller
// holding a generator passes its draw.
#pragma once

#include <cfloat>

#include "common.cuh"

namespace tecs {

struct GridDev {
  GridP g;
  int dims;
  const float4* B;       // sorted positions (w: bin key)
  const unsigned* Bid;   // index of each sorted slot
  const unsigned* off;   // bin offsets, nbins + 1
};

__host__ __device__ __forceinline__ int gq_clamp(int v, int hi) { return v < hi ? (v < 0 ? 0 : v) : hi; }

// grid.hpp:222-230: truncating division, clamped into the grid
__host__ __device__ __forceinline__ void gq_coords(const GridDev& G, const float* p, int* c) {
  for (int d = 0; d < 3; ++d) c[d] = 0;
  for (int d = 0; d < G.dims; ++d) c[d] = gq_clamp((int)((p[d] - G.g.mn[d]) / G.g.bin_size), G.g.ext[d] - 1);
}

// bin of task t of the (2r+1)^d block around c, or -1 when it lies outside
__device__ __forceinline__ long long gq_task_bin(const GridDev& G, const int* c, int t, int side, int r) {
  int o[3] = {t % side - r, 0, 0};
  if (G.dims == 2) o[1] = t / side - r;
  if (G.dims == 3) {
    const int tmp = t / side;
    o[1] = tmp % side - r;
    o[2] = tmp / side - r;
  }
  int nb[3] = {0, 0, 0};
  for (int d = 0; d < G.dims; ++d) {
    nb[d] = c[d] + o[d];
    if (nb[d] < 0 || nb[d] >= G.g.ext[d]) return -1;
  }
  return (long long)nb[0] + (long long)nb[1] * G.g.ext[0] + (long long)nb[2] * ((long long)G.g.ext[0] * G.g.ext[1]);
}

__device__ __forceinline__ float gq_dist2(const GridDev& G, const float* p, const float4& v) {
  float s = 0.0f;
  const float e0 = p[0] - v.x;
  s = s + e0 * e0;
  if (G.dims >= 2) { const float e1 = p[1] - v.y; s = s + e1 * e1; }
  if (G.dims >= 3) { const float e2 = p[2] - v.z; s = s + e2 * e2; }
  return s;
}

__device__ __forceinline__ int gq_tasks(const GridDev& G, int side) {
  return G.dims == 2 ? side * side : side * side * side;
}

// Grid::get_nearest_point_index (grid.hpp:413-441): -1 when the block is empty
__device__ __forceinline__ int grid_nearest(const GridDev& G, const float* p, int r) {
  int c[3];
  gq_coords(G, p, c);
  const int side = 2 * r + 1;
  int best = -1;
  float bd = FLT_MAX;
  for (int t = 0; t < gq_tasks(G, side); ++t) {
    const long long b = gq_task_bin(G, c, t, side, r);
    if (b < 0) continue;
    const unsigned e = G.off[b + 1];
    for (unsigned k = G.off[b]; k < e; ++k) {
      const float s = gq_dist2(G, p, G.B[k]);
      if (s < bd) { best = (int)G.Bid[k]; bd = s; }
    }
  }
  return best;
}

// Grid::get_random_point_index_in_neighbourhood_bins (grid.hpp:453-492)
__device__ __forceinline__ int grid_random_in_bins(const GridDev& G, const float* p, int r, unsigned draw) {
  int c[3];
  gq_coords(G, p, c);
  const int side = 2 * r + 1;
  int total = 0;
  for (int t = 0; t < gq_tasks(G, side); ++t) {
    const long long b = gq_task_bin(G, c, t, side, r);
    if (b >= 0) total += (int)(G.off[b + 1] - G.off[b]);
  }
  const int target = total > 0 ? (int)(draw % (unsigned)total) : 0;
  int seen = 0;
  for (int t = 0; t < gq_tasks(G, side); ++t) {
    const long long b = gq_task_bin(G, c, t, side, r);
    if (b < 0) continue;
    const int count = (int)(G.off[b + 1] - G.off[b]);
    if (count == 0) continue;
    if (target < seen + count) return (int)G.Bid[G.off[b] + (unsigned)(target - seen)];
    seen += count;
  }
  return -1;
}

struct GridAcceptAll {
  __device__ bool operator()(int) const { return true; }
};

// Grid::get_random_point_index_in_neighbourhood (grid.hpp:505-637): points
// within the physical radius (<= r^2) that pass the filter
template <class Filter = GridAcceptAll>
__device__ __forceinline__ int grid_random_in_radius(const GridDev& G, const float* p, float radius, unsigned draw,
                                                     const Filter& filter = Filter{}) {
  int rb = (int)ceilf(radius / G.g.bin_size);
  rb = rb < 1 ? 1 : rb;
  int c[3];
  gq_coords(G, p, c);
  const int side = 2 * rb + 1;
  const float r2 = radius * radius;
  int total = 0;
  for (int t = 0; t < gq_tasks(G, side); ++t) {
    const long long b = gq_task_bin(G, c, t, side, rb);
    if (b < 0) continue;
    const unsigned e = G.off[b + 1];
    for (unsigned k = G.off[b]; k < e; ++k)
      if (gq_dist2(G, p, G.B[k]) <= r2 && filter((int)G.Bid[k])) ++total;
  }
  if (total == 0) return -1;
  const int target = (int)(draw % (unsigned)total);
  int seen = 0;
  for (int t = 0; t < gq_tasks(G, side); ++t) {
    const long long b = gq_task_bin(G, c, t, side, rb);
    if (b < 0) continue;
    const unsigned e = G.off[b + 1];
    for (unsigned k = G.off[b]; k < e; ++k) {
      if (gq_dist2(G, p, G.B[k]) <= r2 && filter((int)G.Bid[k])) {
        if (seen == target) return (int)G.Bid[k];
        ++seen;
      }
    }
  }
  return -1;
}

}  // namespace tecs
