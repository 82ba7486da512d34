// common.cuh -- shared device helpers for the TECS cell-step kernels (sm_103a).
//
// Arithmetic that decides which pairs exist (squared distances, midpoints,
// Gabriel radii, bin coordinates) follows the operation order of the
// reference's VectorN code (include/types/vector.hpp) and is compiled with
// -fmad=false, so no multiply-add is contracted and the pair sets agree bit
// for bit with the reference's Serial backend.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>

namespace tecs {

constexpr float kFltEpsilon = 1.19209290e-7f;  // Kokkos::Experimental::epsilon_v<float>

// Uniform bin grid, include/utils/grid.hpp:71-85 and :201-259.
struct GridP {
  float mn[3];
  float bin_size;   // bin_size_scale * cutoff
  float inv_bin;    // 1 / bin_size
  int ext[3];       // ceil((max - min) / bin_size), 1 for unused dimensions
  int R;            // search radius in bins, ceil(cutoff * inv_bin)
  unsigned nbins;   // product of extents
  int pow2;         // bin_size is a power of two: (p - min) / bin_size == (p - min) * inv_bin exactly
};

// Sets g.pow2 from g.bin_size (host side, after bin_size and inv_bin are set).
// Dividing by 2^k and multiplying by 2^-k round the same real number, so the
// two forms of the bin coordinate agree bit for bit.
inline void grid_set_pow2(GridP& g) {
  int e = 0;
  const float m = std::frexp(g.bin_size, &e);
  g.pow2 = (m == 0.5f && g.inv_bin * g.bin_size == 1.0f) ? 1 : 0;
}

// Built-in force descriptor plus the pair predicates' constants.
struct ForceP {
  int force;        // tecs_force
  float k_rep, r_rep, k_adh, r_adh, k_pol;
  float rc2;        // cutoff * cutoff
  float gab_factor; // c*c*0.25f  (binned_gabriel.hpp:42)
  float gab_csq;    // c*c        (naive_gabriel.hpp:26)
};

__device__ __forceinline__ int clampi(int v, int hi) { return v < hi ? (v < 0 ? 0 : v) : hi; }

// grid.hpp:222-230: clamp(int((p - min) / bin_size), 0, ext - 1); with a
// power-of-two bin size the division is the (identical) multiplication
template <int D>
__device__ __forceinline__ void bin_coords_div(const GridP& g, const float* p, int* c) {
  if (g.pow2) {
#pragma unroll
    for (int d = 0; d < D; ++d) c[d] = clampi((int)((p[d] - g.mn[d]) * g.inv_bin), g.ext[d] - 1);
  } else {
#pragma unroll
    for (int d = 0; d < D; ++d) c[d] = clampi((int)((p[d] - g.mn[d]) / g.bin_size), g.ext[d] - 1);
  }
}
// binned_all_pairs.hpp:103-109: the same with the inverse bin size
template <int D>
__device__ __forceinline__ void bin_coords_mul(const GridP& g, const float* p, int* c) {
#pragma unroll
  for (int d = 0; d < D; ++d) c[d] = clampi((int)((p[d] - g.mn[d]) * g.inv_bin), g.ext[d] - 1);
}
template <int D>
__device__ __forceinline__ unsigned flatten(const GridP& g, const int* c) {
  unsigned b = (unsigned)c[0];
  if (D >= 2) b += (unsigned)c[1] * (unsigned)g.ext[0];
  if (D >= 3) b += (unsigned)c[2] * ((unsigned)g.ext[0] * (unsigned)g.ext[1]);
  return b;
}

__device__ __forceinline__ unsigned id_of(const float4& v) { return __float_as_uint(v.w); }

// Counter-based RNG keyed by (seed, step, cell id, stream).  SplitMix64's
// finaliser (Steele, Lea & Flood 2014) applied twice.
__host__ __device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__host__ __device__ __forceinline__ uint64_t hash64(uint64_t seed, uint64_t step, uint64_t cell, uint64_t stream) {
  uint64_t k = step * 0x9E3779B97F4A7C15ull + cell * 0xD1B54A32D192ED03ull + stream * 0x94D049BB133111EBull + 1ull;
  return mix64(seed ^ mix64(k));
}
__host__ __device__ __forceinline__ double u01(uint64_t h) { return (double)(h >> 11) * (1.0 / 9007199254740992.0); }

}  // namespace tecs
