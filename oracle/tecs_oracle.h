/*
 * tecs_oracle.h -- CPU restatement of the TECS per-timestep hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This oracle is the CPU result that the CUDA
 * path is compared against; it is never linked into, loaded by, or called
 * from the product library.  Only the test suite, the smoke check and the benchmark's
 * CPU-baseline leg use it.
 *
 * Parity pin: the restatement is checked against golden vectors produced by
 * the reference's own headers (compiled unmodified against a Kokkos-API
 * shim, recipe in oracle/Makefile) and committed under tests/golden/.
 *
 * Arithmetic is FP32 with contraction disabled (-ffp-contract=off), in the
 * operation order of the reference's VectorN / Polarity_ code, so the
 * restatement reproduces the reference's Serial-backend results bit for bit
 * where no libm transcendental is involved.
 */
#ifndef TECS_ORACLE_H
#define TECS_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Pair finders (include/pair_finders/*.hpp). */
enum {
  TECS_O_NAIVE_ALL_PAIRS = 0,   /* naive_all_pairs.hpp:41-103          */
  TECS_O_BINNED_ALL_PAIRS = 1,  /* binned_all_pairs.hpp:66-183         */
  TECS_O_NAIVE_GABRIEL = 2,     /* naive_gabriel.hpp:36-120            */
  TECS_O_BINNED_GABRIEL = 3,    /* binned_gabriel.hpp:71-362           */
  TECS_O_NAIVE_DELAUNAY = 4     /* naive_delaunay.hpp:31-294           */
};

/* Built-in pairwise force laws. */
enum {
  TECS_O_FORCE_NONE = 0,        /* pair capture only, no deltas          */
  TECS_O_FORCE_SPRING2R = 1,    /* k_rep*max(r_rep-d,0) - k_adh*max(d-r_adh,0), forces/predefined.hpp:107-144 form */
  TECS_O_FORCE_POLARITY = 2     /* spring2r + k_pol*(bending + bidirectional alignment), types/polarity.hpp:131-198 */
};

typedef struct {
  int dims;                   /* 2 or 3                                         */
  int finder;                 /* TECS_O_*                                       */
  int symmetric;              /* 1: j<i half-shell with +d/-d (…_symmetric.hpp) */
  float cutoff;
  float gabriel_coefficient;
  float min_bounds[3];
  float max_bounds[3];
  float bin_size_scale;
  int rebuild_every_n;
  int integrator;             /* 0 Euler (euler.hpp), 1 Heun (heun.hpp)          */
  int com_fix;                /* 0 NoComFixer, 1 GlobalComFixer                  */
  int force;                  /* TECS_O_FORCE_*                                  */
  float k_rep, r_rep, k_adh, r_adh, k_pol;
  int has_polarity;
  unsigned capacity;
  /* cell division after each step (pattern of examples/growth_w_wall.cpp:119-136) */
  double division_probability;
  float division_offset;
  uint64_t seed;
} tecs_oracle_desc;

typedef struct tecs_oracle tecs_oracle;

tecs_oracle* tecs_oracle_create(const tecs_oracle_desc* desc);
void tecs_oracle_destroy(tecs_oracle* o);

/* positions: n*dims floats (AoS, like View<VectorN<float,dims>>); polarity: n*2 floats or NULL */
int tecs_oracle_set_state(tecs_oracle* o, const float* positions, const float* polarity, unsigned n);
unsigned tecs_oracle_count(const tecs_oracle* o);
int tecs_oracle_get_state(const tecs_oracle* o, float* positions, float* polarity);

/* Links (include/types/link.hpp) with the constant-pull link law of
 * examples/intercalation.cpp:65-71: every force evaluation adds, after the
 * pairwise forces and in link order, k*(x_b - x_a)/|x_b - x_a| to cell a and
 * its negative to cell b; links with a == b are skipped
 * (integrators/base.hpp:197-234).  links: n_links (a, b) pairs; 0 clears. */
int tecs_oracle_set_links(tecs_oracle* o, const uint32_t* links, unsigned n_links, float strength);

/* n_steps integrator steps (plus division when enabled) */
int tecs_oracle_step(tecs_oracle* o, double dt, int n_steps, int threads);

/* One full-step force evaluation (grid rebuilt) on the current state:
 * writes the per-cell deltas (position: n*dims, polarity: n*2 or NULL) and,
 * if pairs != NULL, the directed (self, other) pairs in evaluation order.
 * Returns the number of pairs (may exceed pair_capacity; only the first
 * pair_capacity are written), or -1 on error. */
long tecs_oracle_evaluate(tecs_oracle* o, float* delta_positions, float* delta_polarity,
                          uint32_t* pairs, long pair_capacity, int threads);

/* Counter-based RNG shared with the CUDA path (division decisions). */
uint64_t tecs_oracle_hash(uint64_t seed, uint64_t step, uint64_t cell, uint64_t stream);

/* The reference's standalone acceleration::Grid (utils/grid.hpp:29-638) over
 * n points (float[n][dims]), bins of bin_size over [min, max), queried at m
 * points: nearest point in 3^d (near1) and 5^d (near2) bins, a random point of
 * the 3^d bins (rbins), a random point within `radius` (rrad) and the same
 * among indices not divisible by 3 (rfilt), the random targets being
 * draws[q] mod (number of eligible points).  Any output may be NULL. */
int tecs_oracle_grid_query(int dims, const float* points, unsigned n, const float* min_bounds,
                           const float* max_bounds, float bin_size, const float* queries, unsigned m,
                           const uint32_t* draws, float radius, int32_t* near1, int32_t* near2, int32_t* rbins,
                           int32_t* rrad, int32_t* rfilt);

const char* tecs_oracle_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
