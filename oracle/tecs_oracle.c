/*
 * tecs_oracle.c -- CPU restatement of the TECS per-timestep hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the CPU result the CUDA path is compared
 * against, used by tests/, the smoke check and the benchmark's CPU-baseline
 * leg.  Never part of the
 * product library.
 *
 * Every function cites the reference file:line it restates (paths relative
 * to the reference project root).  Build with -ffp-contract=off so that no
 * multiply-add is fused: the reference's Serial build then agrees bit for bit
 * on everything that does not call a libm transcendental.
 */
#include "tecs_oracle.h"

#include <float.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static __thread char g_err[256];
static void set_err(const char* m) { snprintf(g_err, sizeof g_err, "%s", m); }
const char* tecs_oracle_last_error(void) { return g_err; }

struct tecs_oracle {
  tecs_oracle_desc d;
  unsigned n;
  /* stage buffers, capacity-sized (integrators/detail.hpp:277-309) */
  float *x, *p;        /* stage 0 */
  float *d1x, *d1p;    /* stage 1 */
  float *x2, *p2;      /* stage 2 (Heun predictor) */
  float *d3x, *d3p;    /* stage 3 (Heun corrector deltas) */
  float *vold;         /* old_velocities (integrators/base.hpp:59) */
  /* grid (utils/grid.hpp:71-85) */
  float bin_size, inv_bin;
  int search_radius;
  int ext[3];
  long nbins;
  unsigned *perm, *offsets, *bins_scratch;
  unsigned perm_cap;
  int step_count;      /* pair finder rebuild counter (binned_gabriel.hpp:58-59) */
  uint64_t step_index; /* integrator steps taken, keys the division RNG */
  uint32_t* links;     /* (a, b) pairs */
  unsigned n_links;
  float link_strength;
};

/* ------------------------------------------------------------------------ */
/* counter-based RNG (ours; the reference's Random_XorShift64_Pool is not    */
/* reproducible across backends, simulation.hpp:89)                          */
static uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
uint64_t tecs_oracle_hash(uint64_t seed, uint64_t step, uint64_t cell, uint64_t stream) {
  uint64_t k = step * 0x9E3779B97F4A7C15ull + cell * 0xD1B54A32D192ED03ull +
               stream * 0x94D049BB133111EBull + 1ull;
  return mix64(seed ^ mix64(k));
}
static double u01(uint64_t h) { return (double)(h >> 11) * (1.0 / 9007199254740992.0); }

/* ------------------------------------------------------------------------ */
tecs_oracle* tecs_oracle_create(const tecs_oracle_desc* desc) {
  if (!desc || (desc->dims != 2 && desc->dims != 3)) { set_err("dims must be 2 or 3"); return NULL; }
  if (desc->capacity == 0) { set_err("capacity must be > 0"); return NULL; }
  if (desc->finder < 0 || desc->finder > TECS_O_NAIVE_DELAUNAY) { set_err("unknown finder"); return NULL; }
  if (desc->finder == TECS_O_NAIVE_DELAUNAY && desc->symmetric) {
    set_err("the Delaunay finder has no symmetric variant"); return NULL;
  }
  tecs_oracle* o = (tecs_oracle*)calloc(1, sizeof *o);
  o->d = *desc;
  const size_t cap = desc->capacity, D = (size_t)desc->dims;
  o->x = calloc(cap * D, 4);   o->p = calloc(cap * 2, 4);
  o->d1x = calloc(cap * D, 4); o->d1p = calloc(cap * 2, 4);
  o->x2 = calloc(cap * D, 4);  o->p2 = calloc(cap * 2, 4);
  o->d3x = calloc(cap * D, 4); o->d3p = calloc(cap * 2, 4);
  o->vold = calloc(cap * D, 4);
  /* binned_gabriel.hpp:28-42 / binned_all_pairs.hpp:27-39 */
  o->bin_size = desc->bin_size_scale * desc->cutoff;
  o->inv_bin = 1.0f / o->bin_size;
  o->search_radius = (int)ceilf(desc->cutoff * o->inv_bin);
  /* grid.hpp:201-215 calc_bin_extents / calc_bin_count */
  o->nbins = 1;
  for (int d = 0; d < 3; ++d) o->ext[d] = 1;
  for (int d = 0; d < desc->dims; ++d) {
    o->ext[d] = (int)ceilf((desc->max_bounds[d] - desc->min_bounds[d]) / o->bin_size);
    o->nbins *= o->ext[d];
  }
  return o;
}

void tecs_oracle_destroy(tecs_oracle* o) {
  if (!o) return;
  free(o->x); free(o->p); free(o->d1x); free(o->d1p); free(o->x2); free(o->p2);
  free(o->d3x); free(o->d3p); free(o->vold); free(o->links);
  free(o->perm); free(o->offsets); free(o->bins_scratch);
  free(o);
}

int tecs_oracle_set_state(tecs_oracle* o, const float* pos, const float* pol, unsigned n) {
  if (n > o->d.capacity) { set_err("n exceeds capacity"); return -1; }
  const size_t cap = o->d.capacity, D = (size_t)o->d.dims;
  memset(o->x, 0, cap * D * 4); memset(o->p, 0, cap * 8);
  memcpy(o->x, pos, (size_t)n * D * 4);
  if (pol) memcpy(o->p, pol, (size_t)n * 8);
  memset(o->d1x, 0, cap * D * 4); memset(o->d1p, 0, cap * 8);
  memset(o->d3x, 0, cap * D * 4); memset(o->d3p, 0, cap * 8);
  memset(o->vold, 0, cap * D * 4);
  o->n = n;
  o->step_count = 0;  /* Simulation::set_agent_count -> finder.set_agent_count (binned_gabriel.hpp:61-64) */
  /* step_index (the division stream) counts the steps since creation: a new state does not restart it */
  return 0;
}

unsigned tecs_oracle_count(const tecs_oracle* o) { return o->n; }

int tecs_oracle_get_state(const tecs_oracle* o, float* pos, float* pol) {
  memcpy(pos, o->x, (size_t)o->n * o->d.dims * 4);
  if (pol) memcpy(pol, o->p, (size_t)o->n * 8);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* grid                                                                     */

/* grid.hpp:222-230: clamp(int((p - min) / bin_size), 0, ext - 1), truncation */
static void bin_coords_div(const tecs_oracle* o, const float* pt, int* c) {
  for (int d = 0; d < o->d.dims; ++d) {
    int v = (int)((pt[d] - o->d.min_bounds[d]) / o->bin_size);
    int hi = o->ext[d] - 1;
    c[d] = v < hi ? v : hi;
    if (c[d] < 0) c[d] = 0;
  }
}
/* binned_all_pairs.hpp:103-109: same, but multiplied by the inverse bin size */
static void bin_coords_mul(const tecs_oracle* o, const float* pt, int* c) {
  for (int d = 0; d < o->d.dims; ++d) {
    int v = (int)((pt[d] - o->d.min_bounds[d]) * o->inv_bin);
    int hi = o->ext[d] - 1;
    c[d] = v < hi ? v : hi;
    if (c[d] < 0) c[d] = 0;
  }
}
/* grid.hpp:235-259 flatten_bin_index (x fastest) */
static long flatten(const tecs_oracle* o, const int* c) {
  long b = c[0];
  if (o->d.dims >= 2) b += (long)c[1] * o->ext[0];
  if (o->d.dims >= 3) b += (long)c[2] * ((long)o->ext[0] * o->ext[1]);
  return b;
}

/* grid.hpp:389-401 rebuild + Kokkos BinSort (count, exclusive scan, binning
 * in ascending cell order, as the Serial backend executes it). */
static void grid_rebuild(tecs_oracle* o, const float* xin) {
  const unsigned n = o->n;
  const int D = o->d.dims;
  if (!o->offsets) o->offsets = (unsigned*)malloc(((size_t)o->nbins + 1) * 4);
  if (o->perm_cap < o->d.capacity) {
    free(o->perm); free(o->bins_scratch);
    o->perm = (unsigned*)malloc((size_t)o->d.capacity * 4);
    o->bins_scratch = (unsigned*)malloc((size_t)o->d.capacity * 4);
    o->perm_cap = o->d.capacity;
  }
  unsigned* cnt = (unsigned*)calloc((size_t)o->nbins + 1, 4);
  for (unsigned i = 0; i < n; ++i) {
    int c[3];
    bin_coords_div(o, xin + (size_t)i * D, c);
    long b = flatten(o, c);
    o->bins_scratch[i] = (unsigned)b;
    cnt[b]++;
  }
  unsigned acc = 0;
  for (long b = 0; b <= o->nbins; ++b) { o->offsets[b] = acc; acc += cnt[b]; cnt[b] = 0; }
  for (unsigned i = 0; i < n; ++i) {
    unsigned b = o->bins_scratch[i];
    o->perm[o->offsets[b] + cnt[b]++] = i;
  }
  free(cnt);
}

/* ------------------------------------------------------------------------ */
/* force laws                                                               */

typedef struct { float dx[3]; float dp[2]; } acc_t;

static void polarity_to_vector3(const float* pol, float* v) {
  /* types/polarity.hpp:111-118 */
  v[0] = sinf(pol[0]) * cosf(pol[1]);
  v[1] = sinf(pol[0]) * sinf(pol[1]);
  v[2] = cosf(pol[0]);
}
static float dot3(const float* a, const float* b) {
  /* types/vector.hpp dot: result{} then += a_i*b_i in index order */
  float r = 0.0f;
  r = r + a[0] * b[0];
  r = r + a[1] * b[1];
  r = r + a[2] * b[2];
  return r;
}
/* types/polarity.hpp:146-157 unidirectional_polarization_force */
static void unidirectional(const float* self, const float* other, float* res) {
  res[0] = cosf(self[0]) * sinf(other[0]) * cosf(self[1] - other[1]) - sinf(self[0]) * cosf(other[0]);
  res[1] = 0.0f;
  float sin_theta = sinf(self[0]);
  if (fabsf(sin_theta) > FLT_EPSILON) res[1] = -sinf(other[0]) * sinf(self[1] - other[1]) / sin_theta;
}
/* types/polarity.hpp:132-136 dot */
static float pol_dot(const float* a, const float* b) {
  return sinf(a[0]) * sinf(b[0]) * cosf(a[1] - b[1]) + cosf(a[0]) * cosf(b[0]);
}

/* The pairwise force for one (self=i, other=j) pair.  disp = x_i - x_j. */
static void pair_force(const tecs_oracle* o, const float* disp, float dist,
                       const float* pol_i, const float* pol_j, acc_t* a) {
  const int D = o->d.dims;
  if (o->d.force == TECS_O_FORCE_NONE) return;
  /* spring2r in the form of forces/predefined.hpp:107-144 (PiecewiseLinear
   * with separate repulsion / adhesion radii): zero vector when dist == 0 */
  if (dist != 0.0f) {
    float F = o->d.k_rep * fmaxf(o->d.r_rep - dist, 0.0f) - o->d.k_adh * fmaxf(dist - o->d.r_adh, 0.0f);
    for (int d = 0; d < D; ++d) a->dx[d] = a->dx[d] + (disp[d] * F) / dist;
  }
  if (o->d.force == TECS_O_FORCE_POLARITY) {
    /* types/polarity.hpp:181-198 bending_force (3-D only) */
    const float k = o->d.k_pol;
    float tv[3], ov[3];
    polarity_to_vector3(pol_i, tv);
    float prod_i = dot3(tv, disp) / dist;
    polarity_to_vector3(pol_j, ov);
    float prod_j = dot3(ov, disp) / dist;
    /* Kokkos::pow(float, int) promotes to double; the quotient is rounded to float on use */
    float si = -prod_i / dist;
    float qi = (float)(pow((double)prod_i, 2.0) / pow((double)dist, 2.0));
    float sj = -prod_j / dist;
    float qj = (float)(pow((double)prod_j, 2.0) / pow((double)dist, 2.0));
    float vec[3];
    for (int d = 0; d < 3; ++d) {
      float t = si * tv[d];
      t = t + qi * disp[d];
      t = t + sj * ov[d];
      t = t + qj * disp[d];
      vec[d] = t;
    }
    /* from_vector3(disp, dist): polarity.hpp:62-66 */
    float q = disp[2] / dist;
    float dpol[2] = {acosf(fminf(1.0f, fmaxf(-1.0f, q))), atan2f(disp[1], disp[0])};
    float uni[2];
    unidirectional(pol_i, dpol, uni);
    float bp[2] = {-prod_i * uni[0], -prod_i * uni[1]};
    for (int d = 0; d < 3; ++d) a->dx[d] = a->dx[d] + vec[d] * k;
    a->dp[0] = a->dp[0] + bp[0] * k;
    a->dp[1] = a->dp[1] + bp[1] * k;
    /* bidirectional_polarization_force: polarity.hpp:165-168 */
    float dt_ = pol_dot(pol_i, pol_j);
    float u2[2];
    unidirectional(pol_i, pol_j, u2);
    float al[2] = {dt_ * u2[0], dt_ * u2[1]};
    a->dp[0] = a->dp[0] + al[0] * k;
    a->dp[1] = a->dp[1] + al[1] * k;
  }
}

/* ------------------------------------------------------------------------ */
/* pair finders: one evaluation pass                                        */

typedef struct {
  uint32_t* pairs; long cap; long count;
} pair_sink;

/* Gabriel witness test over the bins overlapping the ball around the
 * midpoint, binned_gabriel.hpp:133-209.  Returns 1 when blocked. */
static int gabriel_blocked_binned(const tecs_oracle* o, const float* xin, unsigned i, unsigned j,
                                  const float* xi, const float* disp, float d2) {
  const int D = o->d.dims;
  float m[3], rsq, r;
  for (int d = 0; d < D; ++d) m[d] = xi[d] - disp[d] * 0.5f;
  const float factor = o->d.gabriel_coefficient * o->d.gabriel_coefficient * 0.25f;  /* :42 */
  rsq = d2 * factor;
  r = sqrtf(rsq);
  int mn[3] = {0, 0, 0}, span[3] = {1, 1, 1};
  int tasks = 1;
  for (int d = 0; d < D; ++d) {
    int hi = o->ext[d] - 1;
    int a = (int)floorf((m[d] - r - o->d.min_bounds[d]) * o->inv_bin);
    a = a < hi ? a : hi; if (a < 0) a = 0;
    int b = (int)floorf((m[d] + r - o->d.min_bounds[d]) * o->inv_bin);
    b = b < hi ? b : hi; if (b < 0) b = 0;
    mn[d] = a; span[d] = b - a + 1; tasks *= span[d];
  }
  for (int t = 0; t < tasks; ++t) {
    int c[3] = {0, 0, 0};
    if (D == 2) { c[0] = mn[0] + t % span[0]; c[1] = mn[1] + t / span[0]; }
    else { int tmp = t / span[0]; c[0] = mn[0] + t % span[0]; c[1] = mn[1] + tmp % span[1]; c[2] = mn[2] + tmp / span[1]; }
    long b = flatten(o, c);
    for (unsigned idx = o->offsets[b]; idx < o->offsets[b + 1]; ++idx) {
      unsigned k = o->perm[idx];
      if (k == i || k == j) continue;
      const float* xk = xin + (size_t)k * D;
      float s = 0.0f;  /* vector.hpp distance_to_squared */
      for (int d = 0; d < D; ++d) { float e = xk[d] - m[d]; s = s + e * e; }
      if (s < rsq) return 1;
    }
  }
  return 0;
}

/* naive_gabriel.hpp:71-80: every k, radius (d2 * 0.25) * c^2 */
static int gabriel_blocked_naive(const tecs_oracle* o, const float* xin, unsigned i, unsigned j,
                                 const float* xi, const float* disp, float d2) {
  const int D = o->d.dims;
  float m[3];
  for (int d = 0; d < D; ++d) m[d] = xi[d] - disp[d] * 0.5f;
  const float csq = o->d.gabriel_coefficient * o->d.gabriel_coefficient;
  const float rsq = d2 * 0.25f * csq;
  for (unsigned k = 0; k < o->n; ++k) {
    if (k == i || k == j) continue;
    const float* xk = xin + (size_t)k * D;
    float s = 0.0f;
    for (int d = 0; d < D; ++d) { float e = xk[d] - m[d]; s = s + e * e; }
    if (s < rsq) return 1;
  }
  return 0;
}

static float dist2(const float* a, const float* b, int D) {  /* vector.hpp distance_to_squared */
  float s = 0.0f;
  for (int d = 0; d < D; ++d) { float e = a[d] - b[d]; s = s + e * e; }
  return s;
}

/* naive_delaunay.hpp: how many times the pair (i, j) is applied.
 * 2-D (:45-99): once per third point k whose circumcircle through i, j, k is
 * non-degenerate (|den| > eps) and holds no other point (<= r^2 rejects).
 * 3-D (:158-292): once per third point k for which some l > k gives a
 * non-degenerate tetrahedron whose circumsphere holds no other point (the
 * axis-aligned prefilter |p_m - c| > r skips a point before its distance test). */
static int delaunay_count(const tecs_oracle* o, const float* xin, unsigned i, unsigned j) {
  const int D = o->d.dims;
  const unsigned n = o->n;
  const float eps = FLT_EPSILON;
  const float* pi = xin + (size_t)i * D;
  const float* pj = xin + (size_t)j * D;
  int count = 0;
  if (D == 2) {
    const float li = dist2(pi, (const float[3]){0, 0, 0}, 2), lj = dist2(pj, (const float[3]){0, 0, 0}, 2);
    for (unsigned k = 0; k < n; ++k) {
      if (k == i || k == j) continue;
      const float* pk = xin + (size_t)k * 2;
      const float den = 2.0f * (pi[0] * (pj[1] - pk[1]) + pj[0] * (pk[1] - pi[1]) + pk[0] * (pi[1] - pj[1]));
      if (fabsf(den) <= eps) continue;
      const float lk = dist2(pk, (const float[3]){0, 0, 0}, 2);
      float c[2];
      c[0] = (li * (pj[1] - pk[1]) + lj * (pk[1] - pi[1]) + lk * (pi[1] - pj[1])) / den;
      c[1] = (li * (pk[0] - pj[0]) + lj * (pi[0] - pk[0]) + lk * (pj[0] - pi[0])) / den;
      const float r2 = dist2(pi, c, 2);
      int ok = 1;
      for (unsigned m = 0; m < n && ok; ++m) {
        if (m == i || m == j || m == k) continue;
        if (dist2(xin + (size_t)m * 2, c, 2) <= r2) ok = 0;
      }
      count += ok;
    }
    return count;
  }
  const float zero[3] = {0, 0, 0};
  const float li = dist2(pi, zero, 3), lj = dist2(pj, zero, 3);
  for (unsigned k = 0; k < n; ++k) {
    if (k == i || k == j) continue;
    const float* pk = xin + (size_t)k * 3;
    const float lk = dist2(pk, zero, 3);
    for (unsigned l = k + 1; l < n; ++l) {
      if (l == i || l == j) continue;
      const float* pl = xin + (size_t)l * 3;
      float e1[3], e2[3], e3[3];
      for (int d = 0; d < 3; ++d) { e1[d] = pj[d] - pi[d]; e2[d] = pk[d] - pi[d]; e3[d] = pl[d] - pi[d]; }
      const float den = 2.0f * (e1[0] * (e2[1] * e3[2] - e2[2] * e3[1]) - e1[1] * (e2[0] * e3[2] - e2[2] * e3[0]) +
                                e1[2] * (e2[0] * e3[1] - e2[1] * e3[0]));
      if (fabsf(den) <= eps) continue;
      const float ll = dist2(pl, zero, 3);
      const float b1 = lj - li, b2 = lk - li, b3 = ll - li;
      float c[3];
      c[0] = pi[0] + (b1 * (e2[1] * e3[2] - e2[2] * e3[1]) - e1[1] * (b2 * e3[2] - e2[2] * b3) +
                      e1[2] * (b2 * e3[1] - e2[1] * b3)) / den;
      c[1] = pi[1] + (e1[0] * (b2 * e3[2] - e2[2] * b3) - b1 * (e2[0] * e3[2] - e2[2] * e3[0]) +
                      e1[2] * (e2[0] * b3 - b2 * e3[0])) / den;
      c[2] = pi[2] + (e1[0] * (e2[1] * b3 - b2 * e3[1]) - e1[1] * (e2[0] * b3 - b2 * e3[0]) +
                      b1 * (e2[0] * e3[1] - e2[1] * e3[0])) / den;
      const float r2 = dist2(pi, c, 3);
      const float r = sqrtf(r2);
      int ok = 1;
      for (unsigned m = 0; m < n; ++m) {
        if (m == i || m == j || m == k || m == l) continue;
        const float* pm = xin + (size_t)m * 3;
        if (fabsf(pm[0] - c[0]) > r || fabsf(pm[1] - c[1]) > r || fabsf(pm[2] - c[2]) > r) continue;
        if (dist2(pm, c, 3) <= r2) { ok = 0; break; }
      }
      if (ok) { ++count; break; }
    }
  }
  return count;
}

/* Candidate j for cell i: cutoff + Gabriel predicate, then the force.
 * Returns how many times the pair is applied: 0 or 1, or the Delaunay count. */
static int visit_pair(const tecs_oracle* o, const float* xin, const float* pin, unsigned i, unsigned j,
                      const float* xi, acc_t* a) {
  const int D = o->d.dims;
  const float* xj = xin + (size_t)j * D;
  float disp[3] = {0, 0, 0};
  float d2 = 0.0f;
  for (int d = 0; d < D; ++d) disp[d] = xi[d] - xj[d];
  for (int d = 0; d < D; ++d) d2 = d2 + disp[d] * disp[d];  /* vector.hpp length_squared */
  const float rc2 = o->d.cutoff * o->d.cutoff;
  if (d2 >= rc2) return 0;
  if (o->d.finder == TECS_O_BINNED_GABRIEL && gabriel_blocked_binned(o, xin, i, j, xi, disp, d2)) return 0;
  if (o->d.finder == TECS_O_NAIVE_GABRIEL && gabriel_blocked_naive(o, xin, i, j, xi, disp, d2)) return 0;
  int reps = 1;
  if (o->d.finder == TECS_O_NAIVE_DELAUNAY && (reps = delaunay_count(o, xin, i, j)) == 0) return 0;
  float dist = sqrtf(d2);
  /* each application adds into the cell's delta in turn (naive_delaunay.hpp:86-99) */
  for (int r = 0; r < reps; ++r)
    pair_force(o, disp, dist, pin ? pin + (size_t)i * 2 : NULL, pin ? pin + (size_t)j * 2 : NULL, a);
  return reps;
}

/* The link forces of one evaluation, after the pairwise ones: Serial order of
 * integrators/base.hpp:205-233, each endpoint's accumulator starting at zero. */
static void apply_links(const tecs_oracle* o, const float* xin, float* ox) {
  const int D = o->d.dims;
  const float k = o->link_strength;
  for (unsigned l = 0; l < o->n_links; ++l) {
    const unsigned a = o->links[2 * l], b = o->links[2 * l + 1];
    if (a == b) continue;
    float disp[3] = {0, 0, 0}, d2 = 0.0f;
    for (int d = 0; d < D; ++d) disp[d] = xin[(size_t)b * D + d] - xin[(size_t)a * D + d];
    for (int d = 0; d < D; ++d) d2 = d2 + disp[d] * disp[d];
    const float dist = sqrtf(d2);
    for (int d = 0; d < D; ++d) ox[(size_t)a * D + d] = ox[(size_t)a * D + d] + (0.0f + (k * disp[d]) / dist);
    for (int d = 0; d < D; ++d) ox[(size_t)b * D + d] = ox[(size_t)b * D + d] + (0.0f + (-k * disp[d]) / dist);
  }
}

int tecs_oracle_set_links(tecs_oracle* o, const uint32_t* links, unsigned n_links, float strength) {
  for (unsigned l = 0; l < 2 * n_links; ++l)
    if (links[l] >= o->d.capacity) { set_err("link endpoint beyond capacity"); return -1; }
  free(o->links);
  o->links = NULL;
  o->n_links = 0;
  if (n_links) {
    o->links = (uint32_t*)malloc((size_t)n_links * 8);
    memcpy(o->links, links, (size_t)n_links * 8);
  }
  o->n_links = n_links;
  o->link_strength = strength;
  return 0;
}

/* One pass of finder.evaluate_force: in = (xin, pin), out = (ox, op).
 * Non-symmetric finders: each cell i owns its accumulator (…/binned_gabriel.hpp:95-361,
 * binned_all_pairs.hpp:97-182, naive_*.hpp).  Symmetric finders: j < i only, +delta
 * to i and -delta to j in evaluation order (binned_gabriel_symmetric.hpp:156-305). */
static void eval_pass(tecs_oracle* o, const float* xin, const float* pin, float* ox, float* op,
                      int is_full_step, pair_sink* sink, int threads) {
  const int D = o->d.dims;
  const unsigned n = o->n;
  const int binned = (o->d.finder == TECS_O_BINNED_ALL_PAIRS || o->d.finder == TECS_O_BINNED_GABRIEL);
  if (binned && is_full_step) {  /* binned_gabriel.hpp:83-89 */
    if (o->step_count == 0 || o->step_count >= o->d.rebuild_every_n) {
      grid_rebuild(o, xin);
      o->step_count = 0;
    }
    o->step_count++;
  }
  const int side = 2 * o->search_radius + 1;
  const int tasks = D == 2 ? side * side : side * side * side;
  const float eps = FLT_EPSILON;

  if (o->d.symmetric) {
    /* sequential: the order of the +/- updates is the Serial order */
    float* tdrag = (float*)calloc(n ? n : 1, 4);
    float* tvel = (float*)calloc((size_t)(n ? n : 1) * D, 4);
    for (unsigned i = 0; i < n; ++i) {
      const float* xi = xin + (size_t)i * D;
      int bc[3] = {0, 0, 0};
      if (binned) bin_coords_div(o, xi, bc);
      long ncand = binned ? tasks : 1;
      for (long t = 0; t < ncand; ++t) {
        unsigned lo, hi;
        if (binned) {
          int c[3] = {0, 0, 0}, tmp = (int)t, out = 0;
          for (int d = 0; d < D; ++d) { c[d] = bc[d] + tmp % side - o->search_radius; tmp /= side; if (c[d] < 0 || c[d] >= o->ext[d]) out = 1; }
          if (out) continue;
          long b = flatten(o, c); lo = o->offsets[b]; hi = o->offsets[b + 1];
        } else { lo = 0; hi = n; }
        for (unsigned idx = lo; idx < hi; ++idx) {
          unsigned j = binned ? o->perm[idx] : idx;
          if (j >= i) continue;
          acc_t a; memset(&a, 0, sizeof a);
          if (!visit_pair(o, xin, pin, i, j, xi, &a)) continue;
          if (sink) { if (sink->count < sink->cap) { sink->pairs[2 * sink->count] = i; sink->pairs[2 * sink->count + 1] = j; } sink->count++; }
          for (int d = 0; d < D; ++d) ox[(size_t)i * D + d] += a.dx[d];
          if (op) { op[(size_t)i * 2] += a.dp[0]; op[(size_t)i * 2 + 1] += a.dp[1]; }
          for (int d = 0; d < D; ++d) ox[(size_t)j * D + d] += -a.dx[d];
          if (op) { op[(size_t)j * 2] += -a.dp[0]; op[(size_t)j * 2 + 1] += -a.dp[1]; }
          /* drag: built-in laws leave pairwise_drag = 0 */
          for (int d = 0; d < D; ++d) {
            tvel[(size_t)i * D + d] += 0.0f * o->vold[(size_t)j * D + d];
            tvel[(size_t)j * D + d] += 0.0f * o->vold[(size_t)i * D + d];
          }
        }
      }
    }
    for (unsigned i = 0; i < n; ++i)
      for (int d = 0; d < D; ++d) ox[(size_t)i * D + d] += tvel[(size_t)i * D + d] / fmaxf(tdrag[i], eps);
    free(tdrag); free(tvel);
    apply_links(o, xin, ox);
    return;
  }

  /* directed pairs are captured in evaluation order; with threads > 1 each
   * cell records into a private buffer that is concatenated afterwards */
  int nth = 1;
#ifdef _OPENMP
  nth = threads > 0 ? threads : omp_get_max_threads();
  if (sink) nth = 1;
#else
  (void)threads;
#endif
  #pragma omp parallel for schedule(dynamic, 256) num_threads(nth) if (nth > 1)
  for (long ii = 0; ii < (long)n; ++ii) {
    const unsigned i = (unsigned)ii;
    const float* xi = xin + (size_t)i * D;
    acc_t a; memset(&a, 0, sizeof a);
    float tvel[3] = {0, 0, 0};
    const float tdrag = 0.0f;
    if (binned) {
      int bc[3] = {0, 0, 0};
      if (o->d.finder == TECS_O_BINNED_ALL_PAIRS) bin_coords_mul(o, xi, bc);
      else bin_coords_div(o, xi, bc);
      for (int t = 0; t < tasks; ++t) {
        int c[3] = {0, 0, 0}, tmp = t, out = 0;
        for (int d = 0; d < D; ++d) { c[d] = bc[d] + tmp % side - o->search_radius; tmp /= side; if (c[d] < 0 || c[d] >= o->ext[d]) out = 1; }
        if (out) continue;
        long b = flatten(o, c);
        for (unsigned idx = o->offsets[b]; idx < o->offsets[b + 1]; ++idx) {
          unsigned j = o->perm[idx];
          if (j == i) continue;
          if (!visit_pair(o, xin, pin, i, j, xi, &a)) continue;
          if (sink) { if (sink->count < sink->cap) { sink->pairs[2 * sink->count] = i; sink->pairs[2 * sink->count + 1] = j; } sink->count++; }
          for (int d = 0; d < D; ++d) tvel[d] = tvel[d] + 0.0f * o->vold[(size_t)j * D + d];
        }
      }
    } else {
      for (unsigned j = 0; j < n; ++j) {
        if (j == i) continue;
        const int reps = visit_pair(o, xin, pin, i, j, xi, &a);
        for (int r = 0; r < reps; ++r) {
          if (sink) { if (sink->count < sink->cap) { sink->pairs[2 * sink->count] = i; sink->pairs[2 * sink->count + 1] = j; } sink->count++; }
          for (int d = 0; d < D; ++d) tvel[d] = tvel[d] + 0.0f * o->vold[(size_t)j * D + d];
        }
      }
    }
    /* commit: views(i) += total; first(i) += total_velocity / fmax(total_drag, eps) */
    for (int d = 0; d < D; ++d) ox[(size_t)i * D + d] = ox[(size_t)i * D + d] + a.dx[d];
    if (op) { op[(size_t)i * 2] = op[(size_t)i * 2] + a.dp[0]; op[(size_t)i * 2 + 1] = op[(size_t)i * 2 + 1] + a.dp[1]; }
    for (int d = 0; d < D; ++d) ox[(size_t)i * D + d] = ox[(size_t)i * D + d] + tvel[d] / fmaxf(tdrag, eps);
  }
  apply_links(o, xin, ox);
}

/* com_fixers.hpp:24-45: sum over extent(0) == capacity, divided by it */
static void com_mean(const tecs_oracle* o, const float* dx, float* c) {
  const int D = o->d.dims;
  for (int d = 0; d < 3; ++d) c[d] = 0.0f;
  if (!o->d.com_fix) return;
  const size_t cap = o->d.capacity;
  float s[3] = {0, 0, 0};
  for (size_t i = 0; i < cap; ++i)
    for (int d = 0; d < D; ++d) s[d] = s[d] + dx[i * D + d];
  for (int d = 0; d < D; ++d) c[d] = s[d] / (float)cap;
}

/* cell division after a step, deterministic: ascending parent id, daughter
 * appended at the next free slot (growth_w_wall.cpp:119-131 pattern) */
static void divide(tecs_oracle* o) {
  if (o->d.division_probability <= 0.0) return;
  const int D = o->d.dims;
  const unsigned n = o->n;
  unsigned next = n;
  for (unsigned i = 0; i < n; ++i) {
    double u = u01(tecs_oracle_hash(o->d.seed, o->step_index, i, 0));
    if (u > o->d.division_probability) continue;
    if (next >= o->d.capacity) break;
    double th = acos(2.0 * u01(tecs_oracle_hash(o->d.seed, o->step_index, i, 1)) - 1.0);
    double ph = u01(tecs_oracle_hash(o->d.seed, o->step_index, i, 2)) * 2.0 * 3.14159265358979323846;
    float pol[2] = {(float)th, (float)ph};
    float v[3];
    polarity_to_vector3(pol, v);
    for (int d = 0; d < D; ++d) o->x[(size_t)next * D + d] = o->x[(size_t)i * D + d] + o->d.division_offset * v[d];
    o->p[(size_t)next * 2] = o->p[(size_t)i * 2];
    o->p[(size_t)next * 2 + 1] = o->p[(size_t)i * 2 + 1];
    next++;
  }
  if (next != n) { o->n = next; o->step_count = 0; }
}

int tecs_oracle_step(tecs_oracle* o, double dt, int n_steps, int threads) {
  const int D = o->d.dims;
  const float fdt = (float)dt;  /* VectorN * Scalar narrows dt (vector.hpp:264-267) */
  const int pol = o->d.has_polarity;
  for (int s = 0; s < n_steps; ++s) {
    const unsigned n = o->n;
    float c[3];
    if (o->d.integrator == 0) {
      /* euler.hpp:49-85 */
      eval_pass(o, o->x, pol ? o->p : NULL, o->d1x, pol ? o->d1p : NULL, 1, NULL, threads);
      com_mean(o, o->d1x, c);
      for (unsigned i = 0; i < n; ++i) {
        for (int d = 0; d < D; ++d) {
          size_t k = (size_t)i * D + d;
          o->d1x[k] = o->d1x[k] - c[d];
          o->vold[k] = o->d1x[k];
          o->x[k] = o->x[k] + o->d1x[k] * fdt;
          o->d1x[k] = 0.0f;
        }
        if (pol) for (int d = 0; d < 2; ++d) {
          size_t k = (size_t)i * 2 + d;
          o->p[k] = o->p[k] + o->d1p[k] * fdt;
          o->d1p[k] = 0.0f;
        }
      }
    } else {
      /* heun.hpp:112-119 */
      eval_pass(o, o->x, pol ? o->p : NULL, o->d1x, pol ? o->d1p : NULL, 1, NULL, threads);
      com_mean(o, o->d1x, c);                       /* apply_euler_predictor, :54-68 */
      for (unsigned i = 0; i < n; ++i) {
        for (int d = 0; d < D; ++d) {
          size_t k = (size_t)i * D + d;
          o->d1x[k] = o->d1x[k] - c[d];
          o->x2[k] = o->x[k] + o->d1x[k] * fdt;
        }
        if (pol) for (int d = 0; d < 2; ++d) {
          size_t k = (size_t)i * 2 + d;
          o->p2[k] = o->p[k] + o->d1p[k] * fdt;
        }
      }
      eval_pass(o, o->x2, pol ? o->p2 : NULL, o->d3x, pol ? o->d3p : NULL, 0, NULL, threads);
      com_mean(o, o->d3x, c);                       /* apply_heun_corrector, :78-98 */
      for (unsigned i = 0; i < n; ++i) {
        for (int d = 0; d < D; ++d) {
          size_t k = (size_t)i * D + d;
          o->d3x[k] = o->d3x[k] - c[d];
          float sum = o->d1x[k] + o->d3x[k];
          o->vold[k] = sum * 0.5f;
          o->x[k] = o->x[k] + (sum * 0.5f) * fdt;
          o->d1x[k] = 0.0f; o->d3x[k] = 0.0f;
        }
        if (pol) for (int d = 0; d < 2; ++d) {
          size_t k = (size_t)i * 2 + d;
          float sum = o->d1p[k] + o->d3p[k];
          o->p[k] = o->p[k] + (sum * 0.5f) * fdt;
          o->d1p[k] = 0.0f; o->d3p[k] = 0.0f;
        }
      }
    }
    divide(o);
    o->step_index++;
  }
  return 0;
}

long tecs_oracle_evaluate(tecs_oracle* o, float* dpos, float* dpol, uint32_t* pairs, long pair_capacity,
                          int threads) {
  const int D = o->d.dims;
  const size_t n = o->n;
  float* ox = (float*)calloc(n ? n * D : 1, 4);
  float* op = (float*)calloc(n ? n * 2 : 1, 4);
  pair_sink sink = {pairs, pair_capacity, 0};
  const int saved = o->step_count;
  o->step_count = 0;  /* force a rebuild, as on the first full step */
  eval_pass(o, o->x, o->d.has_polarity ? o->p : NULL, ox, o->d.has_polarity ? op : NULL, 1,
            pairs ? &sink : NULL, threads);
  o->step_count = saved;
  if (dpos) memcpy(dpos, ox, n * D * 4);
  if (dpol) memcpy(dpol, op, n * 8);
  free(ox); free(op);
  return pairs ? sink.count : 0;
}

/* ------------------------------------------------------------------------ */
/* standalone grid queries: acceleration::Grid (utils/grid.hpp:29-638)       */

typedef struct {
  int dims;
  float mn[3];
  float bin_size;
  int ext[3];
  long nbins;
  const float* x;
  unsigned* offsets; /* nbins + 1 */
  unsigned* perm;
} grid_q;

/* grid.hpp:222-230 (division, truncation, clamp) and :235-259 (x fastest) */
static void gq_coords(const grid_q* g, const float* p, int* c) {
  for (int d = 0; d < g->dims; ++d) {
    int v = (int)((p[d] - g->mn[d]) / g->bin_size);
    int hi = g->ext[d] - 1;
    v = v < hi ? v : hi;
    c[d] = v < 0 ? 0 : v;
  }
}
static long gq_flat(const grid_q* g, const int* c) {
  long b = c[0];
  if (g->dims >= 2) b += (long)c[1] * g->ext[0];
  if (g->dims >= 3) b += (long)c[2] * ((long)g->ext[0] * g->ext[1]);
  return b;
}
/* grid.hpp:307-340 linear_index_to_offset + :346-373 is_bin_outside_extents:
 * the bin of task t around c, or -1 outside the grid */
static long gq_task_bin(const grid_q* g, const int* c, int t, int side, int r) {
  int nb[3] = {0, 0, 0};
  int off[3] = {t % side - r, 0, 0};
  if (g->dims == 2) off[1] = t / side - r;
  if (g->dims == 3) { int tmp = t / side; off[1] = tmp % side - r; off[2] = tmp / side - r; }
  for (int d = 0; d < g->dims; ++d) {
    nb[d] = c[d] + off[d];
    if (nb[d] < 0 || nb[d] >= g->ext[d]) return -1;
  }
  return gq_flat(g, nb);
}
static int gq_tasks(const grid_q* g, int side) { return g->dims == 2 ? side * side : side * side * side; }

/* grid.hpp:413-441: nearest point within the (2r+1)^d bins, strict < keeps the first */
static int gq_nearest(const grid_q* g, const float* p, int r) {
  int c[3];
  gq_coords(g, p, c);
  const int side = 2 * r + 1;
  int best = -1;
  float bd = FLT_MAX;
  for (int t = 0; t < gq_tasks(g, side); ++t) {
    long b = gq_task_bin(g, c, t, side, r);
    if (b < 0) continue;
    for (unsigned k = g->offsets[b]; k < g->offsets[b + 1]; ++k) {
      const unsigned j = g->perm[k];
      const float s = dist2(p, g->x + (size_t)j * g->dims, g->dims);
      if (s < bd) { best = (int)j; bd = s; }
    }
  }
  return best;
}

/* grid.hpp:453-492: the target-th point of the (2r+1)^d bins in task order,
 * target = rand(0, total) = draw mod total */
static int gq_random_bins(const grid_q* g, const float* p, int r, uint32_t draw) {
  int c[3];
  gq_coords(g, p, c);
  const int side = 2 * r + 1;
  int total = 0;
  for (int t = 0; t < gq_tasks(g, side); ++t) {
    long b = gq_task_bin(g, c, t, side, r);
    if (b >= 0) total += (int)(g->offsets[b + 1] - g->offsets[b]);
  }
  const int target = total > 0 ? (int)(draw % (uint32_t)total) : 0;
  int seen = 0;
  for (int t = 0; t < gq_tasks(g, side); ++t) {
    long b = gq_task_bin(g, c, t, side, r);
    if (b < 0) continue;
    const int count = (int)(g->offsets[b + 1] - g->offsets[b]);
    if (count == 0) continue;
    if (target < seen + count) return (int)g->perm[g->offsets[b] + (unsigned)(target - seen)];
    seen += count;
  }
  return -1;
}

/* grid.hpp:505-637: among the points within the physical radius (<= r^2),
 * optionally those whose index is not a multiple of 3 (the filtered form),
 * the target-th in task order, target = urand(total) = draw mod total */
static int gq_random_radius(const grid_q* g, const float* p, float radius, uint32_t draw, int filtered) {
  int rb = (int)ceilf(radius / g->bin_size);
  if (rb < 1) rb = 1;
  int c[3];
  gq_coords(g, p, c);
  const int side = 2 * rb + 1;
  const float r2 = radius * radius;
  int total = 0;
  for (int t = 0; t < gq_tasks(g, side); ++t) {
    long b = gq_task_bin(g, c, t, side, rb);
    if (b < 0) continue;
    for (unsigned k = g->offsets[b]; k < g->offsets[b + 1]; ++k) {
      const unsigned j = g->perm[k];
      if (dist2(p, g->x + (size_t)j * g->dims, g->dims) <= r2 && (!filtered || j % 3 != 0)) ++total;
    }
  }
  if (total == 0) return -1;
  const int target = (int)(draw % (uint32_t)total);
  int seen = 0;
  for (int t = 0; t < gq_tasks(g, side); ++t) {
    long b = gq_task_bin(g, c, t, side, rb);
    if (b < 0) continue;
    for (unsigned k = g->offsets[b]; k < g->offsets[b + 1]; ++k) {
      const unsigned j = g->perm[k];
      if (dist2(p, g->x + (size_t)j * g->dims, g->dims) <= r2 && (!filtered || j % 3 != 0)) {
        if (seen == target) return (int)j;
        ++seen;
      }
    }
  }
  return -1;
}

int tecs_oracle_grid_query(int dims, const float* points, unsigned n, const float* min_bounds,
                           const float* max_bounds, float bin_size, const float* queries, unsigned m,
                           const uint32_t* draws, float radius, int32_t* near1, int32_t* near2, int32_t* rbins,
                           int32_t* rrad, int32_t* rfilt) {
  if (dims != 2 && dims != 3) { set_err("dims must be 2 or 3"); return -1; }
  if (!(bin_size > 0.0f)) { set_err("bin size must be > 0"); return -1; }
  grid_q g;
  memset(&g, 0, sizeof g);
  g.dims = dims;
  g.bin_size = bin_size;
  g.nbins = 1;
  for (int d = 0; d < 3; ++d) g.ext[d] = 1;
  for (int d = 0; d < dims; ++d) {
    g.mn[d] = min_bounds[d];
    g.ext[d] = (int)ceilf((max_bounds[d] - min_bounds[d]) / bin_size); /* grid.hpp:201-206 */
    if (g.ext[d] < 1) { set_err("max_bounds must exceed min_bounds"); return -1; }
    g.nbins *= g.ext[d];
  }
  g.x = points;
  g.offsets = (unsigned*)calloc((size_t)g.nbins + 1, 4);
  g.perm = (unsigned*)malloc((size_t)(n ? n : 1) * 4);
  unsigned* key = (unsigned*)malloc((size_t)(n ? n : 1) * 4);
  unsigned* cnt = (unsigned*)calloc((size_t)g.nbins + 1, 4);
  /* rebuild (grid.hpp:389-401): bin keys, BinSort in ascending index order */
  for (unsigned i = 0; i < n; ++i) {
    int c[3];
    gq_coords(&g, points + (size_t)i * dims, c);
    key[i] = (unsigned)gq_flat(&g, c);
    cnt[key[i]]++;
  }
  unsigned acc = 0;
  for (long b = 0; b <= g.nbins; ++b) { g.offsets[b] = acc; acc += cnt[b]; cnt[b] = 0; }
  for (unsigned i = 0; i < n; ++i) g.perm[g.offsets[key[i]] + cnt[key[i]]++] = i;
  for (unsigned q = 0; q < m; ++q) {
    const float* p = queries + (size_t)q * dims;
    if (near1) near1[q] = gq_nearest(&g, p, 1);
    if (near2) near2[q] = gq_nearest(&g, p, 2);
    if (rbins) rbins[q] = gq_random_bins(&g, p, 1, draws[q]);
    if (rrad) rrad[q] = gq_random_radius(&g, p, radius, draws[q], 0);
    if (rfilt) rfilt[q] = gq_random_radius(&g, p, radius, draws[q], 1);
  }
  free(g.offsets); free(g.perm); free(key); free(cnt);
  return 0;
}
