// delaunay_star.cuh -- the Delaunay finder for any number of cells.
//
// The reference's NaiveDelaunay (include/pair_finders/naive_delaunay.hpp:31-294)
// applies an in-cutoff pair (i, j)
//   2-D (:45-99):   once per third point k whose float circumcircle through
//                   i, j, k is non-degenerate (|den| > FLT_EPSILON) and holds
//                   no other point (distance^2 <= r^2 rejects);
//   3-D (:158-292): once per third point k for which some l > k spans a
//                   non-degenerate tetrahedron whose sphere holds no other
//                   point.
// It tries every k (and l) over all cells: O(N^3) work per cell.  This file
// finds the multiplicities from each cell's Delaunay star:
//
//  1. A counting-sorted copy of the positions on a uniform grid (about two
//     cells per bin) answers every geometric search below exactly: a search
//     visits every row of bins that its region (the shells around a point, a
//     ball, an open half-space, a band along a line) can touch, each row cut
//     to the region.
//  2. Star of cell i, in double.  From i's nearest neighbour a, the walk
//     moves through i's Voronoi cell: from a point x on it along a direction
//     w, the first point p that becomes as close to x + s w as i is the one
//     with the least s = (|x - p|^2 - |x - i|^2) / (2 w.(p - i)) over the
//     points with w.(p - i) > 0 (ties by index).  The midpoint of (i, a)
//     leads to a Voronoi edge (2-D: a vertex), each Voronoi edge to its
//     vertices, each vertex's faces to the next vertices; every vertex is the
//     centre of one empty circle/sphere through i ("star sphere"), and the
//     points on it with i form a simplex of i's star.
//  3. 2-D: the reference's float predicate decides, not the double geometry.
//     A triangle the float test can accept has an almost empty circumcircle,
//     so its points lie on, or within rounding of, one of i's star circles.
//     Every star circle collects the points within a tolerance of it (the
//     rounding of the float circumcentre, from the coordinates' size and the
//     triangle's shape, times a safety factor), and the reference's own float
//     test (with its emptiness check over every point the test can reach,
//     found through the grid) runs on every (j, k) drawn from that set.  On
//     the hull, the points near the line of each hull edge at i form one more
//     set (three collinear points can pass the float test there).  mult(i, j)
//     is the number of distinct k accepted: the reference's multiplicities,
//     bit for bit.
//  4. 3-D: the reference's quotients solve 2 (x_m - x_i).c = |x_m|^2 -
//     |x_i|^2, so they are the circumcentre itself; it adds x_i once more, and
//     its sphere (centre x_i + c, radius |c|) passes through i but not through
//     j, k or l.  Its test accepts simplices whose number grows with the cell
//     count, which no local search can enumerate.  The 3-D form here applies
//     the reference's counting rule to the Delaunay tetrahedra: mult(i, j) is
//     the number of distinct k = min(k, l) over the star tetrahedra
//     (i, j, k, l).
//
// The same code runs on the device (one warp per cell, k_dl_mult; Warp
// below) and on the host (the tests' driver; Solo), so the walk can be
// checked on the CPU against the naive restatement (2-D) and an independent
// Delaunay triangulation (3-D).
#pragma once

#include <float.h>
#include <math.h>
#include <stdint.h>

#if defined(__CUDACC__)
#define TECS_DL_HD __host__ __device__ __forceinline__
#else
#define TECS_DL_HD inline
#endif

namespace tecs {
namespace dl {

struct alignas(16) Pt {
  float x, y, z, w;  // a position (w unused)
};

// Bin grid of the active cells.  Bin b along dimension d covers
// [lo + b h, lo + (b + 1) h); bin1() is the one binning function, used for
// the points and for every search range, so a point inside a range's bounds
// is always inside the range's bins (floor and the affine map are monotone).
struct Grid {
  double lo[3];
  double h, inv;
  int dims[3];
  unsigned nbins;
  const unsigned* off;  // bin offsets, nbins + 1
  const unsigned* idx;  // slot of each sorted entry
  const Pt* sp;         // positions in sorted order
  const Pt* P;          // positions by slot
  unsigned n;           // active cells
  float rc2;            // cutoff^2 of the in-cutoff test
};

// error bits of one cell's search
enum : unsigned {
  kErrStar = 1u,   // more star simplices or spheres than the local arrays hold
  kErrNear = 2u,   // more points near one circle than the local array holds
  kErrPairs = 4u,  // more accepted (j, k) than the local array holds
  kErrList = 8u    // more partners than the output row holds
};

constexpr int kMaxTet = 192;     // star simplices (3-D tetrahedra, 2-D triangles)
constexpr int kMaxSph = 192;     // distinct star spheres (3-D: one per tetrahedron)
constexpr int kMaxNear = 48;     // points near one circle (2-D)
constexpr int kMaxPairs = 320;   // accepted (j, k)
constexpr double kInf = 1.0e300;
constexpr double kEps = (double)FLT_EPSILON;

// Lane policies.  Every search visits entries; Solo visits them in one
// thread (the host), Warp in the 32 lanes of a warp, each lane taking every
// 32nd entry.  Every result of a visit is combined across the warp (a vote,
// a minimum, candidates merged in lane order) before anything depends on it.
// The star and the candidate lists (Scratch) are one copy per warp, in
// shared memory on the device: every lane reads them, the leader lane writes
// them between two sync() calls.
struct Solo {
  static constexpr unsigned width = 1;
  TECS_DL_HD unsigned lane() const { return 0u; }
  TECS_DL_HD bool leader() const { return true; }
  TECS_DL_HD void sync() const {}
  TECS_DL_HD bool any(bool b) const { return b; }
  TECS_DL_HD unsigned ballot(bool b) const { return b ? 1u : 0u; }
  TECS_DL_HD unsigned bcast(unsigned v, int) const { return v; }
  TECS_DL_HD double bcast(double v, int) const { return v; }
};

#if defined(__CUDACC__)
struct Warp {
  static constexpr unsigned width = 32;
  __device__ __forceinline__ unsigned lane() const { return threadIdx.x & 31u; }
  __device__ __forceinline__ bool leader() const { return (threadIdx.x & 31u) == 0u; }
  __device__ __forceinline__ void sync() const { __syncwarp(); }
  __device__ __forceinline__ bool any(bool b) const { return __any_sync(0xffffffffu, b); }
  __device__ __forceinline__ unsigned ballot(bool b) const { return __ballot_sync(0xffffffffu, b); }
  __device__ __forceinline__ unsigned bcast(unsigned v, int src) const { return __shfl_sync(0xffffffffu, v, src); }
  __device__ __forceinline__ double bcast(double v, int src) const { return __shfl_sync(0xffffffffu, v, src); }
};
#endif

// the lowest set bit's index
TECS_DL_HD int low_bit(unsigned m) {
  int b = 0;
  while (!(m & 1u)) { m >>= 1; ++b; }
  return b;
}

// the least (key, id) over the lanes, in every lane
template <class W>
TECS_DL_HD void lane_min(const W& w, double& key, unsigned& id) {
  for (unsigned sh = W::width / 2; sh > 0; sh >>= 1) {
    const int src = (int)(w.lane() ^ sh);
    const double k2 = w.bcast(key, src);
    const unsigned i2 = w.bcast(id, src);
    if (k2 < key || (k2 == key && i2 < id)) { key = k2; id = i2; }
  }
}

struct NoRound {
  TECS_DL_HD void operator()() const {}
};

TECS_DL_HD double dmax(double a, double b) { return a > b ? a : b; }
TECS_DL_HD int imax(int a, int b) { return a > b ? a : b; }
TECS_DL_HD int imin(int a, int b) { return a < b ? a : b; }

TECS_DL_HD int bin1(const Grid& g, int d, double x) {
  const double t = floor((x - g.lo[d]) * g.inv);
  if (!(t >= 0.0)) return 0;  // also NaN
  if (t >= (double)(g.dims[d] - 1)) return g.dims[d] - 1;
  return (int)t;
}

// Bin edge and extents from the cells' bounding box [mn, mx]: about two cells
// per bin over the dimensions the cells spread along (a flat dimension gets
// one bin), at most max_bins bins.
template <int D>
TECS_DL_HD void plan_grid(Grid& g, const double* mn, const double* mx, unsigned n, unsigned max_bins) {
  double ext[3] = {0.0, 0.0, 0.0};
  // a span that is not finite (a cell at infinity) gets one bin
  for (int d = 0; d < D; ++d) ext[d] = (mx[d] - mn[d] > 0.0 && mx[d] - mn[d] < 1.0e30) ? mx[d] - mn[d] : 0.0;
  double target = n > 2u ? 0.5 * (double)n : 1.0;
  if (target > (double)max_bins) target = (double)max_bins;
  bool thin[3] = {false, false, false};
  double h = 1.0;
  for (int it = 0; it < 3; ++it) {
    double vol = 1.0;
    int k = 0;
    for (int d = 0; d < D; ++d)
      if (!thin[d]) { vol *= ext[d]; ++k; }
    if (k == 0 || !(vol > 0.0)) {
      // every spread dimension is flat: one bin per dimension of zero extent
      double m = 0.0;
      for (int d = 0; d < D; ++d) m = dmax(m, ext[d]);
      h = m > 0.0 ? m : 1.0;
      break;
    }
    h = pow(vol / target, 1.0 / (double)k);
    bool changed = false;
    for (int d = 0; d < D; ++d)
      if (!thin[d] && ext[d] < h) { thin[d] = true; changed = true; }
    if (!changed) break;
  }
  if (!(h > 0.0) || !(h < 1.0e300)) h = 1.0;
  for (;;) {
    double prod = 1.0;
    for (int d = 0; d < 3; ++d) {
      const double q = d < D ? floor(ext[d] / h) + 1.0 : 1.0;
      g.dims[d] = q < 1.0 ? 1 : (q > 2.0e9 ? 2000000000 : (int)q);
      prod *= (double)g.dims[d];
    }
    if (prod <= (double)max_bins) break;
    h *= 1.25;
  }
  for (int d = 0; d < 3; ++d) g.lo[d] = d < D ? mn[d] : 0.0;
  g.h = h;
  g.inv = 1.0 / h;
  g.nbins = (unsigned)g.dims[0] * (unsigned)g.dims[1] * (unsigned)g.dims[2];
}

TECS_DL_HD unsigned flat(const Grid& g, int x, int y, int z) {
  return ((unsigned)z * (unsigned)g.dims[1] + (unsigned)y) * (unsigned)g.dims[0] + (unsigned)x;
}

// Every entry of the bins [b0, b1] (inclusive); f(slot, pos) returns false
// to stop (the warp stops when any lane does).  round() runs in every lane
// after each round of entries (one entry per lane), where the caller merges
// what the lanes found.  One thread loads four entries at a time, to keep
// several loads in flight.
template <int D, class W, class F, class R = NoRound>
TECS_DL_HD bool visit_box(const W& w, const Grid& g, const int* b0, const int* b1, F&& f, R&& round = R{}) {
  const int z0 = D >= 3 ? b0[2] : 0, z1 = D >= 3 ? b1[2] : 0;
  for (int z = z0; z <= z1; ++z)
    for (int y = b0[1]; y <= b1[1]; ++y) {
      const unsigned lo = g.off[flat(g, b0[0], y, z)], hi = g.off[flat(g, b1[0], y, z) + 1];
      if (W::width == 1) {
        unsigned e = lo;
        for (; e + 4 <= hi; e += 4) {
          const unsigned i0 = g.idx[e], i1 = g.idx[e + 1], i2 = g.idx[e + 2], i3 = g.idx[e + 3];
          const Pt p0 = g.sp[e], p1 = g.sp[e + 1], p2 = g.sp[e + 2], p3 = g.sp[e + 3];
          if (!f(i0, p0)) return false;
          round();
          if (!f(i1, p1)) return false;
          round();
          if (!f(i2, p2)) return false;
          round();
          if (!f(i3, p3)) return false;
          round();
        }
        for (; e < hi; ++e) {
          if (!f(g.idx[e], g.sp[e])) return false;
          round();
        }
      } else {
        for (unsigned base = lo; base < hi; base += W::width) {
          const unsigned e = base + w.lane();
          bool stop = false;
          if (e < hi) stop = !f(g.idx[e], g.sp[e]);
          if (w.any(stop)) return false;
          round();
        }
      }
    }
  return true;
}

// The bins at Chebyshev distance k from bc.
template <int D, class W, class F, class R = NoRound>
TECS_DL_HD bool visit_shell(const W& w, const Grid& g, const int* bc, int k, F&& f, R&& round = R{}) {
  const int z0 = D >= 3 ? bc[2] - k : 0, z1 = D >= 3 ? bc[2] + k : 0;
  for (int z = z0; z <= z1; ++z) {
    if (z < 0 || z >= g.dims[2]) continue;
    const bool zface = D >= 3 && (z == z0 || z == z1);
    for (int y = bc[1] - k; y <= bc[1] + k; ++y) {
      if (y < 0 || y >= g.dims[1]) continue;
      const bool full = zface || y == bc[1] - k || y == bc[1] + k;
      int xs[2], nx = 0;
      if (full) {
        const int a = imax(bc[0] - k, 0), b = imin(bc[0] + k, g.dims[0] - 1);
        if (a > b) continue;
        const int lo3[3] = {a, y, z}, hi3[3] = {b, y, z};
        if (!visit_box<3>(w, g, lo3, hi3, f, round)) return false;
        continue;
      }
      if (bc[0] - k >= 0) xs[nx++] = bc[0] - k;
      if (k > 0 && bc[0] + k < g.dims[0]) xs[nx++] = bc[0] + k;
      for (int q = 0; q < nx; ++q) {
        const int c3[3] = {xs[q], y, z};
        if (!visit_box<3>(w, g, c3, c3, f, round)) return false;
      }
    }
  }
  return true;
}

// Row ranges in float.  A search region's rows are the same in every lane
// of a warp, and FP64 is scarce on this part, so the bounds are formed in
// float with a margin m far above float rounding (1e-3 of a bin plus the
// rounding of bin numbers and coordinates of the grid's size): a range can
// only grow, so no point is lost, and the tests on the points stay exact.
struct GridF {
  float lo[3], h, inv, m;
  int dims[3];
};

TECS_DL_HD GridF grid_f(const Grid& g) {
  GridF f;
  double span = 0.0;
  int dm = 1;
  for (int d = 0; d < 3; ++d) {
    f.lo[d] = (float)g.lo[d];
    f.dims[d] = g.dims[d];
    span = dmax(span, fabs(g.lo[d]) + (double)g.dims[d] * g.h);
    dm = imax(dm, g.dims[d]);
  }
  f.h = (float)g.h;
  f.inv = (float)g.inv;
  f.m = (float)(g.h * (1.0e-3 + 1.0e-6 * (double)dm) + 2.0e-6 * span);
  return f;
}

TECS_DL_HD int bin1f(const GridF& f, int d, float x) {
  const float t = floorf((x - f.lo[d]) * f.inv);
  if (!(t >= 0.0f)) return 0;  // also NaN
  if (t >= (float)(f.dims[d] - 1)) return f.dims[d] - 1;
  return (int)t;
}

// Distance from v to the interval that bin b of dimension d covers (0
// inside), the interval widened by the margin.
TECS_DL_HD float gap_to_bin(const GridF& f, int d, int b, float v) {
  const float lo = f.lo[d] + (float)b * f.h - f.m, hi = f.lo[d] + (float)(b + 1) * f.h + f.m;
  return v < lo ? lo - v : (v > hi ? v - hi : 0.0f);
}

// The bins [a, b] of row (y, z) that can hold a point p with w.(p - o) > 0.
template <int D>
TECS_DL_HD void half_range(const GridF& f, int y, int z, const float* o, const float* w, int& a, int& b) {
  // the largest w1 (y - o1) + w2 (z - o2) over the row's box, then its margin
  float off = 0.0f, aw = 0.0f;
  for (int d = 1; d < D; ++d) {
    const int bb = d == 1 ? y : z;
    const float lo = f.lo[d] + (float)bb * f.h - f.m, hi = f.lo[d] + (float)(bb + 1) * f.h + f.m;
    off += w[d] > 0.0f ? w[d] * (hi - o[d]) : w[d] * (lo - o[d]);
    aw += fabsf(w[d]);
  }
  off += aw * f.m;
  // need w0 (x - o0) + off > 0
  a = 0;
  b = f.dims[0] - 1;
  if (w[0] > 0.0f) a = bin1f(f, 0, o[0] - off / w[0] - f.m);
  else if (w[0] < 0.0f) b = bin1f(f, 0, o[0] - off / w[0] + f.m);
  else if (!(off >= 0.0f)) { a = 1; b = 0; }
}

// Every entry within distance rad of c (and a few just outside): the rows
// of bins (along x) that the ball touches, each cut to the ball's chord --
// and, given a plane (o, w), to the bins that reach its open side.
template <int D, class W, class F, class R = NoRound>
TECS_DL_HD bool visit_ball(const W& ln, const Grid& g, const double* c, double rad, F&& f, const double* o = nullptr,
                           const double* w = nullptr, R&& round = R{}) {
  if (!(rad < 1.0e18)) {
    const int b0[3] = {0, 0, 0}, b1[3] = {g.dims[0] - 1, g.dims[1] - 1, g.dims[2] - 1};
    return visit_box<D>(ln, g, b0, b1, f, round);
  }
  const GridF gf = grid_f(g);
  const float cf[3] = {(float)c[0], (float)c[1], (float)c[2]};
  const float rf = (float)rad * 1.00001f + gf.m;
  float of[3] = {0.f, 0.f, 0.f}, wf[3] = {0.f, 0.f, 0.f};
  if (w)
    for (int d = 0; d < 3; ++d) { of[d] = (float)o[d]; wf[d] = (float)w[d]; }
  const int z0 = D >= 3 ? bin1f(gf, 2, cf[2] - rf) : 0, z1 = D >= 3 ? bin1f(gf, 2, cf[2] + rf) : 0;
  const int y0 = bin1f(gf, 1, cf[1] - rf), y1 = bin1f(gf, 1, cf[1] + rf);
  const float r2 = rf * rf;
  for (int z = z0; z <= z1; ++z) {
    const float gz = D >= 3 ? gap_to_bin(gf, 2, z, cf[2]) : 0.0f;
    for (int y = y0; y <= y1; ++y) {
      const float gy = gap_to_bin(gf, 1, y, cf[1]);
      const float rem2 = r2 - gy * gy - gz * gz + 1.0e-5f * r2;
      if (rem2 < 0.0f) continue;
      const float rem = sqrtf(rem2) + gf.m;
      int a = bin1f(gf, 0, cf[0] - rem), b = bin1f(gf, 0, cf[0] + rem);
      if (w) {
        int ha, hb;
        half_range<D>(gf, y, z, of, wf, ha, hb);
        a = imax(a, ha);
        b = imin(b, hb);
        if (a > b) continue;
      }
      const int lo3[3] = {a, y, z}, hi3[3] = {b, y, z};
      if (!visit_box<3>(ln, g, lo3, hi3, f, round)) return false;
    }
  }
  return true;
}

// Every entry p with w.(p - o) > 0 (and a few on the boundary): each row of
// bins cut to the part that can reach the open side.
template <int D, class W, class F>
TECS_DL_HD bool visit_half(const W& ln, const Grid& g, const double* o, const double* w, F&& f) {
  const GridF gf = grid_f(g);
  const float of[3] = {(float)o[0], (float)o[1], (float)o[2]}, wf[3] = {(float)w[0], (float)w[1], (float)w[2]};
  const int z1 = D >= 3 ? g.dims[2] - 1 : 0;
  for (int z = 0; z <= z1; ++z)
    for (int y = 0; y < g.dims[1]; ++y) {
      int a, b;
      half_range<D>(gf, y, z, of, wf, a, b);
      if (a > b) continue;
      const int lo3[3] = {a, y, z}, hi3[3] = {b, y, z};
      if (!visit_box<3>(ln, g, lo3, hi3, f)) return false;
    }
  return true;
}

// 2-D: every entry within distance del of the line through o with unit
// normal nrm (and a few just outside): each row of bins cut to the band.
template <class W, class F, class R>
TECS_DL_HD bool visit_band(const W& w, const Grid& g, const double* o, const double* nrm, double del, F&& f,
                           R&& round) {
  const double m = 1.0e-9 * g.h;
  for (int y = 0; y < g.dims[1]; ++y) {
    const double ylo = g.lo[1] + (double)y * g.h - m, yhi = g.lo[1] + (double)(y + 1) * g.h + m;
    int a = 0, b = g.dims[0] - 1;
    if (fabs(nrm[0]) > 1.0e-12) {
      // n0 (x - o0) + n1 (y - o1) in [-del, del] over the row's y interval
      double xmn = kInf, xmx = -kInf;
      for (int e = 0; e < 4; ++e) {
        const double yy = (e & 1) ? yhi : ylo, sg = (e & 2) ? del : -del;
        const double x = o[0] + (sg - nrm[1] * (yy - o[1])) / nrm[0];
        xmn = x < xmn ? x : xmn;
        xmx = x > xmx ? x : xmx;
      }
      a = bin1(g, 0, xmn - m);
      b = bin1(g, 0, xmx + m);
    } else {
      const double half = del / fabs(nrm[1]);
      if (yhi < o[1] - half || ylo > o[1] + half) continue;
    }
    const int lo3[3] = {a, y, 0}, hi3[3] = {b, y, 0};
    if (!visit_box<3>(w, g, lo3, hi3, f, round)) return false;
  }
  return true;
}

template <int D>
TECS_DL_HD int shells_to_cover(const Grid& g, const int* bc) {
  int k = 0;
  for (int d = 0; d < D; ++d) k = imax(k, imax(bc[d], g.dims[d] - 1 - bc[d]));
  return k;
}

template <int D>
TECS_DL_HD void bin_of(const Grid& g, const double* x, int* b) {
  for (int d = 0; d < 3; ++d) b[d] = d < D ? bin1(g, d, x[d]) : 0;
}

TECS_DL_HD void load(const Pt& p, double* q) { q[0] = p.x; q[1] = p.y; q[2] = p.z; }

// ---------------------------------------------------------------------------
// The reference's float predicates, operation for operation.

TECS_DL_HD float sqlen2(const Pt& p) { return p.x * p.x + p.y * p.y; }
TECS_DL_HD float sqlen3(const Pt& p) { return (p.x * p.x + p.y * p.y) + p.z * p.z; }

// in-cutoff test: displacement = x_i - x_j, length_squared() < cutoff^2
template <int D>
TECS_DL_HD bool in_cutoff(const Grid& g, const Pt& pi, const Pt& pj) {
  const float e0 = pi.x - pj.x, e1 = pi.y - pj.y;
  float d2 = e0 * e0 + e1 * e1;
  if (D >= 3) { const float e2 = pi.z - pj.z; d2 = d2 + e2 * e2; }
  return d2 < g.rc2;
}

// naive_delaunay.hpp:62-99: triangle (i, j, k) accepted
template <class W>
TECS_DL_HD bool tri_pass(const W& w, const Grid& g, unsigned i, unsigned j, unsigned k) {
  const Pt pi = g.P[i], pj = g.P[j], pk = g.P[k];
  const float den = 2.0f * (pi.x * (pj.y - pk.y) + pj.x * (pk.y - pi.y) + pk.x * (pi.y - pj.y));
  if (fabsf(den) <= FLT_EPSILON) return false;
  const float li = sqlen2(pi), lj = sqlen2(pj), lk = sqlen2(pk);
  float c[2];
  c[0] = (li * (pj.y - pk.y) + lj * (pk.y - pi.y) + lk * (pi.y - pj.y)) / den;
  c[1] = (li * (pk.x - pj.x) + lj * (pi.x - pk.x) + lk * (pj.x - pi.x)) / den;
  const float e0 = pi.x - c[0], e1 = pi.y - c[1];
  const float r2 = e0 * e0 + e1 * e1;
  // every point the test can reach: float distance^2 <= r2 means a true
  // distance within sqrt(r2) (1 + a few eps)
  const double cc[3] = {c[0], c[1], 0.0};
  const double reach = (double)sqrtf(r2) * (1.0 + 8.0 * kEps) + 1.0e-30;
  const bool finite = cc[0] > -1.0e30 && cc[0] < 1.0e30 && cc[1] > -1.0e30 && cc[1] < 1.0e30;
  return visit_ball<2>(w, g, cc, finite ? reach : kInf, [&](unsigned m, const Pt& pm) {
    if (m == i || m == j || m == k) return true;
    const float f0 = pm.x - c[0], f1 = pm.y - c[1];
    return !(f0 * f0 + f1 * f1 <= r2);
  });
}

// ---------------------------------------------------------------------------
// Geometry of the star, in double.

struct Hit {
  unsigned id;
  double s;
};

// The first point p (not in ex) that becomes as close to x0 + s w as i is:
// the least s = (|x0 - p|^2 - |x0 - i|^2) / (2 w.(p - i)) over w.(p - i) > 0.
// Every point with parameter <= s lies in the ball B(s) about x0 + s w
// through i (on the open side of the plane through i), and B(s) grows with
// s.  So: balls of doubling s, each cut to the open side, from the radius
// of the empty ball about x0, until one holds a point; its least
// parameter is then the answer (after one more ball at that parameter, for
// points just outside the last ball's bins); past the grid's size, every
// bin on the open side of the plane.
template <int D, class W>
TECS_DL_HD Hit shoot(const W& ln, const Grid& g, const double* x0, const double* w, const double* pi,
                     const unsigned* ex, int nex) {
  double pow0 = 0.0;
  for (int d = 0; d < D; ++d) { const double v = x0[d] - pi[d]; pow0 += v * v; }
  Hit best{~0u, kInf};  // this lane's, then the warp's after each visit
  auto take = [&](unsigned id, const Pt& p) {
    for (int e = 0; e < nex; ++e)
      if (id == ex[e]) return true;
    double q[3];
    load(p, q);
    double wp = 0.0, nn = 0.0, num = 0.0;
    for (int d = 0; d < D; ++d) {
      const double v = q[d] - pi[d], u = q[d] - x0[d];
      wp += w[d] * v;
      nn += v * v;
      num += u * u;
    }
    if (!(wp > 0.0) || wp * wp <= 1.0e-18 * nn) return true;  // on or behind the plane through i
    const double s = (num - pow0) / (2.0 * wp);
    if (s < best.s || (s == best.s && id < best.id)) best = Hit{id, s};
    return true;
  };
  auto reduce = [&]() { lane_min(ln, best.s, best.id); };
  // visits B(s) (with a margin)
  auto ball_at = [&](double s) {
    double c[3] = {0.0, 0.0, 0.0}, r2 = 0.0;
    for (int d = 0; d < D; ++d) {
      c[d] = x0[d] + s * w[d];
      const double v = c[d] - pi[d];
      r2 += v * v;
    }
    visit_ball<D>(ln, g, c, sqrt(r2) * (1.0 + 1.0e-9) + 1.0e-9 * g.h, take, pi, w);
    reduce();
  };
  // the first ball: s = the distance from x0 to i (the radius of the empty
  // ball the search starts from), at least a twentieth of a bin
  double span2 = 0.0;
  for (int d = 0; d < D; ++d) { const double e = (double)g.dims[d] * g.h; span2 += e * e; }
  const double span = sqrt(span2);
  for (double s = dmax(sqrt(pow0), 0.05 * g.h); s < 4.0 * span; s *= 2.0) {
    ball_at(s);
    if (best.id != ~0u) {
      if (best.s > s) ball_at(best.s);
      return best;
    }
  }
  visit_half<D>(ln, g, pi, w, take);
  reduce();
  return best;
}

// i's nearest other cell at a non-zero distance (ties by index).
template <int D, class W>
TECS_DL_HD unsigned nearest(const W& ln, const Grid& g, const double* pi, unsigned self) {
  double bd = kInf;
  unsigned bid = ~0u;
  int bc[3];
  bin_of<D>(g, pi, bc);
  const int kmax = shells_to_cover<D>(g, bc);
  for (int k = 0; k <= kmax; ++k) {
    visit_shell<D>(ln, g, bc, k, [&](unsigned id, const Pt& p) {
      if (id == self) return true;
      double q[3];
      load(p, q);
      double d2 = 0.0;
      for (int d = 0; d < D; ++d) { const double v = q[d] - pi[d]; d2 += v * v; }
      if (d2 > 0.0 && (d2 < bd || (d2 == bd && id < bid))) { bd = d2; bid = id; }
      return true;
    });
    lane_min(ln, bd, bid);
    if (bid != ~0u && ((double)k - 1.0e-3) * g.h >= sqrt(bd)) break;
  }
  return bid;
}

struct Tet {
  unsigned v[3];  // the simplex's other points, ascending (2-D: v[2] unused)
  int sph;
  unsigned done;  // bit f: the face opposite v[f] has been crossed
};

struct Sph {
  double c[3];
  double R;    // squared radius
  double tol;  // half-width of the near shell, in units of |p - c|^2 - R
};

struct Star {
  Tet t[kMaxTet];
  Sph s[kMaxSph];
  int nt, ns;
  unsigned err;
  unsigned open_end[2];  // 2-D: the neighbours at which the walk left the grid (i on the hull)
  int n_open;
};

struct JK {
  unsigned j, k;
};

// One cell's working state: the star, the accepted (j, k), one circle's
// candidate points.
struct Scratch {
  Star st;
  JK pairs[kMaxPairs];
  unsigned near[kMaxNear];
  double dev[kMaxNear];
};

// Rounding of the reference's float circumcentre for a simplex of this shape
// and coordinate size, as a tolerance on |p - c|^2 - R, with a safety factor.
template <int D>
TECS_DL_HD double shell_tol(const double* pi, const double (*e)[3], double R) {
  double L = 0.0, hm = 0.0;
  for (int d = 0; d < D; ++d) L = dmax(L, fabs(pi[d]));
  for (int q = 0; q < D; ++q) {
    double n2 = 0.0;
    for (int d = 0; d < D; ++d) { n2 += e[q][d] * e[q][d]; L = dmax(L, fabs(pi[d] + e[q][d])); }
    hm = dmax(hm, sqrt(n2));
  }
  double det;
  if (D == 2) det = e[0][0] * e[1][1] - e[0][1] * e[1][0];
  else det = e[0][0] * (e[1][1] * e[2][2] - e[1][2] * e[2][1]) - e[0][1] * (e[1][0] * e[2][2] - e[1][2] * e[2][0]) +
             e[0][2] * (e[1][0] * e[2][1] - e[1][1] * e[2][0]);
  const double den = dmax(2.0 * fabs(det), 1.0e-300);
  double hp = 1.0;
  for (int q = 0; q < D - 1; ++q) hp *= hm;
  // Centre error (u = eps/2, the unit roundoff): the |x|^2 terms carry about
  // 3 u L^2 each, times cofactors of size h^(D-1), summed over D + 1 terms
  // with as many roundings of partial sums of size L^2 h^(D-1); the
  // determinant's own relative error (about 6 u L h^(D-1) / den) moves a
  // centre of size L by as much again: about 21 u L^2 h^(D-1) / den in all,
  // taken here with a factor 2 to spare.
  const double u = 0.5 * kEps;
  const double dc = 48.0 * u * (L * L + hm * hm) * hp / den + 8.0 * u * L;
  // |p - c|^2 - R moves by 2 r dc + dc^2 with the centre; the distance
  // test's own roundings add a few u (R + L r); a factor 4 over both
  const double r = sqrt(R);
  return 4.0 * (2.0 * r * dc + dc * dc) + 32.0 * u * (R + L * r);
}

template <int D>
TECS_DL_HD int find_sphere(Star& st, const double* c, double R) {
  const double rr = sqrt(R);
  for (int q = 0; q < st.ns; ++q) {
    double d2 = 0.0;
    for (int d = 0; d < D; ++d) { const double v = st.s[q].c[d] - c[d]; d2 += v * v; }
    const double lim = 1.0e-9 * (rr + sqrt(st.s[q].R)) + 1.0e-200;
    if (d2 <= lim * lim) return q;
  }
  return -1;
}

// Adds the simplex (i, a, b[, d]) with circumcentre c; returns its index.
// Every lane computes the same values from the same snapshot; the leader
// writes them.
template <int D, class W>
TECS_DL_HD int add_simplex(const W& ln, const Grid& g, Star& st, const double* pi, unsigned a, unsigned b,
                           unsigned d3, const double* c) {
  unsigned v[3] = {a, b, D == 3 ? d3 : ~0u};
  // ascending (three elements)
  for (int x = 0; x < 2; ++x)
    for (int y = 0; y < 2 - x; ++y)
      if (v[y] > v[y + 1]) { const unsigned t = v[y]; v[y] = v[y + 1]; v[y + 1] = t; }
  const int nt = st.nt, ns = st.ns;
  for (int q = 0; q < nt; ++q)
    if (st.t[q].v[0] == v[0] && st.t[q].v[1] == v[1] && st.t[q].v[2] == v[2]) return q;
  double R = 0.0;
  for (int d = 0; d < D; ++d) { const double u = c[d] - pi[d]; R += u * u; }
  // 3-D counts come from the tetrahedra; their centres only start the next
  // searches, so each keeps its own (no merging, no tolerance)
  double tol = 0.0;
  int sp = -1;
  if (D == 2) {
    double e[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    for (int q = 0; q < D; ++q) {
      double p[3];
      load(g.P[v[q]], p);
      for (int d = 0; d < D; ++d) e[q][d] = p[d] - pi[d];
    }
    tol = shell_tol<D>(pi, e, R);
    sp = find_sphere<D>(st, c, R);
  }
  const bool fresh = sp < 0;
  const bool full = nt >= kMaxTet || (fresh && ns >= kMaxSph);
  const double old_tol = fresh ? 0.0 : st.s[sp].tol;
  ln.sync();  // every lane has read what the leader writes next
  if (ln.leader()) {
    if (full) {
      st.err |= kErrStar;
    } else {
      const int spw = fresh ? ns : sp;
      if (fresh) {
        for (int d = 0; d < 3; ++d) st.s[spw].c[d] = d < D ? c[d] : 0.0;
        st.s[spw].R = R;
        st.s[spw].tol = tol;
        st.ns = ns + 1;
      } else if (tol > old_tol) {
        st.s[spw].tol = tol;
      }
      st.t[nt].v[0] = v[0];
      st.t[nt].v[1] = v[1];
      st.t[nt].v[2] = v[2];
      st.t[nt].sph = spw;
      st.t[nt].done = 0u;
      st.nt = nt + 1;
    }
  }
  ln.sync();
  return full ? -1 : nt;
}

template <class W>
TECS_DL_HD void mark_face(const W& ln, Star& st, int q, unsigned opposite) {
  if (q < 0) return;
  unsigned bits = st.t[q].done;
  for (int f = 0; f < 3; ++f)
    if (st.t[q].v[f] == opposite) bits |= 1u << f;
  ln.sync();
  if (ln.leader()) st.t[q].done = bits;
  ln.sync();
}

template <class W>
TECS_DL_HD void add_open_end(const W& ln, Star& st, unsigned e) {
  const int k = st.n_open;
  ln.sync();
  if (ln.leader() && k < 2) {
    st.open_end[k] = e;
    st.n_open = k + 1;
  }
  ln.sync();
}

TECS_DL_HD void normalize3(double* v, int D) {
  double n = 0.0;
  for (int d = 0; d < D; ++d) n += v[d] * v[d];
  n = sqrt(n);
  if (n > 0.0)
    for (int d = 0; d < D; ++d) v[d] /= n;
}

TECS_DL_HD void cross3(const double* a, const double* b, double* c) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}

// 2-D: walk around i's Voronoi polygon from the edge of its nearest
// neighbour a: from the midpoint of (i, a) to the vertex on one side, then
// from vertex to vertex, each time across the edge of the newest neighbour,
// until the walk is back at a (closed) or leaves the grid (i on the hull);
// then the same from the other side.
template <class W>
TECS_DL_HD void star2(const W& ln, const Grid& g, unsigned i, Star& st) {
  double pi[3];
  load(g.P[i], pi);
  const unsigned a = nearest<2>(ln, g, pi, i);
  if (a == ~0u) return;
  double pa[3];
  load(g.P[a], pa);
  const double x0[3] = {(pi[0] + pa[0]) * 0.5, (pi[1] + pa[1]) * 0.5, 0.0};
  double u[3] = {-(pa[1] - pi[1]), pa[0] - pi[0], 0.0};
  normalize3(u, 2);
  for (int side = 0; side < 2; ++side) {
    const double w[3] = {side ? -u[0] : u[0], side ? -u[1] : u[1], 0.0};
    const unsigned ex[2] = {i, a};
    const Hit h = shoot<2>(ln, g, x0, w, pi, ex, 2);
    if (h.id == ~0u) {
      add_open_end(ln, st, a);  // (i, a) is a hull edge
      continue;
    }
    const double c[3] = {x0[0] + h.s * w[0], x0[1] + h.s * w[1], 0.0};
    const int nt0 = st.nt;
    int q = add_simplex<2>(ln, g, st, pi, a, h.id, ~0u, c);
    if (q < 0 || (side == 1 && st.nt == nt0)) return;
    unsigned prev = a, cur = h.id;
    double v[3] = {c[0], c[1], 0.0};
    bool closed = false;
    for (int guard = 0; guard < kMaxTet && !closed; ++guard) {
      double pc[3], pp[3];
      load(g.P[cur], pc);
      load(g.P[prev], pp);
      double n[3] = {-(pc[1] - pi[1]), pc[0] - pi[0], 0.0};
      if (n[0] * (pp[0] - pi[0]) + n[1] * (pp[1] - pi[1]) > 0.0) { n[0] = -n[0]; n[1] = -n[1]; }
      normalize3(n, 2);
      const unsigned ex2[3] = {i, cur, prev};
      const Hit h2 = shoot<2>(ln, g, v, n, pi, ex2, 3);
      if (h2.id == ~0u) {  // open: (i, cur) is a hull edge
        add_open_end(ln, st, cur);
        break;
      }
      const double c2[3] = {v[0] + h2.s * n[0], v[1] + h2.s * n[1], 0.0};
      const int cur_sph = st.t[q].sph, ns0 = st.ns, nt1 = st.nt;
      const int q2 = add_simplex<2>(ln, g, st, pi, cur, h2.id, ~0u, c2);
      if (q2 < 0) return;
      // back at a, at a triangle met before, or at an earlier vertex: closed
      closed = h2.id == a || st.nt == nt1 || (st.ns == ns0 && st.t[q2].sph != cur_sph);
      prev = cur;
      cur = h2.id;
      v[0] = c2[0];
      v[1] = c2[1];
      q = q2;
    }
    if (closed) return;
  }
}

// 3-D: breadth-first over i's Voronoi vertices, crossing each face of each
// star tetrahedron that contains i once.
template <class W>
TECS_DL_HD void star3(const W& ln, const Grid& g, unsigned i, Star& st) {
  double pi[3];
  load(g.P[i], pi);
  const unsigned a = nearest<3>(ln, g, pi, i);
  if (a == ~0u) return;
  double pa[3];
  load(g.P[a], pa);
  const double ea[3] = {pa[0] - pi[0], pa[1] - pi[1], pa[2] - pi[2]};
  double x0[3] = {(pi[0] + pa[0]) * 0.5, (pi[1] + pa[1]) * 0.5, (pi[2] + pa[2]) * 0.5};
  // a direction across the bisector plane of (i, a)
  int ax = 0;
  if (fabs(ea[1]) < fabs(ea[ax])) ax = 1;
  if (fabs(ea[2]) < fabs(ea[ax])) ax = 2;
  double unit[3] = {0, 0, 0};
  unit[ax] = 1.0;
  double u[3];
  cross3(ea, unit, u);
  normalize3(u, 3);
  const unsigned ex[2] = {i, a};
  Hit h = shoot<3>(ln, g, x0, u, pi, ex, 2);
  if (h.id == ~0u) {
    for (int d = 0; d < 3; ++d) u[d] = -u[d];
    h = shoot<3>(ln, g, x0, u, pi, ex, 2);
  }
  if (h.id == ~0u) return;  // every other point on the line through i and a
  const unsigned b = h.id;
  const double x1[3] = {x0[0] + h.s * u[0], x0[1] + h.s * u[1], x0[2] + h.s * u[2]};
  double pb[3];
  load(g.P[b], pb);
  const double eb[3] = {pb[0] - pi[0], pb[1] - pi[1], pb[2] - pi[2]};
  double n[3];
  cross3(ea, eb, n);
  normalize3(n, 3);
  const unsigned ex3[3] = {i, a, b};
  int q0[2] = {-1, -1};
  unsigned apex[2] = {~0u, ~0u};
  for (int side = 0; side < 2; ++side) {
    double w[3] = {side ? -n[0] : n[0], side ? -n[1] : n[1], side ? -n[2] : n[2]};
    const Hit hd = shoot<3>(ln, g, x1, w, pi, ex3, 3);
    if (hd.id == ~0u) continue;
    const double c[3] = {x1[0] + hd.s * w[0], x1[1] + hd.s * w[1], x1[2] + hd.s * w[2]};
    q0[side] = add_simplex<3>(ln, g, st, pi, a, b, hd.id, c);
    apex[side] = hd.id;
  }
  // the face (i, a, b) between the two first tetrahedra is crossed
  mark_face(ln, st, q0[0], apex[0]);
  mark_face(ln, st, q0[1], apex[1]);
  for (int q = 0; q < st.nt; ++q) {
    for (int f = 0; f < 3; ++f) {
      const unsigned done = st.t[q].done;
      if (done & (1u << f)) continue;
      ln.sync();
      if (ln.leader()) st.t[q].done = done | (1u << f);
      ln.sync();
      const unsigned O = st.t[q].v[f], A = st.t[q].v[(f + 1) % 3], B = st.t[q].v[(f + 2) % 3];
      double pA[3], pB[3], pO[3];
      load(g.P[A], pA);
      load(g.P[B], pB);
      load(g.P[O], pO);
      const double eA[3] = {pA[0] - pi[0], pA[1] - pi[1], pA[2] - pi[2]};
      const double eB[3] = {pB[0] - pi[0], pB[1] - pi[1], pB[2] - pi[2]};
      double w[3];
      cross3(eA, eB, w);
      if (w[0] * (pO[0] - pi[0]) + w[1] * (pO[1] - pi[1]) + w[2] * (pO[2] - pi[2]) > 0.0)
        for (int d = 0; d < 3; ++d) w[d] = -w[d];
      normalize3(w, 3);
      const Sph& S = st.s[st.t[q].sph];
      const unsigned exf[4] = {i, A, B, O};
      const Hit hf = shoot<3>(ln, g, S.c, w, pi, exf, 4);
      if (hf.id == ~0u) continue;  // open face: i is on the hull
      const double c[3] = {S.c[0] + hf.s * w[0], S.c[1] + hf.s * w[1], S.c[2] + hf.s * w[2]};
      const int q2 = add_simplex<3>(ln, g, st, pi, A, B, hf.id, c);
      if (q2 < 0) return;
      mark_face(ln, st, q2, hf.id);
    }
  }
}

// ---------------------------------------------------------------------------
// One cell: its partners and how often the reference applies each pair.
// out[0..return) = (j, reps), ascending j; *err gets the error bits.

template <int D, class W>
TECS_DL_HD unsigned cell_mult(const W& ln, const Grid& g, unsigned i, unsigned* out_j, unsigned* out_r, unsigned cap,
                              unsigned* err, Scratch& sc) {
  Star& st = sc.st;
  JK* pairs = sc.pairs;
  unsigned* near = sc.near;
  double* dev = sc.dev;
  ln.sync();
  if (ln.leader()) {
    st.nt = 0;
    st.ns = 0;
    st.err = 0u;
    st.n_open = 0;
  }
  ln.sync();
  if (D == 2) star2(ln, g, i, st);
  else star3(ln, g, i, st);
  unsigned e = st.err;
  int np = 0;
  const Pt Pi = g.P[i];
  auto record = [&](unsigned j, unsigned k) {
    for (int p = 0; p < np; ++p)
      if (pairs[p].j == j && pairs[p].k == k) return;
    if (np >= kMaxPairs) { e |= kErrPairs; return; }
    ln.sync();
    if (ln.leader()) pairs[np] = JK{j, k};
    ln.sync();
    ++np;
  };
  if (D == 3) {
    // every star tetrahedron (i, a, b, c): j one of them, k the lesser other
    for (int q = 0; q < st.nt; ++q) {
      const unsigned* v = st.t[q].v;
      for (int f = 0; f < 3; ++f) {
        const unsigned j = v[f], k = v[f == 0 ? 1 : 0];
        if (in_cutoff<3>(g, Pi, g.P[j])) record(j, k);
      }
    }
  } else {
    // the star circles, then one group per hull edge at i
    for (int q = 0; q < st.ns + st.n_open; ++q) {
      // the circle's own triangle points first (deviation -1: never dropped),
      // then every point on or near it, or inside; when the array is full
      // the point farthest from the circle gives way
      int nn = 0;
      auto put = [&](unsigned id, double f) {
        for (int x = 0; x < nn; ++x)
          if (near[x] == id) return;
        int at = nn;
        if (nn >= kMaxNear) {
          e |= kErrNear;
          at = 0;
          for (int x = 1; x < nn; ++x)
            if (dev[x] > dev[at]) at = x;
          if (!(f < dev[at])) return;
        }
        ln.sync();
        if (ln.leader()) { near[at] = id; dev[at] = f; }
        ln.sync();
        if (at == nn) ++nn;
      };
      // a lane's candidate of the current round, put by every lane in lane order
      bool has = false;
      unsigned cid = 0u;
      double cdev = 0.0;
      auto merge = [&]() {
        unsigned m = ln.ballot(has);
        while (m) {
          const int src = low_bit(m);
          m &= m - 1u;
          put(ln.bcast(cid, src), ln.bcast(cdev, src));
        }
        has = false;
      };
      if (q < st.ns) {
        const Sph S = st.s[q];
        double pi2[3], hm = 0.0;
        load(Pi, pi2);
        for (int t = 0; t < st.nt; ++t)
          if (st.t[t].sph == q)
            for (int v = 0; v < 2; ++v) {
              put(st.t[t].v[v], -1.0);
              double pv[3];
              load(g.P[st.t[t].v[v]], pv);
              hm = dmax(hm, sqrt((pv[0] - pi2[0]) * (pv[0] - pi2[0]) + (pv[1] - pi2[1]) * (pv[1] - pi2[1])));
            }
        // |p - c|^2 - R <= tol, in float with a margin above its rounding:
        // the set may only grow (every member's triangles are tested by the
        // reference's float test), so no double work is needed per point
        const float cx = (float)S.c[0], cy = (float)S.c[1], Rf = (float)S.R, tf = (float)S.tol;
        const float reach = sqrtf(fmaxf(Rf + tf, 0.0f));
        const float slack = 1.0e-5f * (Rf + tf + 2.0f * reach * (fabsf(cx) + fabsf(cy) + reach)) + 1.0e-30f;
        auto near_test = [&](unsigned id, const Pt& p) {
          if (id == i) return true;
          const float u0 = p.x - cx, u1 = p.y - cy;
          const float f = u0 * u0 + u1 * u1 - Rf;
          if (f <= tf + slack) { has = true; cid = id; cdev = fabs((double)f); }
          return true;
        };
        // An alternative triangle to the circle's own is local: its points
        // lie within a few of the triangle's edges of i.  A circle much
        // larger than its triangle (a hull triangle, bulging out of the
        // hull) meets the other cells only along the hull, where a wide
        // float tolerance would take in cells far from i whose triangles
        // with i enclose the hull's interior; those are searched near i.
        const double rad = sqrt(S.R + S.tol) * (1.0 + 1.0e-9) + 1.0e-9 * g.h;
        const double local = 4.0 * hm + 4.0 * g.h;
        if (local < rad) visit_ball<2>(ln, g, pi2, local, near_test, nullptr, nullptr, merge);
        else visit_ball<2>(ln, g, S.c, rad, near_test, nullptr, nullptr, merge);
      } else {
        // A hull edge (i, e): three points that are collinear in exact
        // arithmetic can still give the reference a determinant above
        // FLT_EPSILON (it rounds products of size L h, L the coordinates'
        // size), and the huge circle of such a triangle holds no point when
        // it bulges out of the hull, along a supporting line of i.  So the
        // points near the line of each hull edge form one more group.
        const unsigned e_id = st.open_end[q - st.ns];
        double pi2[3], pe[3];
        load(Pi, pi2);
        load(g.P[e_id], pe);
        double nrm[3] = {-(pe[1] - pi2[1]), pe[0] - pi2[0], 0.0};
        normalize3(nrm, 2);
        const double L = dmax(dmax(fabs(g.lo[0]), fabs(g.lo[0] + g.dims[0] * g.h)),
                              dmax(fabs(g.lo[1]), fabs(g.lo[1] + g.dims[1] * g.h)));
        const double span = (double)(g.dims[0] + g.dims[1]) * g.h;
        const double del = 64.0 * 0.5 * kEps * L * (1.0 + span) + (double)FLT_EPSILON;
        put(e_id, -1.0);
        visit_band(ln, g, pi2, nrm, del, [&](unsigned id, const Pt& p) {
          if (id == i) return true;
          const double f = fabs(((double)p.x - pi2[0]) * nrm[0] + ((double)p.y - pi2[1]) * nrm[1]);
          if (f <= del) { has = true; cid = id; cdev = f; }
          return true;
        }, merge);
      }
      // the reference's test on every choice of j (in cutoff) and k among them
      for (int a = 0; a < nn; ++a) {
        const unsigned j = near[a];
        if (!in_cutoff<2>(g, Pi, g.P[j])) continue;
        for (int b = 0; b < nn; ++b) {
          const unsigned k = near[b];
          if (k == j) continue;
          bool have = false;
          for (int p = 0; p < np && !have; ++p) have = pairs[p].j == j && pairs[p].k == k;
          if (!have && tri_pass(ln, g, i, j, k)) record(j, k);
        }
      }
    }
  }
  // (j, number of distinct k), ascending j: sorted by the leader
  ln.sync();
  if (ln.leader())
    for (int x = 1; x < np; ++x) {
      const JK v = pairs[x];
      int y = x - 1;
      while (y >= 0 && (pairs[y].j > v.j || (pairs[y].j == v.j && pairs[y].k > v.k))) { pairs[y + 1] = pairs[y]; --y; }
      pairs[y + 1] = v;
    }
  ln.sync();
  unsigned len = 0;
  for (int x = 0; x < np;) {
    int y = x;
    while (y < np && pairs[y].j == pairs[x].j) ++y;
    if (len < cap) {
      out_j[len] = pairs[x].j;
      out_r[len] = (unsigned)(y - x);
      ++len;
    } else {
      e |= kErrList;
    }
    x = y;
  }
  *err = e;
  return len;
}

}  // namespace dl
}  // namespace tecs
