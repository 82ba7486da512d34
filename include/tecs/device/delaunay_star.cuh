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
//     visits every bin that a ball or box can touch, in growing shells.
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
//     found through the grid) runs on every (j, k) drawn from that set.
//     mult(i, j) is the number of distinct k accepted: the reference's
//     multiplicities, bit for bit.
//  4. 3-D: the reference's quotients solve 2 (x_m - x_i).c = |x_m|^2 -
//     |x_i|^2, so they are the circumcentre itself; it adds x_i once more, and
//     its sphere (centre x_i + c, radius |c|) passes through i but not through
//     j, k or l.  Its test accepts simplices whose number grows with the cell
//     count, which no local search can enumerate.  The 3-D form here applies
//     the reference's counting rule to the Delaunay tetrahedra: mult(i, j) is
//     the number of distinct k = min(k, l) over the star tetrahedra
//     (i, j, k, l).
//
// The same code runs on the device (one thread per cell, k_dl_mult) and on
// the host (the tests' driver), so the walk can be checked on the CPU against
// the naive restatement (2-D) and an independent Delaunay triangulation (3-D).
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
constexpr int kMaxSph = 128;     // distinct star spheres
constexpr int kMaxNear = 48;     // points near one circle (2-D)
constexpr int kMaxPairs = 320;   // accepted (j, k)
constexpr double kInf = 1.0e300;
constexpr double kEps = (double)FLT_EPSILON;

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

// Every entry of the bins [b0, b1] (inclusive); f(slot, pos) returns false to stop.
template <int D, class F>
TECS_DL_HD bool visit_box(const Grid& g, const int* b0, const int* b1, F&& f) {
  const int z0 = D >= 3 ? b0[2] : 0, z1 = D >= 3 ? b1[2] : 0;
  for (int z = z0; z <= z1; ++z)
    for (int y = b0[1]; y <= b1[1]; ++y) {
      const unsigned lo = g.off[flat(g, b0[0], y, z)], hi = g.off[flat(g, b1[0], y, z) + 1];
      for (unsigned e = lo; e < hi; ++e)
        if (!f(g.idx[e], g.sp[e])) return false;
    }
  return true;
}

// The bins at Chebyshev distance k from bc.
template <int D, class F>
TECS_DL_HD bool visit_shell(const Grid& g, const int* bc, int k, F&& f) {
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
        if (!visit_box<3>(g, lo3, hi3, f)) return false;
        continue;
      }
      if (bc[0] - k >= 0) xs[nx++] = bc[0] - k;
      if (k > 0 && bc[0] + k < g.dims[0]) xs[nx++] = bc[0] + k;
      for (int q = 0; q < nx; ++q) {
        const int c3[3] = {xs[q], y, z};
        if (!visit_box<3>(g, c3, c3, f)) return false;
      }
    }
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

// Box of bins that holds every point a float test at (c, reach) can reach.
template <int D>
TECS_DL_HD void reach_bins(const Grid& g, const float* c, float reach, int* b0, int* b1) {
  bool all = !(reach < 3.0e38f);
  for (int d = 0; d < D; ++d) all = all || !(c[d] > -3.0e38f && c[d] < 3.0e38f);
  for (int d = 0; d < 3; ++d) { b0[d] = 0; b1[d] = g.dims[d] - 1; }
  if (all) return;
  const double m = (double)reach * (1.0 + 8.0 * kEps) + 1.0e-30;
  for (int d = 0; d < D; ++d) {
    b0[d] = bin1(g, d, (double)c[d] - m);
    b1[d] = bin1(g, d, (double)c[d] + m);
  }
}

// naive_delaunay.hpp:62-99: triangle (i, j, k) accepted
TECS_DL_HD bool tri_pass(const Grid& g, unsigned i, unsigned j, unsigned k) {
  const Pt pi = g.P[i], pj = g.P[j], pk = g.P[k];
  const float den = 2.0f * (pi.x * (pj.y - pk.y) + pj.x * (pk.y - pi.y) + pk.x * (pi.y - pj.y));
  if (fabsf(den) <= FLT_EPSILON) return false;
  const float li = sqlen2(pi), lj = sqlen2(pj), lk = sqlen2(pk);
  float c[2];
  c[0] = (li * (pj.y - pk.y) + lj * (pk.y - pi.y) + lk * (pi.y - pj.y)) / den;
  c[1] = (li * (pk.x - pj.x) + lj * (pi.x - pk.x) + lk * (pj.x - pi.x)) / den;
  const float e0 = pi.x - c[0], e1 = pi.y - c[1];
  const float r2 = e0 * e0 + e1 * e1;
  int b0[3], b1[3];
  reach_bins<2>(g, c, sqrtf(r2), b0, b1);
  return visit_box<2>(g, b0, b1, [&](unsigned m, const Pt& pm) {
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

// The first point p (not in ex) that becomes as close to x0 + s w as i is.
template <int D>
TECS_DL_HD Hit shoot(const Grid& g, const double* x0, const double* w, const double* pi, const unsigned* ex,
                     int nex) {
  double pow0 = 0.0;
  for (int d = 0; d < D; ++d) { const double v = x0[d] - pi[d]; pow0 += v * v; }
  Hit best{~0u, kInf};
  int bc[3];
  bin_of<D>(g, x0, bc);
  const int kmax = shells_to_cover<D>(g, bc);
  for (int k = 0; k <= kmax; ++k) {
    visit_shell<D>(g, bc, k, [&](unsigned id, const Pt& p) {
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
      if (!(wp > 1.0e-9 * sqrt(nn))) return true;  // on or behind the plane through i
      const double s = (num - pow0) / (2.0 * wp);
      if (s < best.s || (s == best.s && id < best.id)) best = Hit{id, s};
      return true;
    });
    if (best.id != ~0u) {
      double r2 = 0.0;
      for (int d = 0; d < D; ++d) { const double v = x0[d] + best.s * w[d] - pi[d]; r2 += v * v; }
      if (((double)k - 1.0e-3) * g.h >= fabs(best.s) + sqrt(r2)) break;
    }
  }
  return best;
}

// i's nearest other cell at a non-zero distance (ties by index).
template <int D>
TECS_DL_HD unsigned nearest(const Grid& g, const double* pi, unsigned self) {
  double bd = kInf;
  unsigned bid = ~0u;
  int bc[3];
  bin_of<D>(g, pi, bc);
  const int kmax = shells_to_cover<D>(g, bc);
  for (int k = 0; k <= kmax; ++k) {
    visit_shell<D>(g, bc, k, [&](unsigned id, const Pt& p) {
      if (id == self) return true;
      double q[3];
      load(p, q);
      double d2 = 0.0;
      for (int d = 0; d < D; ++d) { const double v = q[d] - pi[d]; d2 += v * v; }
      if (d2 > 0.0 && (d2 < bd || (d2 == bd && id < bid))) { bd = d2; bid = id; }
      return true;
    });
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
  int nt = 0, ns = 0;
  unsigned err = 0;
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
  // centre error: the b terms (|p|^2 differences, absolute error ~ eps L^2)
  // times cofactors of size h^(D-1), over the determinant
  const double dc = 32.0 * kEps * (L * L + hm * hm) * hp / den + 8.0 * kEps * L;
  const double r = sqrt(R);
  return 16.0 * (2.0 * r * dc + dc * dc) + 64.0 * kEps * (R + L * r);
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
template <int D>
TECS_DL_HD int add_simplex(const Grid& g, Star& st, const double* pi, unsigned a, unsigned b, unsigned d3,
                           const double* c) {
  unsigned v[3] = {a, b, D == 3 ? d3 : ~0u};
  // ascending (three elements)
  for (int x = 0; x < 2; ++x)
    for (int y = 0; y < 2 - x; ++y)
      if (v[y] > v[y + 1]) { const unsigned t = v[y]; v[y] = v[y + 1]; v[y + 1] = t; }
  for (int q = 0; q < st.nt; ++q)
    if (st.t[q].v[0] == v[0] && st.t[q].v[1] == v[1] && st.t[q].v[2] == v[2]) return q;
  if (st.nt >= kMaxTet) { st.err |= kErrStar; return -1; }
  double R = 0.0;
  for (int d = 0; d < D; ++d) { const double u = c[d] - pi[d]; R += u * u; }
  double e[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  for (int q = 0; q < D; ++q) {
    double p[3];
    load(g.P[v[q]], p);
    for (int d = 0; d < D; ++d) e[q][d] = p[d] - pi[d];
  }
  const double tol = shell_tol<D>(pi, e, R);
  int sp = find_sphere<D>(st, c, R);
  if (sp < 0) {
    if (st.ns >= kMaxSph) { st.err |= kErrStar; return -1; }
    sp = st.ns++;
    for (int d = 0; d < 3; ++d) st.s[sp].c[d] = d < D ? c[d] : 0.0;
    st.s[sp].R = R;
    st.s[sp].tol = tol;
  } else if (tol > st.s[sp].tol) {
    st.s[sp].tol = tol;
  }
  const int q = st.nt++;
  st.t[q].v[0] = v[0]; st.t[q].v[1] = v[1]; st.t[q].v[2] = v[2];
  st.t[q].sph = sp;
  st.t[q].done = 0u;
  return q;
}

TECS_DL_HD void mark_face(Star& st, int q, unsigned opposite) {
  if (q < 0) return;
  for (int f = 0; f < 3; ++f)
    if (st.t[q].v[f] == opposite) st.t[q].done |= 1u << f;
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
TECS_DL_HD void star2(const Grid& g, unsigned i, Star& st) {
  double pi[3];
  load(g.P[i], pi);
  const unsigned a = nearest<2>(g, pi, i);
  if (a == ~0u) return;
  double pa[3];
  load(g.P[a], pa);
  const double x0[3] = {(pi[0] + pa[0]) * 0.5, (pi[1] + pa[1]) * 0.5, 0.0};
  double u[3] = {-(pa[1] - pi[1]), pa[0] - pi[0], 0.0};
  normalize3(u, 2);
  for (int side = 0; side < 2; ++side) {
    const double w[3] = {side ? -u[0] : u[0], side ? -u[1] : u[1], 0.0};
    const unsigned ex[2] = {i, a};
    const Hit h = shoot<2>(g, x0, w, pi, ex, 2);
    if (h.id == ~0u) continue;
    const double c[3] = {x0[0] + h.s * w[0], x0[1] + h.s * w[1], 0.0};
    const int nt0 = st.nt;
    int q = add_simplex<2>(g, st, pi, a, h.id, ~0u, c);
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
      const Hit h2 = shoot<2>(g, v, n, pi, ex2, 3);
      if (h2.id == ~0u) break;  // open: i is on the hull
      const double c2[3] = {v[0] + h2.s * n[0], v[1] + h2.s * n[1], 0.0};
      const int cur_sph = st.t[q].sph, ns0 = st.ns, nt1 = st.nt;
      const int q2 = add_simplex<2>(g, st, pi, cur, h2.id, ~0u, c2);
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
TECS_DL_HD void star3(const Grid& g, unsigned i, Star& st) {
  double pi[3];
  load(g.P[i], pi);
  const unsigned a = nearest<3>(g, pi, i);
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
  Hit h = shoot<3>(g, x0, u, pi, ex, 2);
  if (h.id == ~0u) {
    for (int d = 0; d < 3; ++d) u[d] = -u[d];
    h = shoot<3>(g, x0, u, pi, ex, 2);
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
    const Hit hd = shoot<3>(g, x1, w, pi, ex3, 3);
    if (hd.id == ~0u) continue;
    const double c[3] = {x1[0] + hd.s * w[0], x1[1] + hd.s * w[1], x1[2] + hd.s * w[2]};
    q0[side] = add_simplex<3>(g, st, pi, a, b, hd.id, c);
    apex[side] = hd.id;
  }
  // the face (i, a, b) between the two first tetrahedra is crossed
  mark_face(st, q0[0], apex[0]);
  mark_face(st, q0[1], apex[1]);
  for (int q = 0; q < st.nt; ++q) {
    for (int f = 0; f < 3; ++f) {
      if (st.t[q].done & (1u << f)) continue;
      st.t[q].done |= 1u << f;
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
      const Hit hf = shoot<3>(g, S.c, w, pi, exf, 4);
      if (hf.id == ~0u) continue;  // open face: i is on the hull
      const double c[3] = {S.c[0] + hf.s * w[0], S.c[1] + hf.s * w[1], S.c[2] + hf.s * w[2]};
      const int q2 = add_simplex<3>(g, st, pi, A, B, hf.id, c);
      if (q2 < 0) return;
      mark_face(st, q2, hf.id);
    }
  }
}

// ---------------------------------------------------------------------------
// One cell: its partners and how often the reference applies each pair.
// out[0..return) = (j, reps), ascending j; *err gets the error bits.

struct JK {
  unsigned j, k;
};

template <int D>
TECS_DL_HD unsigned cell_mult(const Grid& g, unsigned i, unsigned* out_j, unsigned* out_r, unsigned cap,
                              unsigned* err, Star& st) {
  st.nt = 0;
  st.ns = 0;
  st.err = 0;
  if (D == 2) star2(g, i, st);
  else star3(g, i, st);
  unsigned e = st.err;
  JK pairs[kMaxPairs];
  int np = 0;
  const Pt Pi = g.P[i];
  auto record = [&](unsigned j, unsigned k) {
    for (int p = 0; p < np; ++p)
      if (pairs[p].j == j && pairs[p].k == k) return;
    if (np >= kMaxPairs) { e |= kErrPairs; return; }
    pairs[np++] = JK{j, k};
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
    unsigned near[kMaxNear];
    double dev[kMaxNear];
    for (int q = 0; q < st.ns; ++q) {
      const Sph S = st.s[q];
      // the circle's own triangle points first (deviation -1: never dropped),
      // then every point on or near it, or inside; when the array is full
      // the point farthest from the circle gives way
      int nn = 0;
      auto put = [&](unsigned id, double f) {
        for (int x = 0; x < nn; ++x)
          if (near[x] == id) return;
        if (nn < kMaxNear) { near[nn] = id; dev[nn] = f; ++nn; return; }
        e |= kErrNear;
        int w = 0;
        for (int x = 1; x < nn; ++x)
          if (dev[x] > dev[w]) w = x;
        if (f < dev[w]) { near[w] = id; dev[w] = f; }
      };
      for (int t = 0; t < st.nt; ++t)
        if (st.t[t].sph == q) { put(st.t[t].v[0], -1.0); put(st.t[t].v[1], -1.0); }
      const double rad = sqrt(S.R + S.tol) * (1.0 + 1.0e-9) + 1.0e-200;
      int b0[3], b1[3];
      for (int d = 0; d < 3; ++d) {
        b0[d] = d < 2 ? bin1(g, d, S.c[d] - rad) : 0;
        b1[d] = d < 2 ? bin1(g, d, S.c[d] + rad) : 0;
      }
      visit_box<2>(g, b0, b1, [&](unsigned id, const Pt& p) {
        if (id == i) return true;
        const double u0 = (double)p.x - S.c[0], u1 = (double)p.y - S.c[1];
        const double f = u0 * u0 + u1 * u1 - S.R;
        if (f <= S.tol) put(id, fabs(f));
        return true;
      });
      // the reference's test on every choice of j (in cutoff) and k among them
      for (int a = 0; a < nn; ++a) {
        const unsigned j = near[a];
        if (!in_cutoff<2>(g, Pi, g.P[j])) continue;
        for (int b = 0; b < nn; ++b) {
          const unsigned k = near[b];
          if (k == j) continue;
          bool have = false;
          for (int p = 0; p < np && !have; ++p) have = pairs[p].j == j && pairs[p].k == k;
          if (!have && tri_pass(g, i, j, k)) record(j, k);
        }
      }
    }
  }
  // (j, number of distinct k), ascending j
  for (int x = 1; x < np; ++x) {
    const JK v = pairs[x];
    int y = x - 1;
    while (y >= 0 && (pairs[y].j > v.j || (pairs[y].j == v.j && pairs[y].k > v.k))) { pairs[y + 1] = pairs[y]; --y; }
    pairs[y + 1] = v;
  }
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
