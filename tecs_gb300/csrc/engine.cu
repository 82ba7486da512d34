// engine.cu -- many independent simulations advanced by one step graph.
//
// The batched and served forms share this engine.  Every resident simulation
// ("slot") owns a contiguous region of one global bin-key space
// (bin_base + its own flattened bin index) and a row in a device-resident
// parameter table (its grid, force constants, finder, integrator, polarity).
// One step is a fixed kernel sequence over the whole capacity:
//
//   k_ecount -> k_scan_reduce -> k_scan_apply -> k_escatter -> k_eorder_gather
//   -> k_epass<1> -> k_epass<2>
//
// Cells of slots marked inactive get no bin and drop out at the sort, so the
// sorted copy is always compact; cells of a newly admitted slot are appended
// after the resident ones and merged in by the next sort.  The step reads the
// resident count and the table from device memory, so the captured graph
// stays valid while simulations come and go.  The per-cell arithmetic is the
// single-simulation path's (same device functions, same summation order), so
// every simulation's trajectory equals a plain run of it.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "../../include/tecs_gpu.h"
#include "../../include/tecs/device/kernels.cuh"

namespace tecs {
int set_last_error(const std::string& m);
}

using namespace tecs;

namespace {

int fail(const std::string& m) { return set_last_error(m); }
#define ECK(call)                                                                             \
  do {                                                                                        \
    cudaError_t e_ = (call);                                                                  \
    if (e_ != cudaSuccess) return fail(std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

unsigned cdiv(unsigned long long a, unsigned b) { return (unsigned)((a + b - 1) / b); }

constexpr unsigned kInvalidKey = 0xffffffffu;

// One simulation's row of the device parameter table.
struct SimSlot {
  GridP g;
  ForceP fp;
  unsigned bin_base;
  int finder;       // TECS_FINDER_BINNED_ALL_PAIRS | TECS_FINDER_BINNED_GABRIEL
  int integrator;   // TECS_EULER | TECS_HEUN
  int has_pol;
  int active;
  int gabriel_fast;
  int pad[2];
};

struct EngArgs {
  const SimSlot* table;
  const unsigned* off;    // global bin offsets; off[nb_total] = cells in the sorted copy
  unsigned nb_total;
  const float4* X;        // B (pass 1) or Xt (pass 2)
  const float2* P;        // PB or Pt
  const float4* Bx;       // x_n, sorted (w = bin key)
  const float2* Bp;
  const unsigned* Bid;    // cell ids of the sorted slots
  const unsigned* Bsim;   // slot of each sorted cell
  float4* d1;
  float2* dp1;
  float4* Xt;
  float2* Pt;
  float4* A;              // next state (w = id)
  float2* PA;
  unsigned* Asim;
  float dt;
};

// ---------------------------------------------------------------------------
// binning over all slots

static __global__ void k_ecount(const float4* __restrict__ A, const unsigned* __restrict__ Asim,
                                const Counters* __restrict__ ctr, const SimSlot* __restrict__ table,
                                unsigned* __restrict__ key, unsigned* __restrict__ rank, unsigned* __restrict__ cnt) {
  const unsigned n = ctr->n;
  for (unsigned s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
    const SimSlot& sl = table[Asim[s]];
    if (!sl.active) {
      key[s] = kInvalidKey;
      continue;
    }
    const float4 v = A[s];
    const float p[3] = {v.x, v.y, v.z};
    int c[3] = {0, 0, 0};
    bin_coords_div<3>(sl.g, p, c);
    const unsigned b = sl.bin_base + flatten<3>(sl.g, c);
    key[s] = b;
    rank[s] = atomicAdd(&cnt[b], 1u);
  }
}

static __global__ void k_escatter(const Counters* __restrict__ ctr, const unsigned* __restrict__ key,
                                  const unsigned* __restrict__ rank, const unsigned* __restrict__ off,
                                  unsigned* __restrict__ src) {
  const unsigned n = ctr->n;
  for (unsigned s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
    const unsigned b = key[s];
    if (b != kInvalidKey) src[off[b] + rank[s]] = s;
  }
}

// as k_order_gather, over the compacted count off[nb_total], carrying the slot index
static __global__ void k_eorder_gather(const unsigned* __restrict__ off, unsigned nb_total,
                                       const unsigned* __restrict__ key, const unsigned* __restrict__ src,
                                       const float4* __restrict__ A, const float2* __restrict__ PA,
                                       const unsigned* __restrict__ Asim, float4* __restrict__ B,
                                       float2* __restrict__ PB, unsigned* __restrict__ Bid,
                                       unsigned* __restrict__ Bsim) {
  const unsigned n = off[nb_total];
  for (unsigned t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const unsigned s = src[t];
    const unsigned b = key[s];
    const unsigned lo = off[b], hi = off[b + 1];
    const float4 v = A[s];
    unsigned dst = t;
    if (hi - lo > 1u) {
      const unsigned me = id_of(v);
      unsigned r = 0;
      for (unsigned k = lo; k < hi; ++k) r += id_of(A[src[k]]) < me ? 1u : 0u;
      dst = lo + r;
    }
    B[dst] = make_float4(v.x, v.y, v.z, __uint_as_float(b));
    Bid[dst] = id_of(v);
    Bsim[dst] = Asim[s];
    PB[dst] = PA[s];
  }
}

// ---------------------------------------------------------------------------
// the force pass over all slots: k_pass_gabriel's per-warp phases with each
// cell's simulation parameters taken from the table

// POL: some resident simulation carries polarity; their cells then take the
// cooperative path with the polarity law, its pair terms added in the ordered
// sums -- spring-only engines use the instance without that branch.
// TB: threads per block (64, 96 or 128; the autotuner's choice).
template <int TB>
__device__ __forceinline__ int ecix(int q, int c) { return q * TB + (c ^ q); }

template <int PASS, bool POL, int TB>
static __global__ void __launch_bounds__(TB) k_epass(EngArgs e) {
  constexpr int NB = kMaxNb;  // neighbour slots per cell (more: the per-thread path)
  __shared__ float4 cand[NB * TB];
  __shared__ float4 home[TB];
  __shared__ unsigned short pinfo[NB * TB];
  __shared__ unsigned short wcls[TB / 32][NB + 1];  // pairs per (warp, neighbour count)
  __shared__ unsigned amask[TB];
  __shared__ unsigned char ncnt[TB];
  __shared__ unsigned hsim[TB];
  const unsigned n = e.off[e.nb_total];
  const int t = threadIdx.x;
  const unsigned i = blockIdx.x * TB + t;
  const bool active = i < n;
  const unsigned sim = active ? e.Bsim[i] : 0u;
  const SimSlot& sl = e.table[sim];
  // Euler simulations take one pass; their second-pass cells sit out
  const bool run = active && (PASS == 1 || sl.integrator == TECS_HEUN);
  const bool polar = run && sl.has_pol;
  const bool gab = sl.finder == TECS_FINDER_BINNED_GABRIEL;
  float xi[3] = {0.f, 0.f, 0.f};
  float4 vi = make_float4(0.f, 0.f, 0.f, 0.f);
  float2 pi = make_float2(0.f, 0.f);
  int bc[3] = {0, 0, 0};
  int cnt = 0;
  bool fb = (polar && !POL) || (run && gab && !sl.gabriel_fast);
  if (run) {
    vi = __ldg(&e.X[i]);
    xi[0] = vi.x; xi[1] = vi.y; xi[2] = vi.z;
    if (sl.has_pol) pi = e.P[i];
    // i's own bin: division for the Gabriel finder (grid.hpp:222-230),
    // multiplication for BinnedAllPairs (binned_all_pairs.hpp:103-109)
    if (gab) bin_coords_div<3>(sl.g, xi, bc);
    else bin_coords_mul<3>(sl.g, xi, bc);
  }
  if (run && !fb) {
    const GridP& g = sl.g;
    const int x0 = max(bc[0] - 1, 0), x1 = min(bc[0] + 1, g.ext[0] - 1);
    unsigned rlo[9], rhi[9], rb0[9];
#pragma unroll
    for (int r = 0; r < 9; ++r) {
      const int cy = bc[1] + r % 3 - 1, cz = bc[2] + r / 3 - 1;
      const bool ok = cy >= 0 && cy < g.ext[1] && cz >= 0 && cz < g.ext[2];
      int c0[3] = {x0, ok ? cy : 0, ok ? cz : 0};
      const unsigned b0 = sl.bin_base + flatten<3>(g, c0);
      rb0[r] = b0;
      rlo[r] = ok ? __ldg(&e.off[b0]) : 0u;
      rhi[r] = ok ? __ldg(&e.off[b0 + (unsigned)(x1 - x0) + 1u]) : 0u;
    }
    const int rxo = x0 - bc[0] + 1;
    const float rc2 = sl.fp.rc2;
    // as k_pass_gabriel: the three rows of each z-plane scanned together, two
    // candidates at a time, in-cutoff ones appended in candidate order
#pragma unroll
    for (int g0 = 0; g0 < 9; g0 += 3) {
      unsigned len[3];
      unsigned lmax = 0u;
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        len[q] = rhi[g0 + q] - rlo[g0 + q];
        lmax = max(lmax, len[q]);
      }
      if (lmax > 32u) fb = true;
      if (fb) continue;
      unsigned m[3] = {0u, 0u, 0u};
      for (unsigned o = 0; o < lmax; o += 2u) {
        float4 v[3][2];
#pragma unroll
        for (int q = 0; q < 3; ++q)
#pragma unroll
          for (int k = 0; k < 2; ++k)
            v[q][k] = __ldg(&e.X[len[q] ? rlo[g0 + q] + min(o + k, len[q] - 1u) : i]);
#pragma unroll
        for (int q = 0; q < 3; ++q)
#pragma unroll
          for (int k = 0; k < 2; ++k) {
            const unsigned j = rlo[g0 + q] + o + k;
            const float e0 = xi[0] - v[q][k].x, e1 = xi[1] - v[q][k].y, e2 = xi[2] - v[q][k].z;
            float d2 = e0 * e0 + e1 * e1;
            d2 = d2 + e2 * e2;
            if (o + k < len[q] && j != i && d2 < rc2) m[q] |= 1u << (o + k);
          }
      }
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        const int r = g0 + q;
        const unsigned rowcode = 3u * (unsigned)(r % 3) + 9u * (unsigned)(r / 3);
        unsigned mm = m[q];
        if (cnt + __popc(mm) > NB) { fb = true; break; }
        while (mm) {
          const unsigned j = rlo[r] + (unsigned)(__ffs(mm) - 1);
          mm &= mm - 1u;
          const float4 v = __ldg(&e.X[j]);
          const unsigned rx = (unsigned)((int)(__float_as_uint(v.w) - rb0[r]) + rxo);
          cand[ecix<TB>(cnt, t)] = make_float4(v.x, v.y, v.z, __uint_as_float((j << 5) | (rowcode + rx)));
          ++cnt;
        }
      }
    }
  }
  if (fb) cnt = 0;
  home[t] = make_float4(xi[0], xi[1], xi[2],
                        __uint_as_float((unsigned)bc[0] | ((unsigned)bc[1] << 10) | ((unsigned)bc[2] << 20)));
  hsim[t] = sim;
  ncnt[t] = (unsigned char)cnt;
  // Phases 2-4 run per warp over the warp's own 32 cells, as in
  // k_pass_gabriel.  Only cells of Gabriel slots with two or more neighbours
  // need the Gabriel test (a single neighbour has no witness; all-pairs
  // slots accept every in-cutoff pair); their pairs are listed sorted by the
  // cell's neighbour count, so that the witness loops of a round run the
  // same length.
  const int lane = t & 31, warp = t >> 5;
  unsigned short* const wp = pinfo + warp * 32 * NB;
  const bool tested = run && !fb && gab && cnt >= 2;
  const int tcnt = tested ? cnt : 0;
  int P = 0;
  {
    if (lane <= NB) wcls[warp][lane] = 0;
    __syncwarp();
    const unsigned same = __match_any_sync(0xffffffffu, tcnt);
    const int rank = __popc(same & ((1u << lane) - 1u));
    if (rank == 0) wcls[warp][tcnt] = (unsigned short)(__popc(same) * (unsigned)tcnt);
    amask[t] = tested ? 0u : (1u << cnt) - 1u;  // cnt <= 16; 0 for fallback and idle cells
    __syncwarp();
    const unsigned tot = lane <= NB ? (unsigned)wcls[warp][lane] : 0u;
    unsigned incl = tot;
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    P = (int)__shfl_sync(0xffffffffu, incl, NB);
    const int base = (int)__shfl_sync(0xffffffffu, incl - tot, tcnt) + rank * tcnt;
    for (int q = 0; q < tcnt; ++q) wp[base + q] = (unsigned short)((t << 4) | q);
  }
  __syncwarp();

  // ---- Gabriel test, one pair per lane at a time, two witnesses per round
  for (int p = lane; p < P; p += 32) {
    const unsigned info = wp[p];
    const int c = (int)(info >> 4), q = (int)(info & 15u);
    const SimSlot& cs = e.table[hsim[c]];
    const float4 h = home[c];
    const float4 vj = cand[ecix<TB>(q, c)];
    const float hx[3] = {h.x, h.y, h.z};
    const float disp[3] = {hx[0] - vj.x, hx[1] - vj.y, hx[2] - vj.z};
    float d2 = disp[0] * disp[0] + disp[1] * disp[1];
    d2 = d2 + disp[2] * disp[2];
    float m[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) m[d] = hx[d] - disp[d] * 0.5f;
    const float rsq = d2 * cs.fp.gab_factor;
    const int cc = ncnt[c];
    unsigned hits = 0u, bit = 1u;
    for (int w = 0; w < cc; w += 2) {
      const int w1 = min(w + 1, cc - 1);
      const float4 vk0 = cand[ecix<TB>(w, c)], vk1 = cand[ecix<TB>(w1, c)];
      const float f0 = vk0.x - m[0], f1 = vk0.y - m[1], f2 = vk0.z - m[2];
      const float g0 = vk1.x - m[0], g1 = vk1.y - m[1], g2 = vk1.z - m[2];
      float sd0 = f0 * f0 + f1 * f1, sd1 = g0 * g0 + g1 * g1;
      sd0 = sd0 + f2 * f2;
      sd1 = sd1 + g2 * g2;
      if (sd0 < rsq) hits |= bit;
      if (sd1 < rsq) hits |= bit << 1;
      bit <<= 2;
    }
    hits &= ((1u << cc) - 1u) & ~(1u << q);
    bool blocked = false;
    if (hits) {
      // a witness in the ball blocks only from a bin overlapping the ball
      // (binned_gabriel.hpp:142-153), relative to the cell's bin
      const unsigned hb = __float_as_uint(h.w);
      const int hbc[3] = {(int)(hb & 1023u), (int)((hb >> 10) & 1023u), (int)(hb >> 20)};
      const float r = sqrtf(rsq);
      int lo[3], hi[3];
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        lo[d] = clampi((int)floorf((m[d] - r - cs.g.mn[d]) * cs.g.inv_bin), cs.g.ext[d] - 1) - hbc[d];
        hi[d] = clampi((int)floorf((m[d] + r - cs.g.mn[d]) * cs.g.inv_bin), cs.g.ext[d] - 1) - hbc[d];
      }
      while (hits && !blocked) {
        const int w = __ffs(hits) - 1;
        hits &= hits - 1u;
        const unsigned code = __float_as_uint(cand[ecix<TB>(w, c)].w) & 31u;
        const int rel[3] = {(int)(code % 3u) - 1, (int)((code / 3u) % 3u) - 1, (int)(code / 9u) - 1};
        bool inside = true;
#pragma unroll
        for (int d = 0; d < 3; ++d) inside = inside && rel[d] >= lo[d] && rel[d] <= hi[d];
        blocked = inside;
      }
    }
    if (!blocked) atomicOr(&amask[c], 1u << q);
  }
  __syncwarp();
  // the warp's accepted spring pairs, cell by cell, over the pair list (the
  // polarity law's pairs are summed term by term in the ordered sums)
  int PA = 0;
  {
    const bool pol_cell = POL && polar && sl.fp.force == TECS_FORCE_POLARITY;
    const unsigned acc_bits = (fb || pol_cell || !run) ? 0u : amask[t];
    const int na = __popc(acc_bits);
    int incl = na;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    PA = __shfl_sync(0xffffffffu, incl, 31);
    int base = incl - na;
    __syncwarp();
    for (unsigned b = acc_bits; b; b &= b - 1u) wp[base++] = (unsigned short)((t << 4) | (__ffs(b) - 1));
  }
  __syncwarp();
  // ---- spring2r forces of the accepted pairs, written over the candidate slot
  for (int p = lane; p < PA; p += 32) {
    const unsigned info = wp[p];
    const int c = (int)((info >> 4) & 127u), q = (int)(info & 15u);
    const SimSlot& cs = e.table[hsim[c]];
    const float4 h = home[c];
    const float4 vj = cand[ecix<TB>(q, c)];
    const float disp[3] = {h.x - vj.x, h.y - vj.y, h.z - vj.z};
    float d2 = disp[0] * disp[0] + disp[1] * disp[1];
    d2 = d2 + disp[2] * disp[2];
    float4 f = make_float4(0.f, 0.f, 0.f, 0.f);
    const float dist = sqrtf(d2);
    if (cs.fp.force != TECS_FORCE_NONE && dist != 0.0f) {
      // (displacement * F) / distance; a zero F leaves the sum unchanged
      const ForceP& fp = cs.fp;
      const float F = fp.k_rep * fmaxf(fp.r_rep - dist, 0.0f) - fp.k_adh * fmaxf(dist - fp.r_adh, 0.0f);
      if (F != 0.0f) {
        f.x = (disp[0] * F) / dist;
        f.y = (disp[1] * F) / dist;
        f.z = (disp[2] * F) / dist;
      }
    }
    cand[ecix<TB>(q, c)] = f;
  }
  __syncwarp();
  // ---- ordered per-cell sums
  Acc acc = {{0.f, 0.f, 0.f}, {0.f, 0.f}};
  if (run && !fb) {
    const bool pol_law = POL && polar && sl.fp.force == TECS_FORCE_POLARITY;
    for (int q = 0; q < cnt; ++q) {
      if (!((amask[t] >> q) & 1u)) continue;
      const float4 f = cand[ecix<TB>(q, t)];
      if (pol_law) {
        // this pair's spring, bending vector, bending and alignment terms, each
        // added to the sums in turn (polarity.hpp:131-198 as pair_force adds them)
        const float disp[3] = {xi[0] - f.x, xi[1] - f.y, xi[2] - f.z};
        float d2 = disp[0] * disp[0] + disp[1] * disp[1];
        d2 = d2 + disp[2] * disp[2];
        const float2 pj = __ldg(&e.P[__float_as_uint(f.w) >> 5]);
        pair_force<3, 2>(sl.fp, disp, sqrtf(d2), pi, pj, acc);
        continue;
      }
      acc.x[0] = acc.x[0] + f.x;
      acc.x[1] = acc.x[1] + f.y;
      acc.x[2] = acc.x[2] + f.z;
    }
  }
  // the warp's sums are read: its candidate columns serve the per-thread
  // neighbour lists of the overflow path
  __syncwarp();
  if (!run) return;
  if (fb) {
    PassArgs pa{};
    pa.X = e.X;
    pa.P = sl.has_pol ? e.P : nullptr;
    pa.off = e.off + sl.bin_base;  // the slot's own bins, indexed by its local flat index
    pa.Bid = nullptr;
    const unsigned idi = __ldg(&e.Bid[i]);
    const int force = sl.fp.force;
    if (gab) {
      if (force == TECS_FORCE_POLARITY) {
        if (!(sl.gabriel_fast && gabriel_cell_fast<3, 2, NB, TB>(sl.g, sl.fp, pa, i, xi, pi, idi, acc, &cand[t])))
          cell_general<3, 3, 2>(sl.g, sl.fp, pa, n, i, xi, pi, idi, acc);
      } else if (force == TECS_FORCE_SPRING2R) {
        cell_general<3, 3, 1>(sl.g, sl.fp, pa, n, i, xi, pi, idi, acc);
      } else {
        cell_general<3, 3, 0>(sl.g, sl.fp, pa, n, i, xi, pi, idi, acc);
      }
    } else {
      if (force == TECS_FORCE_POLARITY) cell_general<3, 1, 2>(sl.g, sl.fp, pa, n, i, xi, pi, idi, acc);
      else if (force == TECS_FORCE_SPRING2R) cell_general<3, 1, 1>(sl.g, sl.fp, pa, n, i, xi, pi, idi, acc);
      else cell_general<3, 1, 0>(sl.g, sl.fp, pa, n, i, xi, pi, idi, acc);
    }
  }
  // integrator epilogues (euler.hpp:49-69, heun.hpp:54-98; no COM fix)
  float s3[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) s3[d] = 0.0f + acc.x[d];
  const float sp0 = 0.0f + acc.p[0], sp1 = 0.0f + acc.p[1];
  const float dt = e.dt;
  if (PASS == 1 && sl.integrator == TECS_HEUN) {
    e.d1[i] = make_float4(s3[0], s3[1], s3[2], 0.f);
    e.Xt[i] = make_float4(xi[0] + s3[0] * dt, xi[1] + s3[1] * dt, xi[2] + s3[2] * dt, vi.w);
    if (sl.has_pol) {
      e.dp1[i] = make_float2(sp0, sp1);
      e.Pt[i] = make_float2(pi.x + sp0 * dt, pi.y + sp1 * dt);
    }
    return;
  }
  const float4 xb = e.Bx[i];
  float xn[3];
  float2 pn = make_float2(0.f, 0.f);
  if (PASS == 1) {
    xn[0] = xb.x + s3[0] * dt; xn[1] = xb.y + s3[1] * dt; xn[2] = xb.z + s3[2] * dt;
    if (sl.has_pol) { const float2 pb = e.Bp[i]; pn = make_float2(pb.x + sp0 * dt, pb.y + sp1 * dt); }
  } else {
    const float4 q1 = e.d1[i];
    const float h0 = q1.x + s3[0], h1 = q1.y + s3[1], h2 = q1.z + s3[2];
    xn[0] = xb.x + (h0 * 0.5f) * dt; xn[1] = xb.y + (h1 * 0.5f) * dt; xn[2] = xb.z + (h2 * 0.5f) * dt;
    if (sl.has_pol) {
      const float2 pb = e.Bp[i], r1 = e.dp1[i];
      const float g0 = r1.x + sp0, g1 = r1.y + sp1;
      pn = make_float2(pb.x + (g0 * 0.5f) * dt, pb.y + (g1 * 0.5f) * dt);
    }
  }
  e.A[i] = make_float4(xn[0], xn[1], xn[2], __uint_as_float(e.Bid[i]));
  e.PA[i] = pn;
  e.Asim[i] = sim;
}

// Euler cells keep their pass-1 state: nothing to do in pass 2 (handled by `run`).

// pack a host-uploaded AoS simulation into A at offset `at`
static __global__ void k_epack(const float* __restrict__ in, unsigned n, unsigned at, unsigned slot,
                               float4* __restrict__ A, unsigned* __restrict__ Asim) {
  for (unsigned s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
    A[at + s] = make_float4(in[3 * (size_t)s], in[3 * (size_t)s + 1], in[3 * (size_t)s + 2], __uint_as_float(s));
    Asim[at + s] = slot;
  }
}

// unpack one slot's cells (a range of A) into id order
static __global__ void k_eunpack(const unsigned* __restrict__ range, unsigned n, const float4* __restrict__ A,
                                 const float2* __restrict__ PA, float* __restrict__ pos, float2* __restrict__ pol) {
  const unsigned lo = range[0];
  for (unsigned s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
    const float4 v = A[lo + s];
    const unsigned id = id_of(v);
    pos[3 * (size_t)id] = v.x;
    pos[3 * (size_t)id + 1] = v.y;
    pos[3 * (size_t)id + 2] = v.z;
    if (pol) pol[id] = PA[lo + s];
  }
}

// the start of a slot's range in A after the last step: off[bin_base]; or its append point
static __global__ void k_erange(const unsigned* __restrict__ off, unsigned bin_base, unsigned appended_at,
                                int sorted, unsigned* __restrict__ range) {
  range[0] = sorted ? off[bin_base] : appended_at;
}

}  // namespace

struct tecs_engine {
  tecs_engine_desc d{};
  cudaStream_t stream = nullptr, side = nullptr;
  unsigned C = 0, NB = 0, S = 0;
  float4 *A = nullptr, *B = nullptr, *Xt = nullptr, *d1 = nullptr;
  float2 *PA = nullptr, *PB = nullptr, *Pt = nullptr, *dp1 = nullptr;
  unsigned *Asim = nullptr, *Bsim = nullptr, *Bid = nullptr, *key = nullptr, *rank = nullptr, *src = nullptr;
  unsigned *cnt = nullptr, *off = nullptr, *part = nullptr, *range = nullptr;
  Counters* ctr = nullptr;
  SimSlot* table = nullptr;    // device
  SimSlot* htable = nullptr;   // pinned host mirror
  Counters* hctr = nullptr;    // pinned host mirror of the counters' n
  float* stage = nullptr;      // device staging for downloads (C*3 floats)
  float2* stagep = nullptr;
  // host bookkeeping
  struct Info {
    bool used = false, active = false, sorted = false;
    unsigned n = 0, nbins = 0, bin_base = 0, appended_at = 0;
    unsigned long long steps = 0;
  };
  std::vector<Info> info;
  std::map<unsigned, unsigned> free_bins;  // start -> length
  unsigned n_resident = 0;
  bool table_dirty = true, n_dirty = true;
  std::vector<int> pending_free;
  cudaGraphExec_t graph = nullptr;
  float gdt = 0.f;
  unsigned gC = 0, gNB = 0;  // the extents the captured graph covers (cells, bins)
  bool gpol = false;         // the captured graph runs the polarity-capable pass
  int kernels = 7;
  unsigned pass_threads = 96;  // threads per block of the force passes (64, 96 or 128)
  unsigned gTB = 0;            // ... in the captured graph
};

namespace {

int bins_alloc(tecs_engine* e, unsigned nb, unsigned* base) {
  for (auto it = e->free_bins.begin(); it != e->free_bins.end(); ++it) {
    if (it->second >= nb) {
      *base = it->first;
      const unsigned rest = it->second - nb, start = it->first + nb;
      e->free_bins.erase(it);
      if (rest) e->free_bins[start] = rest;
      return 0;
    }
  }
  return -1;
}

void bins_free(tecs_engine* e, unsigned base, unsigned nb) {
  auto it = e->free_bins.emplace(base, nb).first;
  auto nx = std::next(it);
  if (nx != e->free_bins.end() && it->first + it->second == nx->first) {
    it->second += nx->second;
    e->free_bins.erase(nx);
  }
  if (it != e->free_bins.begin()) {
    auto pv = std::prev(it);
    if (pv->first + pv->second == it->first) {
      pv->second += it->second;
      e->free_bins.erase(it);
    }
  }
}

// The step's grids cover a power-of-two class of the resident cells and of the
// highest allocated bin, not the whole capacity: a server sized for hundreds of
// millions of cells then pays per step only for what it holds.  The graph is
// captured again when a class changes.
unsigned extent_class(unsigned long long v, unsigned cap) {
  unsigned long long p = 4096;
  while (p < v && p < cap) p <<= 1;
  return (unsigned)std::min<unsigned long long>(p, cap);
}

int enqueue_engine_step(tecs_engine* e, float dt) {
  const unsigned gb = cdiv(e->gC, 256);
  const unsigned len = e->gNB + 1;
  const unsigned chunks = cdiv(len, kScanChunk);
  k_ecount<<<gb, 256, 0, e->stream>>>(e->A, e->Asim, e->ctr, e->table, e->key, e->rank, e->cnt);
  if (chunks > 1) {  // one chunk: its prefix needs no partial sums
    ECK(cudaMemsetAsync(e->part + chunks, 0, (scan_part_words(len) - chunks) * 4, e->stream));
    k_scan_reduce<<<chunks, kScanThreads, 0, e->stream>>>(e->cnt, len, e->part);
  }
  e->kernels = chunks > 1 ? 7 : 6;
  k_scan_apply<<<chunks, kScanThreads, 0, e->stream>>>(e->cnt, len, e->part, e->off);
  k_escatter<<<gb, 256, 0, e->stream>>>(e->ctr, e->key, e->rank, e->off, e->src);
  k_eorder_gather<<<gb, 256, 0, e->stream>>>(e->off, e->gNB, e->key, e->src, e->A, e->PA, e->Asim, e->B, e->PB,
                                             e->Bid, e->Bsim);
  EngArgs a{};
  a.table = e->table;
  a.off = e->off;
  a.nb_total = e->gNB;
  a.Bx = e->B;
  a.Bp = e->PB;
  a.Bid = e->Bid;
  a.Bsim = e->Bsim;
  a.d1 = e->d1;
  a.dp1 = e->dp1;
  a.Xt = e->Xt;
  a.Pt = e->Pt;
  a.A = e->A;
  a.PA = e->PA;
  a.Asim = e->Asim;
  a.dt = dt;
  EngArgs a1 = a;
  a1.X = e->B;
  a1.P = e->PB;
  EngArgs a2 = a;
  a2.X = e->Xt;
  a2.P = e->Pt;
  const unsigned TB = e->pass_threads;
  const unsigned blocks = cdiv(e->gC, TB);
#define EPASS(T)                                                    \
  if (TB == T) {                                                    \
    if (e->gpol) {                                                  \
      k_epass<1, true, T><<<blocks, T, 0, e->stream>>>(a1);         \
      k_epass<2, true, T><<<blocks, T, 0, e->stream>>>(a2);         \
    } else {                                                        \
      k_epass<1, false, T><<<blocks, T, 0, e->stream>>>(a1);        \
      k_epass<2, false, T><<<blocks, T, 0, e->stream>>>(a2);        \
    }                                                               \
  }
  EPASS(64) EPASS(96) EPASS(128)
#undef EPASS
  ECK(cudaGetLastError());
  return 0;
}

}  // namespace

extern "C" {

int tecs_engine_desc_default(tecs_engine_desc* d) {
  if (!d) return fail("null desc");
  std::memset(d, 0, sizeof *d);
  d->cell_capacity = 1u << 22;
  d->bin_capacity = 1u << 23;
  d->max_sims = 1024;
  d->device = 0;
  return 0;
}

int tecs_engine_create(const tecs_engine_desc* desc, tecs_engine** out) {
  if (!desc || !out) return fail("null argument");
  *out = nullptr;
  if (!desc->cell_capacity || !desc->bin_capacity || !desc->max_sims) return fail("capacities must be > 0");
  if (desc->bin_capacity >= kInvalidKey) return fail("bin capacity too large");
  ECK(cudaSetDevice(desc->device));
  tecs_engine* e = new tecs_engine();
  e->d = *desc;
  e->C = desc->cell_capacity;
  e->NB = desc->bin_capacity;
  e->S = desc->max_sims;
  e->info.resize(e->S);
  e->free_bins[0] = e->NB;
  const size_t C = e->C;
  auto al = [&](void** p, size_t b) { return cudaMalloc(p, b ? b : 16) == cudaSuccess; };
  bool ok = cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking) == cudaSuccess &&
            cudaStreamCreateWithFlags(&e->side, cudaStreamNonBlocking) == cudaSuccess;
  ok = ok && al((void**)&e->A, C * 16) && al((void**)&e->B, C * 16) && al((void**)&e->Xt, C * 16) &&
       al((void**)&e->d1, C * 16) && al((void**)&e->PA, C * 8) && al((void**)&e->PB, C * 8) &&
       al((void**)&e->Pt, C * 8) && al((void**)&e->dp1, C * 8) && al((void**)&e->Asim, C * 4) &&
       al((void**)&e->Bsim, C * 4) && al((void**)&e->Bid, C * 4) && al((void**)&e->key, C * 4) &&
       al((void**)&e->rank, C * 4) && al((void**)&e->src, C * 4) &&
       al((void**)&e->cnt, ((size_t)e->NB + 1) * 4) && al((void**)&e->off, ((size_t)e->NB + 1) * 4) &&
       al((void**)&e->part, scan_part_words((size_t)e->NB + 1) * 4) && al((void**)&e->range, 64) &&
       al((void**)&e->ctr, sizeof(Counters)) && al((void**)&e->table, sizeof(SimSlot) * e->S) &&
       al((void**)&e->stage, C * 12) && al((void**)&e->stagep, C * 8);
  ok = ok && cudaMallocHost((void**)&e->htable, sizeof(SimSlot) * e->S) == cudaSuccess &&
       cudaMallocHost((void**)&e->hctr, sizeof(Counters)) == cudaSuccess;
  if (ok) {
    std::memset(e->htable, 0, sizeof(SimSlot) * e->S);
    std::memset(e->hctr, 0, sizeof(Counters));
    // cleared on the engine's own stream: it is non-blocking, so its kernels
    // are not ordered after work on the legacy default stream, which a plain
    // cudaMemset would use (and a buffer reused from a freed engine would
    // then be read before it is cleared)
    cudaStream_t st = e->stream;
    ok = cudaMemsetAsync(e->cnt, 0, ((size_t)e->NB + 1) * 4, st) == cudaSuccess &&
         cudaMemsetAsync(e->off, 0, ((size_t)e->NB + 1) * 4, st) == cudaSuccess &&
         cudaMemsetAsync(e->ctr, 0, sizeof(Counters), st) == cudaSuccess &&
         cudaMemsetAsync(e->table, 0, sizeof(SimSlot) * e->S, st) == cudaSuccess &&
         cudaMemsetAsync(e->PA, 0, C * 8, st) == cudaSuccess && cudaMemsetAsync(e->PB, 0, C * 8, st) == cudaSuccess &&
         cudaStreamSynchronize(st) == cudaSuccess;
  }
  if (!ok) {
    std::string m = std::string("engine allocation failed: ") + cudaGetErrorString(cudaGetLastError());
    tecs_engine_destroy(e);
    return fail(m);
  }
  *out = e;
  return 0;
}

int tecs_engine_destroy(tecs_engine* e) {
  if (!e) return 0;
  cudaSetDevice(e->d.device);
  if (e->stream) cudaStreamSynchronize(e->stream);
  if (e->side) cudaStreamSynchronize(e->side);
  if (e->graph) cudaGraphExecDestroy(e->graph);
  void* ptrs[] = {e->A, e->B, e->Xt, e->d1, e->PA, e->PB, e->Pt, e->dp1, e->Asim, e->Bsim, e->Bid, e->key,
                  e->rank, e->src, e->cnt, e->off, e->part, e->range, e->ctr, e->table, e->stage, e->stagep};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (e->htable) cudaFreeHost(e->htable);
  if (e->hctr) cudaFreeHost(e->hctr);
  if (e->stream) cudaStreamDestroy(e->stream);
  if (e->side) cudaStreamDestroy(e->side);
  delete e;
  return 0;
}

int tecs_engine_set_pass_threads(tecs_engine* e, unsigned threads) {
  if (!e) return fail("null engine");
  if (threads != 64 && threads != 96 && threads != 128) return fail("pass threads must be 64, 96 or 128");
  e->pass_threads = threads;  // the next step captures its graph again
  return 0;
}

int tecs_engine_free(tecs_engine* e, unsigned* free_cells, unsigned* largest_free_bins) {
  if (!e) return fail("null engine");
  if (free_cells) *free_cells = e->C - e->n_resident;
  unsigned best = 0;
  for (auto& kv : e->free_bins) best = std::max(best, kv.second);
  if (largest_free_bins) *largest_free_bins = best;
  return 0;
}

int tecs_engine_bins_needed(const tecs_sim_desc* d, unsigned* nbins) {
  if (!d || !nbins) return fail("null argument");
  const float bs = d->bin_size_scale * d->cutoff;
  unsigned long long nb = 1;
  for (int k = 0; k < 3; ++k) {
    const int ext = (int)std::ceil((d->max_bounds[k] - d->min_bounds[k]) / bs);
    if (ext < 1) return fail("max_bounds must exceed min_bounds");
    nb *= (unsigned long long)ext;
  }
  if (nb > 0xffffffffull) return fail("bin grid too large");
  *nbins = (unsigned)nb;
  return 0;
}

int tecs_engine_add(tecs_engine* e, const tecs_sim_desc* d, const float* positions, const float* polarity,
                    unsigned n, int* slot_out) {
  if (!e || !d || !slot_out || (n && !positions)) return fail("null argument");
  ECK(cudaSetDevice(e->d.device));
  ECK(cudaStreamSynchronize(e->stream));  // the table mirror and staging buffer are in use by queued work
  if (d->dims != 3) return fail("the engine runs 3-D simulations");
  if (d->finder != TECS_FINDER_BINNED_ALL_PAIRS && d->finder != TECS_FINDER_BINNED_GABRIEL)
    return fail("the engine runs the binned finders");
  if (d->symmetric || d->com_fix || d->division_probability > 0.0)
    return fail("the engine runs non-symmetric finders without COM fix or division");
  if (d->force == TECS_FORCE_POLARITY && !d->has_polarity) return fail("the polarity force needs a polarity field");
  if (d->has_polarity && n && !polarity) return fail("polarity required");
  if (!(d->cutoff > 0.f) || !(d->bin_size_scale > 0.f)) return fail("cutoff and bin_size_scale must be > 0");
  if (e->n_resident + n > e->C) return fail("engine cell capacity exhausted");
  int slot = -1;
  for (unsigned k = 0; k < e->S; ++k)
    if (!e->info[k].used) { slot = (int)k; break; }
  if (slot < 0) return fail("engine simulation slots exhausted");
  SimSlot sl{};
  GridP& g = sl.g;
  g.bin_size = d->bin_size_scale * d->cutoff;
  g.inv_bin = 1.0f / g.bin_size;
  g.R = (int)std::ceil(d->cutoff * g.inv_bin);
  unsigned long long nb = 1;
  for (int k = 0; k < 3; ++k) {
    g.mn[k] = d->min_bounds[k];
    g.ext[k] = (int)std::ceil((d->max_bounds[k] - d->min_bounds[k]) / g.bin_size);
    if (g.ext[k] < 1) return fail("max_bounds must exceed min_bounds");
    if (g.ext[k] > 1023) return fail("the engine packs bin coordinates in 10 bits: extent <= 1023 bins");
    nb *= (unsigned long long)g.ext[k];
  }
  if (g.R != 1 || g.bin_size < d->cutoff) return fail("the engine needs bin_size_scale >= 1");
  g.nbins = (unsigned)nb;
  grid_set_pow2(g);
  unsigned base = 0;
  if (bins_alloc(e, g.nbins, &base)) return fail("engine bin capacity exhausted");
  ForceP& f = sl.fp;
  f.force = d->force;
  f.k_rep = d->k_rep; f.r_rep = d->r_rep; f.k_adh = d->k_adh; f.r_adh = d->r_adh; f.k_pol = d->k_pol;
  f.rc2 = d->cutoff * d->cutoff;
  f.gab_factor = d->gabriel_coefficient * d->gabriel_coefficient * 0.25f;
  f.gab_csq = d->gabriel_coefficient * d->gabriel_coefficient;
  sl.bin_base = base;
  sl.finder = d->finder;
  sl.integrator = d->integrator;
  sl.has_pol = d->has_polarity ? 1 : 0;
  sl.active = 1;
  sl.gabriel_fast = d->gabriel_coefficient <= 0.9f ? 1 : 0;
  // append the cells after the resident ones (the next sort merges them)
  const unsigned at = e->n_resident;
  if (n) {
    ECK(cudaMemcpyAsync(e->stage, positions, (size_t)n * 12, cudaMemcpyHostToDevice, e->stream));
    k_epack<<<cdiv(n, 256), 256, 0, e->stream>>>(e->stage, n, at, (unsigned)slot, e->A, e->Asim);
    ECK(cudaGetLastError());
    if (d->has_polarity) ECK(cudaMemcpyAsync(e->PA + at, polarity, (size_t)n * 8, cudaMemcpyHostToDevice, e->stream));
    else ECK(cudaMemsetAsync(e->PA + at, 0, (size_t)n * 8, e->stream));
  }
  e->htable[slot] = sl;
  tecs_engine::Info& I = e->info[slot];
  I = tecs_engine::Info{};
  I.used = true;
  I.active = true;
  I.n = n;
  I.nbins = g.nbins;
  I.bin_base = base;
  I.appended_at = at;
  e->n_resident += n;
  e->table_dirty = e->n_dirty = true;
  // the staging buffer is reused: finish the upload before returning
  ECK(cudaStreamSynchronize(e->stream));
  *slot_out = slot;
  return 0;
}

int tecs_engine_remove(tecs_engine* e, int slot) {
  if (!e || slot < 0 || (unsigned)slot >= e->S || !e->info[slot].used) return fail("no such simulation");
  tecs_engine::Info& I = e->info[slot];
  if (!I.active) return 0;
  ECK(cudaStreamSynchronize(e->stream));  // a queued table copy reads the mirror
  I.active = false;
  e->htable[slot].active = 0;
  e->table_dirty = true;
  e->pending_free.push_back(slot);
  // Cells and bins of removed simulations are returned by the next step's sort.
  // With none active, nothing resident is needed: return everything now, so an
  // idle engine admits again without a step.
  bool any = false;
  for (unsigned k = 0; k < e->S && !any; ++k) any = e->info[k].used && e->info[k].active;
  if (!any) {
    for (int k : e->pending_free) {
      tecs_engine::Info& J = e->info[k];
      bins_free(e, J.bin_base, J.nbins);
      J = tecs_engine::Info{};
      e->htable[k] = SimSlot{};
    }
    e->pending_free.clear();
    e->n_resident = 0;
    e->n_dirty = true;
  }
  return 0;
}

int tecs_engine_step(tecs_engine* e, double dt, int n_steps) {
  if (!e) return fail("null engine");
  ECK(cudaSetDevice(e->d.device));
  const float fdt = (float)dt;
  for (int it = 0; it < n_steps; ++it) {
    if (e->table_dirty || e->n_dirty) {
      // the pinned mirrors are read by queued copies: let those finish first
      ECK(cudaStreamSynchronize(e->stream));
    }
    if (e->table_dirty) {
      ECK(cudaMemcpyAsync(e->table, e->htable, sizeof(SimSlot) * e->S, cudaMemcpyHostToDevice, e->stream));
      e->table_dirty = false;
    }
    if (e->n_dirty) {
      e->hctr->n = e->n_resident;
      ECK(cudaMemcpyAsync(&e->ctr->n, &e->hctr->n, 4, cudaMemcpyHostToDevice, e->stream));
      e->n_dirty = false;
    }
    unsigned hwm = 0;
    bool pol = false;
    for (unsigned k = 0; k < e->S; ++k)
      if (e->info[k].used) {
        hwm = std::max(hwm, e->info[k].bin_base + e->info[k].nbins);
        pol = pol || e->htable[k].has_pol;
      }
    const unsigned wantC = extent_class(e->n_resident, e->C), wantNB = extent_class(hwm, e->NB);
    if (!e->graph || e->gdt != fdt || wantC != e->gC || wantNB != e->gNB || pol != e->gpol ||
        e->gTB != e->pass_threads) {
      if (e->graph) { cudaGraphExecDestroy(e->graph); e->graph = nullptr; }
      e->gC = wantC;
      e->gNB = wantNB;
      e->gpol = pol;
      e->gTB = e->pass_threads;
      cudaGraph_t g;
      ECK(cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal));
      int rc = enqueue_engine_step(e, fdt);
      cudaError_t ce = cudaStreamEndCapture(e->stream, &g);
      if (rc) return -1;
      if (ce != cudaSuccess) return fail(std::string("engine graph capture: ") + cudaGetErrorString(ce));
      ce = cudaGraphInstantiate(&e->graph, g, 0);
      cudaGraphDestroy(g);
      if (ce != cudaSuccess) return fail(std::string("engine graph instantiate: ") + cudaGetErrorString(ce));
      e->gdt = fdt;
    }
    ECK(cudaGraphLaunch(e->graph, e->stream));
    // after the step the sorted state holds exactly the active slots' cells
    unsigned nres = 0;
    for (unsigned k = 0; k < e->S; ++k) {
      tecs_engine::Info& I = e->info[k];
      if (!I.used) continue;
      if (I.active) {
        I.sorted = true;
        I.steps++;
        nres += I.n;
      }
    }
    for (int k : e->pending_free) {
      tecs_engine::Info& I = e->info[k];
      bins_free(e, I.bin_base, I.nbins);
      I = tecs_engine::Info{};
      e->htable[k] = SimSlot{};
      e->table_dirty = true;
    }
    e->pending_free.clear();
    if (nres != e->n_resident) {
      e->n_resident = nres;
      e->n_dirty = true;
    }
  }
  return 0;
}

int tecs_engine_synchronize(tecs_engine* e) {
  if (!e) return fail("null engine");
  ECK(cudaStreamSynchronize(e->stream));
  ECK(cudaStreamSynchronize(e->side));
  return 0;
}

// Copy one simulation's state to host memory in cell-id order (synchronises).
int tecs_engine_download(tecs_engine* e, int slot, float* positions, float* polarity, unsigned* n_out) {
  if (!e || slot < 0 || (unsigned)slot >= e->S || !e->info[slot].used || !positions) return fail("no such simulation");
  const tecs_engine::Info& I = e->info[slot];
  if (!I.active) return fail("simulation was removed");
  const unsigned n = I.n;
  // pending snapshot copies read the staging buffer this reuses
  ECK(cudaStreamSynchronize(e->side));
  if (n) {
    k_erange<<<1, 1, 0, e->stream>>>(e->off, I.bin_base, I.appended_at, I.sorted ? 1 : 0, e->range);
    k_eunpack<<<cdiv(n, 256), 256, 0, e->stream>>>(e->range, n, e->A, e->PA, e->stage,
                                                   (polarity && e->htable[slot].has_pol) ? e->stagep : nullptr);
    ECK(cudaGetLastError());
    ECK(cudaMemcpyAsync(positions, e->stage, (size_t)n * 12, cudaMemcpyDeviceToHost, e->stream));
    if (polarity && e->htable[slot].has_pol)
      ECK(cudaMemcpyAsync(polarity, e->stagep, (size_t)n * 8, cudaMemcpyDeviceToHost, e->stream));
    ECK(cudaStreamSynchronize(e->stream));
  }
  if (n_out) *n_out = n;
  return 0;
}

// Snapshot without blocking the step stream: the slot's cells are unpacked
// into a staging region on the step stream (cheap, device-side), then copied
// to the caller's pinned host buffers on a side stream.  `*event` receives a
// cudaEvent_t that completes when the host buffers are filled.
int tecs_engine_snapshot_async(tecs_engine* e, int slot, float* pinned_positions, float* pinned_polarity,
                               unsigned stage_offset, void** event) {
  if (!e || slot < 0 || (unsigned)slot >= e->S || !e->info[slot].used || !pinned_positions || !event)
    return fail("no such simulation");
  const tecs_engine::Info& I = e->info[slot];
  if (!I.active) return fail("simulation was removed");
  const unsigned n = I.n;
  if ((unsigned long long)stage_offset + n > e->C) return fail("snapshot staging overflow");
  cudaEvent_t ready, done;
  ECK(cudaEventCreateWithFlags(&ready, cudaEventDisableTiming));
  ECK(cudaEventCreateWithFlags(&done, cudaEventDisableTiming));
  const bool pol = pinned_polarity && e->htable[slot].has_pol;
  float* st = e->stage + 3 * (size_t)stage_offset;
  float2* sp = e->stagep + stage_offset;
  if (n) {
    k_erange<<<1, 1, 0, e->stream>>>(e->off, I.bin_base, I.appended_at, I.sorted ? 1 : 0, e->range);
    k_eunpack<<<cdiv(n, 256), 256, 0, e->stream>>>(e->range, n, e->A, e->PA, st, pol ? sp : nullptr);
    ECK(cudaGetLastError());
  }
  ECK(cudaEventRecord(ready, e->stream));
  ECK(cudaStreamWaitEvent(e->side, ready, 0));
  if (n) {
    ECK(cudaMemcpyAsync(pinned_positions, st, (size_t)n * 12, cudaMemcpyDeviceToHost, e->side));
    if (pol) ECK(cudaMemcpyAsync(pinned_polarity, sp, (size_t)n * 8, cudaMemcpyDeviceToHost, e->side));
  }
  ECK(cudaEventRecord(done, e->side));
  cudaEventDestroy(ready);
  *event = (void*)done;
  return 0;
}

int tecs_engine_event_query(void* event, int* ready) {
  if (!event || !ready) return fail("null argument");
  cudaError_t q = cudaEventQuery((cudaEvent_t)event);
  if (q == cudaSuccess) *ready = 1;
  else if (q == cudaErrorNotReady) *ready = 0;
  else return fail(std::string("event query: ") + cudaGetErrorString(q));
  return 0;
}

int tecs_engine_event_destroy(void* event) {
  if (event) cudaEventDestroy((cudaEvent_t)event);
  return 0;
}

int tecs_engine_count(tecs_engine* e, unsigned* resident, unsigned* sims) {
  if (!e) return fail("null engine");
  unsigned k = 0;
  for (auto& I : e->info) k += (I.used && I.active) ? 1u : 0u;
  if (resident) *resident = e->n_resident;
  if (sims) *sims = k;
  return 0;
}

int tecs_engine_kernels_per_step(tecs_engine* e, int* kernels) {
  if (!e || !kernels) return fail("null argument");
  *kernels = e->kernels;
  return 0;
}

void* tecs_engine_stream(tecs_engine* e) { return e ? (void*)e->stream : nullptr; }

}  // extern "C"
