// pass_rows.cuh -- the binned force pass with each warp's neighbour rows
// staged in shared memory by bulk copies (sm_103a).
//
// Cells are sorted by (bin, id), so for a cell in bin (bx, by, bz) the
// candidates of the binned finders (binned_gabriel.hpp:95-131,
// binned_all_pairs.hpp:97-131) are nine contiguous slot ranges of the sorted
// positions: the rows (by+dy, bz+dz), bins bx-1 .. bx+1.  For 32 consecutive
// cells (one warp) each of those nine ranges moves monotonically with the cell,
// so the union of the warp's ranges per row is one contiguous run of slots.
// The warp copies its nine runs into shared memory with cp.async.bulk (one
// bulk copy per run, completion counted on a per-warp mbarrier), and every
// candidate test then reads shared memory instead of making its own global
// load.  The candidate order is still the reference's (rows in task order,
// ascending slot within a row), so the per-cell sums keep its summation order.
//
// Phases per tile of 32 cells, all within the warp (no block barrier):
//   0  home cells, their nine row ranges, the union runs, bulk copies;
//   1  each lane lists its cell's in-cutoff neighbours (staged index + bin code);
//   2  (binned Gabriel) lanes take the warp's (cell, neighbour) pairs, sorted
//      by the cell's neighbour count, and test the other neighbours as
//      witnesses; accepted pairs set bits per cell;
//   3  each lane adds its accepted pairs' forces in candidate order and writes
//      its cell (the fused integrator epilogues, links, division, bin count).
// The grid is persistent: each warp takes tiles tile, tile + warps, ..., and the
// centre-of-mass partials of all of a block's cells are reduced once at the end.
#pragma once

#include "kernels.cuh"

namespace tecs {

constexpr int kRowsWarps = 4;
constexpr int kRowsThreads = 32 * kRowsWarps;
// staged positions per warp: nine runs of about 34 cells at density 1 per bin;
// a warp whose runs hold more takes them in two halves
constexpr unsigned kStageCap = 368;
// In Heun's second pass a cell may have left its rebuild bin; its rows then
// lie apart from the other lanes' (a row or a plane away in slot order).  The
// warp copies such a cell's nine rows into this many extra stage slots
// instead (a cell whose rows do not fit takes the general path).
constexpr unsigned kStageExtra = 32;
// bounded wait on the bulk copies (each try_wait returns after at most a
// hardware-defined suspension); past it the kernel flags an error and the warp
// stops staging
constexpr unsigned kBarSpinLimit = 1u << 22;
constexpr unsigned kErrStageTimeout = 4u;

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0u;
}
// global -> this CTA's shared memory, bytes a multiple of 16, both addresses
// 16-byte aligned; completion is counted on bar
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}
// orders this warp's earlier shared-memory reads before the next bulk writes
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

template <int NB>
struct __align__(16) RowsWarp {
  float4 stage[kStageCap + kStageExtra];  // the staged runs (x, y, z, bin key), then the extra slots
  unsigned hbc[32];                 // the tile's cells' packed bin coordinates
  unsigned short self[32];          // each cell's own stage entry
  unsigned short list[NB][32];      // per lane: (staged index << 5) | bin code, candidate order
  unsigned short pinfo[NB * 32];    // (lane << 4) | q of the warp's pairs, by neighbour count
  unsigned short wcls[NB + 2];      // pairs per neighbour count
  unsigned amask[32];               // accepted neighbours of each cell, bit q
  unsigned seg0[9];                 // first slot of each row's run
  unsigned segb[9];                 // its first staged index
  unsigned extra_j[kStageExtra];    // slot of each extra stage entry
  unsigned char ncnt[32];
  unsigned long long bar;
};

// Slot of staged entry idx of row rr.
template <int NB>
__device__ __forceinline__ unsigned staged_slot(const RowsWarp<NB>& W, unsigned idx, unsigned rr) {
  return idx >= kStageCap ? W.extra_j[idx - kStageCap] : W.seg0[rr] + (idx - W.segb[rr]);
}

// Row index of a bin code (rx' + 3 ry' + 9 rz', each in 0..2): ry' + 3 rz'.
__device__ __forceinline__ unsigned code_row(unsigned code) { return code / 3u; }

// One accepted pair's terms, and their addition to the cell's sums in the
// reference's order (the spring, then for the polarity law the bending
// vector, the bending and the alignment polarity terms; pair_force's order).
template <int FORCE>
struct RowsPair {
  float sx[3];
  bool spring;  // a non-zero spring term (a zero one adds +-0 to a sum that
                // starts at +0 and so is never -0: the sum is unchanged)
  float bv[FORCE == 2 ? 3 : 1];
  float bp[FORCE == 2 ? 2 : 1];
  float al[FORCE == 2 ? 2 : 1];
};

template <int D, int FORCE, int NB>
__device__ __forceinline__ void rows_pair_terms(const RowsWarp<NB>& W, const PassArgs& a, const ForceP& fp,
                                                unsigned ent, unsigned i, const float* xi, float2 pi,
                                                const PolTrig& ti, RowsPair<FORCE>& t) {
  const float4 vj = W.stage[ent >> 5];
  float disp[3];
  disp[0] = xi[0] - vj.x;
  disp[1] = xi[1] - vj.y;
  disp[2] = D >= 3 ? xi[2] - vj.z : 0.f;
  float d2 = disp[0] * disp[0] + disp[1] * disp[1];
  if (D >= 3) d2 = d2 + disp[2] * disp[2];
  unsigned j = 0u;
  if (a.pairs || FORCE == 2) j = staged_slot(W, ent >> 5, code_row(ent & 31u));
  if (a.pairs) {
    const unsigned long long s = atomicAdd(&a.ctr->pair_count, 1ull);
    if (s < a.pair_cap) a.pairs[s] = make_uint2(id_at(a.X, a.Bid, i), id_at(a.X, a.Bid, j));
  }
  t.spring = false;
  if (FORCE == 0) return;
  const float dist = sqrtf(d2);
  if (dist != 0.0f) {
    const float F = fp.k_rep * fmaxf(fp.r_rep - dist, 0.0f) - fp.k_adh * fmaxf(dist - fp.r_adh, 0.0f);
    if (F != 0.0f) {
      t.spring = true;
#pragma unroll
      for (int d = 0; d < D; ++d) t.sx[d] = (disp[d] * F) / dist;
    }
  }
  if constexpr (FORCE == 2) {
    const float2 pj = __ldg(&a.P[j]);
    polarity_terms(fp, disp, dist, pi, ti, pj, pol_trig(pj), t.bv, t.bp, t.al);
  }
}

template <int FORCE>
__device__ __forceinline__ void rows_pair_add(const RowsPair<FORCE>& t, Acc& acc) {
  if (t.spring) {
#pragma unroll
    for (int d = 0; d < 3; ++d) acc.x[d] = acc.x[d] + t.sx[d];
  }
  if constexpr (FORCE == 2) {
#pragma unroll
    for (int d = 0; d < 3; ++d) acc.x[d] = acc.x[d] + t.bv[d];
    acc.p[0] = acc.p[0] + t.bp[0];
    acc.p[1] = acc.p[1] + t.bp[1];
    acc.p[0] = acc.p[0] + t.al[0];
    acc.p[1] = acc.p[1] + t.al[1];
  }
}

template <int D, int FORCE, int FINDER>
static __global__ void __launch_bounds__(kRowsThreads) k_pass_rows(GridP g, ForceP fp, PassArgs a) {
  static_assert(FORCE <= 1 || (FORCE == 2 && D == 3), "spring laws, or the 3-D polarity law");
  static_assert(FINDER == 1 || FINDER == 3, "the binned finders");
  constexpr int NB = kMaxNb;
  constexpr int kRows = D >= 3 ? 9 : 3;
  __shared__ RowsWarp<NB> smem[kRowsWarps];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  RowsWarp<NB>& W = smem[wib];
  if (lane == 0) mbar_init(&W.bar, 1u);
  mbar_init_fence();
  __syncwarp();
  unsigned parity = 0u;
  bool can_stage = true;
  long long comx = 0, comy = 0, comz = 0;
  const unsigned n = a.ctr->n;
  const unsigned ntiles = (n + 31u) / 32u;
  // tiles are handed out one at a time from a counter, so that warps that
  // meet cheap tiles take more of them
  unsigned tile = 0u;
  if (lane == 0) tile = atomicAdd(&a.ctr->tile_next, 1u);
  tile = __shfl_sync(0xffffffffu, tile, 0);
  for (; tile < ntiles; tile = __shfl_sync(0xffffffffu, tile, 0)) {
    const unsigned i = tile * 32u + (unsigned)lane;
    const bool active = i < n;
    float xi[3] = {0.f, 0.f, 0.f};
    float4 vi = make_float4(0.f, 0.f, 0.f, 0.f);
    float2 pi = make_float2(0.f, 0.f);
    int bc[3] = {0, 0, 0};
    unsigned lo[kRows], hi[kRows];
    // ---- phase 0: this cell's nine row ranges (empty for absent rows)
    if (active) {
      vi = __ldg(&a.X[i]);
      xi[0] = vi.x; xi[1] = vi.y; xi[2] = vi.z;
      if (FORCE == 2) pi = __ldg(&a.P[i]);
      if (FINDER == 1) bin_coords_mul<D>(g, xi, bc);
      else bin_coords_div<D>(g, xi, bc);
    }
    const int x0 = max(bc[0] - 1, 0), x1 = min(bc[0] + 1, g.ext[0] - 1);
#pragma unroll
    for (int r = 0; r < kRows; ++r) {
      const int dy = r % 3 - 1, dz = D >= 3 ? r / 3 - 1 : 0;
      const int cy = bc[1] + dy, cz = D >= 3 ? bc[2] + dz : 0;
      const bool ok = active && cy >= 0 && cy < g.ext[1] && (D < 3 || (cz >= 0 && cz < g.ext[2]));
      lo[r] = hi[r] = 0u;
      if (ok) {
        int c0[3] = {x0, cy, cz};
        const unsigned b0 = flatten<D>(g, c0);
        lo[r] = __ldg(&a.off[b0]);
        hi[r] = __ldg(&a.off[b0 + (unsigned)(x1 - x0) + 1u]);
      }
    }
    W.hbc[lane] = (unsigned)bc[0] | ((unsigned)bc[1] << 10) | ((unsigned)bc[2] << 20);
    // a cell outside its rebuild bin (w holds that bin's key) has its rows staged apart
    bool mover = false;
    if (active) {
      int cc[3] = {bc[0], bc[1], bc[2]};
      mover = flatten<D>(g, cc) != __float_as_uint(vi.w);
    }
    // The warp stages the union runs of its 32 cells; when they hold more
    // than the stage, the low and the high half-warp take turns, each with
    // its own runs (a half that still does not fit takes the general path).
    unsigned gm = 0xffffffffu;
    while (true) {
      const bool member = (gm >> lane) & 1u;
      const bool mine = active && member;
      // the union run of each row over the warp's cells, and its place in the stage
      unsigned total = 0u;
#pragma unroll
      for (int r = 0; r < kRows; ++r) {
        const bool ne = member && !mover && hi[r] > lo[r];
        const unsigned s = __reduce_min_sync(0xffffffffu, ne ? lo[r] : 0xffffffffu);
        const unsigned e = __reduce_max_sync(0xffffffffu, ne ? hi[r] : 0u);
        const unsigned len = e > s ? e - s : 0u;
        const int ridx = D >= 3 ? r : r + 3;
        if (lane == 0) {
          W.seg0[ridx] = len ? s : 0u;
          W.segb[ridx] = total;
        }
        total += len;
      }
      __syncwarp();
      if (total > kStageCap && gm == 0xffffffffu) {
        gm = 0x0000ffffu;
        continue;
      }
      const bool fits = can_stage && total <= kStageCap;
      if (fits && total > 0u) {
        // the warp's earlier reads of the stage are complete (__syncwarp
        // above); lane 0 sets the bytes to expect, then one lane per row
        // issues that row's bulk copy
        fence_proxy_async_smem();
        if (lane == 0) mbar_arrive_expect_tx(&W.bar, total * 16u);
        __syncwarp();
        if (lane < kRows) {
          const int ridx = D >= 3 ? lane : lane + 3;
          const unsigned b = W.segb[ridx];
          const unsigned nxt = (lane + 1 < kRows) ? W.segb[ridx + 1] : total;
          if (nxt > b) bulk_copy_g2s(&W.stage[b], &a.X[W.seg0[ridx]], (nxt - b) * 16u, &W.bar);
        }
        unsigned spins = 0u;
        while (!mbar_try_wait(&W.bar, parity)) {
          if (++spins >= kBarSpinLimit) break;
        }
        parity ^= 1u;
        if (spins >= kBarSpinLimit) {
          // the copies did not complete: never reuse the stage in this launch
          if (lane == 0) atomicOr(&a.ctr->error, kErrStageTimeout);
          can_stage = false;
        }
      }
      // Movers: the warp copies each one's nine rows, one after the other, into
      // the extra slots, one element per lane; mbase0 is where a mover's first
      // row starts there.
      unsigned mbase0 = 0u;
      bool mover_fb = false;
      {
        unsigned mov = __ballot_sync(0xffffffffu, mine && mover);
        unsigned ext = 0u;
        while (mov) {
          const int m = __ffs(mov) - 1;
          mov &= mov - 1u;
          unsigned tot = 0u;
#pragma unroll
          for (int r = 0; r < kRows; ++r) tot += __shfl_sync(0xffffffffu, hi[r] - lo[r], m);
          if (ext + tot > kStageExtra) {
            if (lane == m) mover_fb = true;
            continue;
          }
          if (lane == m) mbase0 = kStageCap + ext;
          for (unsigned t0 = 0u; t0 < tot; t0 += 32u) {
            // the row holding element t: the last row starting at or before it
            const unsigned t = t0 + (unsigned)lane;
            unsigned j = 0u, start = 0u;
#pragma unroll
            for (int r = 0; r < kRows; ++r) {
              const unsigned rlo = __shfl_sync(0xffffffffu, lo[r], m);
              const unsigned rlen = __shfl_sync(0xffffffffu, hi[r] - lo[r], m);
              if (t >= start) j = rlo + (t - start);
              start += rlen;
            }
            if (t < tot) {
              W.stage[kStageCap + ext + t] = __ldg(&a.X[j]);
              W.extra_j[ext + t] = j;
            }
          }
          ext += tot;
        }
        __syncwarp();
      }
      const bool use_stage = fits && can_stage;
      // ---- phase 1: in-cutoff neighbours, from the stage
      int cnt = 0;
      bool fb = mover ? mover_fb : !use_stage;
      if (mine && !fb) {
        unsigned run = mbase0;  // a mover's rows follow each other in the extra slots
#pragma unroll
        for (int r = 0; r < kRows; ++r) {
          const int ridx = D >= 3 ? r : r + 3;
          const unsigned s0 = mover ? run : lo[r] - W.seg0[ridx] + W.segb[ridx];
          run += hi[r] - lo[r];
          const unsigned s1 = s0 + (hi[r] - lo[r]);
          // the cell itself, wherever its slot lies: in Heun's second pass a
          // cell may have left its rebuild bin, so its slot need not be in the
          // centre row
          const unsigned self = (i >= lo[r] && i < hi[r]) ? s0 + (i - lo[r]) : 0xffffffffu;
          if (self != 0xffffffffu) W.self[lane] = (unsigned short)self;
          const int cy = bc[1] + (r % 3 - 1), cz = D >= 3 ? bc[2] + (r / 3 - 1) : 0;
          int c0[3] = {x0, cy, cz};
          // bin code base: rx' = key - (key of the row's first bin) + (x0 - bx + 1)
          const unsigned cbase = 3u * (unsigned)(ridx % 3) + 9u * (unsigned)(ridx / 3) + (unsigned)(x0 - bc[0] + 1) -
                                 flatten<D>(g, c0);
          for (unsigned s = s0; s < s1; s += 2u) {
            const float4 v0 = W.stage[s];
            const float4 v1 = W.stage[s + 1u < s1 ? s + 1u : s];
            const float e0 = xi[0] - v0.x, e1 = xi[1] - v0.y;
            const float f0 = xi[0] - v1.x, f1 = xi[1] - v1.y;
            float d0 = e0 * e0 + e1 * e1, d1 = f0 * f0 + f1 * f1;
            if (D >= 3) {
              const float e2 = xi[2] - v0.z, f2 = xi[2] - v1.z;
              d0 = d0 + e2 * e2;
              d1 = d1 + f2 * f2;
            }
            if (d0 < fp.rc2 && s != self) {
              if (cnt < NB) W.list[cnt][lane] = (unsigned short)((s << 5) | (cbase + __float_as_uint(v0.w)));
              ++cnt;
            }
            if (s + 1u < s1 && d1 < fp.rc2 && s + 1u != self) {
              if (cnt < NB) W.list[cnt][lane] = (unsigned short)(((s + 1u) << 5) | (cbase + __float_as_uint(v1.w)));
              ++cnt;
            }
          }
        }
        if (cnt > NB) fb = true;
      }
      if (fb) cnt = 0;
      W.ncnt[lane] = (unsigned char)cnt;
      // ---- phase 2: Gabriel test of the warp's pairs
      unsigned acc_bits = FINDER == 1 ? (cnt >= 32 ? 0xffffffffu : (1u << cnt) - 1u) : (cnt == 1 ? 1u : 0u);
      if (FINDER == 3) {
        W.amask[lane] = acc_bits;
        if (lane <= NB) W.wcls[lane] = 0;
        __syncwarp();
        const unsigned same = __match_any_sync(0xffffffffu, cnt);
        const int rank = __popc(same & ((1u << lane) - 1u));
        if (rank == 0) W.wcls[cnt] = (unsigned short)(__popc(same) * (unsigned)cnt);
        __syncwarp();
        const unsigned tot = lane <= NB ? (unsigned)W.wcls[lane] : 0u;
        unsigned incl = tot;
        for (int o = 1; o < 32; o <<= 1) {
          const unsigned y = __shfl_up_sync(0xffffffffu, incl, o);
          if (lane >= o) incl += y;
        }
        const int P = (int)__shfl_sync(0xffffffffu, incl, NB);
        const int P1 = (int)__shfl_sync(0xffffffffu, incl, 1);  // single-neighbour cells: no witness
        const int base = (int)__shfl_sync(0xffffffffu, incl - tot, cnt) + rank * cnt;
        for (int q = 0; q < cnt; ++q) W.pinfo[base + q] = (unsigned short)((lane << 4) | q);
        __syncwarp();
        for (int p = P1 + lane; p < P; p += 32) {
          const unsigned info = W.pinfo[p];
          const int c = (int)(info >> 4), q = (int)(info & 15u);
          const float4 h = W.stage[W.self[c]];
          const float4 vj = W.stage[W.list[q][c] >> 5];
          float disp[3];
          disp[0] = h.x - vj.x;
          disp[1] = h.y - vj.y;
          disp[2] = D >= 3 ? h.z - vj.z : 0.f;
          float d2 = disp[0] * disp[0] + disp[1] * disp[1];
          if (D >= 3) d2 = d2 + disp[2] * disp[2];
          float m[3] = {h.x - disp[0] * 0.5f, h.y - disp[1] * 0.5f, D >= 3 ? h.z - disp[2] * 0.5f : 0.f};
          const float rsq = d2 * fp.gab_factor;
          const int cc = W.ncnt[c];
          unsigned hits = 0u, bit = 1u;
          for (int w = 0; w < cc; w += 2) {
            const int w1 = min(w + 1, cc - 1);
            const float4 k0 = W.stage[W.list[w][c] >> 5];
            const float4 k1 = W.stage[W.list[w1][c] >> 5];
            const float f0 = k0.x - m[0], f1 = k0.y - m[1];
            const float g0 = k1.x - m[0], g1 = k1.y - m[1];
            float s0 = f0 * f0 + f1 * f1, s1 = g0 * g0 + g1 * g1;
            if (D >= 3) {
              const float f2 = k0.z - m[2], g2 = k1.z - m[2];
              s0 = s0 + f2 * f2;
              s1 = s1 + g2 * g2;
            }
            if (s0 < rsq) hits |= bit;
            if (s1 < rsq) hits |= bit << 1;
            bit <<= 2;
          }
          hits &= ((1u << cc) - 1u) & ~(1u << q);
          bool blocked = false;
          if (hits) {
            // binned_gabriel.hpp:142-153: a witness in the ball blocks only from a
            // bin that overlaps the ball, [lo, hi] per axis relative to the cell's bin
            const unsigned hb = W.hbc[c];
            const int hbc[3] = {(int)(hb & 1023u), (int)((hb >> 10) & 1023u), (int)(hb >> 20)};
            const float rr = sqrtf(rsq);
            int blo[3] = {-1, -1, -1}, bhi[3] = {1, 1, 1};
#pragma unroll
            for (int d = 0; d < D; ++d) {
              blo[d] = clampi((int)floorf((m[d] - rr - g.mn[d]) * g.inv_bin), g.ext[d] - 1) - hbc[d];
              bhi[d] = clampi((int)floorf((m[d] + rr - g.mn[d]) * g.inv_bin), g.ext[d] - 1) - hbc[d];
            }
            while (hits && !blocked) {
              const int w = __ffs(hits) - 1;
              hits &= hits - 1u;
              const unsigned code = W.list[w][c] & 31u;
              const int rel[3] = {(int)(code % 3u) - 1, (int)((code / 3u) % 3u) - 1, (int)(code / 9u) - 1};
              bool inside = true;
#pragma unroll
              for (int d = 0; d < D; ++d) inside = inside && rel[d] >= blo[d] && rel[d] <= bhi[d];
              blocked = inside;
            }
          }
          if (!blocked) atomicOr(&W.amask[c], 1u << q);
        }
        __syncwarp();
        acc_bits = W.amask[lane];
      }
      // ---- phase 3: this cell's accepted forces in candidate order, then its write
      Acc acc = {{0.f, 0.f, 0.f}, {0.f, 0.f}};
      if (mine) {
        if (fb) {
          cell_general<D, FINDER, FORCE>(g, fp, a, n, i, xi, pi, id_at(a.X, a.Bid, i), acc);
        } else {
          PolTrig ti{};
          if (FORCE == 2 && acc_bits) ti = pol_trig(pi);
          // two pairs at a time: their terms are independent (the square
          // roots and divisions overlap), their sums go in candidate order
          for (unsigned b = acc_bits; b;) {
            RowsPair<FORCE> t[2];
            int m = 0;
#pragma unroll
            for (int u = 0; u < 2; ++u) {
              if (!b) break;
              const int q = __ffs(b) - 1;
              b &= b - 1u;
              rows_pair_terms<D, FORCE>(W, a, fp, W.list[q][lane], i, xi, pi, ti, t[u]);
              ++m;
            }
#pragma unroll
            for (int u = 0; u < 2; ++u)
              if (u < m) rows_pair_add<FORCE>(t[u], acc);
          }
        }
        float s[3];
        cell_commit<D>(g, a, n, i, xi, vi, pi, acc, s);
        if (a.mode == kStore && a.com_part) {
          comx += com_fixed(s[0]);
          comy += com_fixed(s[1]);
          comz += com_fixed(s[2]);
        }
      }
      // the next group or tile overwrites the warp's lists and stage
      __syncwarp();
      if (gm == 0x0000ffffu) {
        gm = 0xffff0000u;
        continue;
      }
      break;
    }
    if (lane == 0) tile = atomicAdd(&a.ctr->tile_next, 1u);
  }
  // the last warp to run out of tiles resets the counters for the next launch
  // (every other warp has made its last fetch before it reports)
  if (lane == 0) {
    __threadfence();
    if (atomicAdd(&a.ctr->tile_exhausted, 1u) == gridDim.x * kRowsWarps - 1u) {
      a.ctr->tile_next = 0u;
      a.ctr->tile_exhausted = 0u;
    }
  }
  if (a.mode == kStore && a.com_part) com_reduce_block(a, comx, comy, comz);
}

}  // namespace tecs
