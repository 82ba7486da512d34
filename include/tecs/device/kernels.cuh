// kernels.cuh -- device kernels of one cell step on sm_103a.
//
// State layout in HBM (per simulation, capacity-sized):
//   A      float4[cap]  x, y, z, cell id (uint bits)   state between steps
//   B      float4[cap]  A reordered by (bin, cell id)   working copy of a step
//   Xt     float4[cap]  Heun predictor x~ (sorted order)
//   d1,d2  float4[cap]  pass-1 / pass-2 position deltas (sorted order)
//   PA,PB,Pt,dp1,dp2    float2 polarity counterparts
//   key,rank,src        uint[cap] bin key, tentative rank, sorted -> unsorted slot
//   cnt,off             uint[nbins+1] bin counts (zero between steps), offsets
#pragma once

#include <cfloat>

#include "common.cuh"
#include "forces.cuh"
#include "delaunay_star.cuh"

namespace tecs {

enum PassMode : int {
  kStore = 0,       // d_out[i] = sum of pair deltas
  kEulerFused = 1,  // A[i] = B[i] + sum * dt                               (euler.hpp:52-68, no COM)
  kHeun1Fused = 2,  // d_out[i] = sum; Xt[i] = B[i] + sum * dt             (heun.hpp:54-68, no COM)
  kHeun2Fused = 3   // A[i] = B[i] + ((d1[i] + sum) * 0.5) * dt            (heun.hpp:78-98, no COM)
};

struct Counters {
  unsigned n;           // active cells
  unsigned div_count;   // daughters requested this step
  unsigned done[2];     // last-block counters of the two COM reductions
  unsigned error;       // bit 0: capacity overflow on division; bit 1: a user law set drag, no old velocities kept;
                        // bit 2: a Delaunay cell search overflowed its arrays (more than kDlRow partners)
  unsigned done_div;    // last-block counter of the division fixup
  unsigned long long step;        // integrator steps taken (keys the division RNG)
  unsigned long long pair_count;  // pairs recorded by the capture hook
};

struct PassArgs {
  const float4* X;      // positions read by the pass (B or Xt)
  const float2* P;      // polarities read by the pass (PB or Pt) or null
  const unsigned* off;  // bin offsets
  Counters* ctr;
  // outputs
  float4* d_out;
  float2* dp_out;
  // fused epilogues
  const float4* Bx;     // x_n (sorted) for the fused updates
  const float2* Bp;
  const float4* d1;     // pass-1 deltas (Heun pass 2)
  const float2* dp1;
  float4* A;            // state written by the fused Euler / Heun-2 epilogue
  float2* PA;
  float4* Xt;           // predictor written by the fused Heun-1 epilogue
  float2* Pt;
  float dt;
  int mode;
  // centre-of-mass reduction (GlobalComFixer) fused into kStore
  double* com_part;     // fixed-point (2^-32) int64 sums, 3 per slot, reused as such
  float* com_out;       // 3 floats
  int com_slot;         // 0 or 1 (which done counter)
  unsigned capacity;
  // division (fused into kEulerFused / kHeun2Fused): a cell divides when
  // (hash >> 11) <= div_thresh = floor(p * 2^53), i.e. u01(hash) <= p exactly
  int div_enabled;
  unsigned long long div_thresh;
  float div_offset;
  unsigned long long seed;
  unsigned* div_parent;
  unsigned* div_slot;
  // pair capture hook
  uint2* pairs;
  unsigned long long pair_cap;
  // Gabriel fast path allowed (gabriel_coefficient <= 0.9 and bin size >= cutoff)
  int gabriel_fast;
  // cell ids of the sorted slots (binned finders keep the bin key in X.w);
  // null when X.w holds the id (naive finders)
  const unsigned* Bid;
  // bin count of the next step's rebuild, fused into the state write
  int count_next;
  unsigned* key;
  unsigned* rank;
  unsigned* cnt;
  unsigned* part;       // scan chunk totals formed while counting (count_bin), or null
  // naive Delaunay: how many times each directed pair is applied, row i at i * capacity
  const unsigned short* dmult;
  // Delaunay (any capacity): cell i's partners and their applications,
  // dl_row[i * kDlRow + t] = (j, reps) for t < dl_len[i], ascending j
  const uint2* dl_row;
  const unsigned* dl_len;
  // links of each cell id, in link order: link_ent[link_off[id] .. link_off[id + 1])
  // = (other cell id, (link index << 1) | 1 when this cell is the link's b
  // end); slot_of maps an id to its slot in X (null when X is in id order)
  const unsigned* link_off;
  const uint2* link_ent;
  const unsigned* slot_of;
  float link_k;
  // the integrator's is_full_step of this evaluation (Euler, Heun pass 1: 1; Heun pass 2: 0), for user laws
  int full_step;
  // the integrator's old velocities by cell id (integrators/base.hpp:74), or
  // null when the simulation does not keep them: user laws that set drag
  // read them (binned_gabriel.hpp:225-226, 356-357), and k_finish writes the
  // step's velocity there (euler.hpp:59, heun.hpp:87)
  float4* old_vel;
  // extra fields: E float components per cell beyond position and polarity
  // (the config's other fields), stored component-major (component k of
  // slot s at k * capacity + s).  Bit k of ex_dbl: component k belongs to a
  // Scalar field, which the reference's integrators update in double
  // (float += delta * double dt); Vector and Polarity components update in
  // float (VectorN * Scalar).
  unsigned E;
  unsigned ex_dbl;
  const float* EX;   // extras read by the pass (EB or Et)
  const float* EBx;  // x_n extras (sorted) for the fused updates
  float* ed_out;     // extra deltas written (kStore, kHeun1Fused)
  const float* ed1;  // pass-1 extra deltas (Heun pass 2, k_finish)
  const float* ed2;  // pass-2 extra deltas (k_finish)
  float* EA;         // extras of the next state
  float* Et;         // extras of the predictor
  double dt64;       // the step's dt as the caller gave it
};

// at most this many extra components per cell
constexpr unsigned kMaxExtra = 8;

// What the user-law pass keeps per cell besides the position and polarity
// sums: the drag sums (the pairs' drag and drag * the other cell's old
// velocity, in pair order, binned_gabriel.hpp:105-106, 225-226) and the NE
// extra components' values and delta sums.
template <unsigned NE>
struct LawCell {
  float drag;
  float v[3];
  float ex_self[NE > 0 ? NE : 1];
  float ex_delta[NE > 0 ? NE : 1];
};

// ---------------------------------------------------------------------------
// binning: key + count, exclusive scan, scatter, per-bin id sort + gather

constexpr int kScanThreads = 256;
constexpr int kScanPer = 16;
constexpr int kScanChunk = kScanThreads * kScanPer;
// The bin scan keeps one partial sum per chunk of kScanChunk bins and, after
// those, one sum per kScanSuper chunks, so a chunk's prefix adds up at most
// len / (kScanChunk * kScanSuper) super sums and kScanSuper - 1 chunk sums:
// linear in the bin count (a server's bin space reaches billions of bins).
constexpr unsigned kScanSuper = 4096;
constexpr size_t scan_part_words(size_t len) {
  const size_t chunks = (len + kScanChunk - 1) / kScanChunk;
  return chunks + (chunks + kScanSuper - 1) / kScanSuper;
}

// Count a cell into bin b and return its tentative rank.  With part set, the
// cell is also added to its scan chunk's total -- what k_scan_reduce would
// form from the finished counts -- with one atomic per group of lanes that
// share the chunk (consecutive cells mostly do: they are in bin order).  The
// super-chunk totals, needed past kScanSuper chunks only, come from
// k_scan_super.
static __device__ __noinline__ void add_chunk_total(unsigned* part, unsigned b) {
  const unsigned c = b / (unsigned)kScanChunk;
  const unsigned grp = __match_any_sync(__activemask(), c);
  if ((threadIdx.x & 31u) == (unsigned)(__ffs(grp) - 1)) atomicAdd(&part[c], (unsigned)__popc(grp));
}
__device__ __forceinline__ unsigned count_bin(unsigned* cnt, unsigned* part, unsigned b) {
  const unsigned r = atomicAdd(&cnt[b], 1u);
  if (part) add_chunk_total(part, b);
  return r;
}

// Super-chunk totals part[chunks + j] = sum of chunk totals j*kScanSuper ..,
// one block per super-chunk.
static __global__ void k_scan_super(unsigned* __restrict__ part, unsigned chunks) {
  __shared__ unsigned sh[32];
  const unsigned lo = blockIdx.x * kScanSuper, hi = min(chunks, lo + kScanSuper);
  unsigned v = 0u;
  for (unsigned c = lo + threadIdx.x; c < hi; c += blockDim.x) v += part[c];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31u) == 0u) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned t = 0u;
    for (unsigned w = 0; w < blockDim.x / 32u; ++w) t += sh[w];
    part[chunks + blockIdx.x] = t;
  }
}

static __global__ void k_count(const float4* __restrict__ A, const Counters* __restrict__ ctr, GridP g, int dims,
                               unsigned* __restrict__ key, unsigned* __restrict__ rank, unsigned* __restrict__ cnt,
                               unsigned* __restrict__ part) {
  const unsigned n = ctr->n;
  for (unsigned s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
    float4 v = A[s];
    float p[3] = {v.x, v.y, v.z};
    int c[3] = {0, 0, 0};
    unsigned b;
    if (dims == 3) { bin_coords_div<3>(g, p, c); b = flatten<3>(g, c); }
    else { bin_coords_div<2>(g, p, c); b = flatten<2>(g, c); }
    key[s] = b;
    rank[s] = count_bin(cnt, part, b);
  }
}

__device__ __forceinline__ unsigned block_sum(unsigned v, unsigned* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  unsigned t = 0;
  if (threadIdx.x < 32) {
    t = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0u;
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  }
  __syncthreads();
  if (threadIdx.x == 0) sh[0] = t;
  __syncthreads();
  t = sh[0];
  __syncthreads();
  return t;
}

// Per-chunk totals of cnt[0..len).
static __global__ void k_scan_reduce(const unsigned* __restrict__ cnt, unsigned len, unsigned* __restrict__ part) {
  __shared__ unsigned sh[32];
  const unsigned base = blockIdx.x * kScanChunk;
  unsigned v = 0;
  for (int k = 0; k < kScanPer; ++k) {
    unsigned idx = base + k * kScanThreads + threadIdx.x;
    if (idx < len) v += cnt[idx];
  }
  unsigned t = block_sum(v, sh);
  if (threadIdx.x == 0) {
    part[blockIdx.x] = t;
    // the super sums follow the chunk partials and are zeroed before this kernel
    atomicAdd(&part[gridDim.x + blockIdx.x / kScanSuper], t);
  }
}

// Exclusive scan of cnt into off, zeroing cnt for the next step.  Each warp
// owns 512 consecutive counts, read 32 at a time (coalesced): a first sweep
// forms the warp totals, the block combines them with the earlier chunks'
// totals, a second sweep (L1 hits) scans and writes.
static __global__ void k_scan_apply(unsigned* __restrict__ cnt, unsigned len, const unsigned* __restrict__ part,
                             unsigned* __restrict__ off) {
  __shared__ unsigned sh[32];
  __shared__ unsigned wtot[kScanThreads / 32];
  unsigned pre = 0;
  const unsigned s0 = blockIdx.x / kScanSuper;
  for (unsigned j = threadIdx.x; j < s0; j += blockDim.x) pre += part[gridDim.x + j];
  for (unsigned b = s0 * kScanSuper + threadIdx.x; b < blockIdx.x; b += blockDim.x) pre += part[b];
  pre = block_sum(pre, sh);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  constexpr int kPerWarp = kScanChunk / (kScanThreads / 32);
  const unsigned base = blockIdx.x * kScanChunk + warp * kPerWarp;
  unsigned tot = 0;
  for (int it = 0; it < kPerWarp / 32; ++it) {
    const unsigned idx = base + it * 32 + lane;
    tot += idx < len ? cnt[idx] : 0u;
  }
  for (int o = 16; o > 0; o >>= 1) tot += __shfl_xor_sync(0xffffffffu, tot, o);
  if (lane == 0) wtot[warp] = tot;
  __syncthreads();
  unsigned carry = pre;
  for (int w = 0; w < warp; ++w) carry += wtot[w];
  for (int it = 0; it < kPerWarp / 32; ++it) {
    const unsigned idx = base + it * 32 + lane;
    const unsigned v = idx < len ? cnt[idx] : 0u;
    unsigned incl = v;
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    if (idx < len) {
      off[idx] = carry + incl - v;
      cnt[idx] = 0u;
    }
    carry += __shfl_sync(0xffffffffu, incl, 31);
  }
}

// (part_words > 0: the scan has read the chunk totals that the counting
// formed; they start again from zero for the next step's count)
static __global__ void k_scatter(const Counters* __restrict__ ctr, const unsigned* __restrict__ key,
                          const unsigned* __restrict__ rank, const unsigned* __restrict__ off,
                          unsigned* __restrict__ src, unsigned* __restrict__ part, unsigned part_words) {
  const unsigned n = ctr->n;
  if (blockIdx.x == 0)
    for (unsigned w = threadIdx.x; w < part_words; w += blockDim.x) part[w] = 0u;
  for (unsigned s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x)
    src[off[key[s]] + rank[s]] = s;
}

// id of sorted slot j
__device__ __forceinline__ unsigned id_at(const float4* X, const unsigned* Bid, unsigned j) {
  return Bid ? __ldg(&Bid[j]) : id_of(__ldg(&X[j]));
}

// One thread per sorted slot: the cell that the scatter put at slot t moves to
// lo + (number of cells of its bin with a smaller id), so every bin lists its
// cells in ascending id -- the order of Kokkos BinSort's binning loop on the
// Serial backend.  Single-cell bins (most of them) copy straight through.
// the extra fields moved along with a state copy
struct ExtraMove {
  unsigned E;
  size_t C;  // capacity (component stride)
  const float* EA;
  float* EB;
};

static __global__ void k_order_gather(const Counters* __restrict__ ctr, const unsigned* __restrict__ key,
                                      const unsigned* __restrict__ off, const unsigned* __restrict__ src,
                                      const float4* __restrict__ A, const float2* __restrict__ PA,
                                      float4* __restrict__ B, float2* __restrict__ PB, unsigned* __restrict__ Bid,
                                      unsigned* __restrict__ slot_of, ExtraMove ex) {
  const unsigned n = ctr->n;
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
    // the sorted copy carries the bin key in w (read by the passes with the
    // position); the id moves to Bid
    B[dst] = make_float4(v.x, v.y, v.z, __uint_as_float(b));
    Bid[dst] = id_of(v);
    if (slot_of) slot_of[id_of(v)] = dst;  // links find their other end by id
    if (PB) PB[dst] = PA[s];
    for (unsigned k = 0; k < ex.E; ++k) ex.EB[k * ex.C + dst] = ex.EA[k * ex.C + s];
  }
}

// A step without a rebuild (rebuild_every_n > 1): the working copy takes the
// new positions in the same slot order and keeps each slot's bin key in w.
static __global__ void k_refresh(const Counters* __restrict__ ctr, const float4* __restrict__ A,
                                 const float2* __restrict__ PA, float4* __restrict__ B, float2* __restrict__ PB,
                                 ExtraMove ex) {
  const unsigned n = ctr->n;
  for (unsigned s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
    const float4 v = A[s];
    B[s] = make_float4(v.x, v.y, v.z, B[s].w);
    if (PB) PB[s] = PA[s];
    for (unsigned k = 0; k < ex.E; ++k) ex.EB[k * ex.C + s] = ex.EA[k * ex.C + s];
  }
}

// Naive finders keep the working copy in cell-id order.
static __global__ void k_id_scatter(const Counters* __restrict__ ctr, const float4* __restrict__ A,
                             const float2* __restrict__ PA, float4* __restrict__ B, float2* __restrict__ PB,
                             ExtraMove ex) {
  const unsigned n = ctr->n;
  for (unsigned s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
    float4 v = A[s];
    unsigned id = id_of(v);
    B[id] = v;
    if (PB) PB[id] = PA[s];
    for (unsigned k = 0; k < ex.E; ++k) ex.EB[k * ex.C + id] = ex.EA[k * ex.C + s];
  }
}

// ---------------------------------------------------------------------------
// block reduction of the COM partials + last-block finalisation

// Centre-of-mass partial sums in 64-bit fixed point (2^-32 units): integer
// addition is associative, so the sum -- and the mean -- is the same whatever
// order the blocks finish in, and no FP64 (slow on this part) is needed.  Each
// block adds its totals to three global accumulators; the last block forms
// mean = sum / capacity (com_fixers.hpp:43 divides by the stage view's extent,
// i.e. the capacity) and clears the accumulators for the next use.
__device__ __forceinline__ long long com_fixed(float v) { return __float2ll_rn(v * 4294967296.0f); }

static __device__ void com_reduce_block(const PassArgs& a, long long x, long long y, long long z) {
  __shared__ long long sh[3][32];
  __shared__ bool last;
  for (int o = 16; o > 0; o >>= 1) {
    x += __shfl_xor_sync(0xffffffffu, x, o);
    y += __shfl_xor_sync(0xffffffffu, y, o);
    z += __shfl_xor_sync(0xffffffffu, z, o);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (lane == 0) { sh[0][warp] = x; sh[1][warp] = y; sh[2][warp] = z; }
  __syncthreads();
  unsigned long long* acc = reinterpret_cast<unsigned long long*>(a.com_part) + 3 * a.com_slot;
  if (threadIdx.x == 0) {
    long long sx = 0, sy = 0, sz = 0;
    for (int w = 0; w < nw; ++w) { sx += sh[0][w]; sy += sh[1][w]; sz += sh[2][w]; }
    atomicAdd(&acc[0], (unsigned long long)sx);
    atomicAdd(&acc[1], (unsigned long long)sy);
    atomicAdd(&acc[2], (unsigned long long)sz);
    __threadfence();
    last = atomicAdd(&a.ctr->done[a.com_slot], 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (last && threadIdx.x == 0) {
    __threadfence();
    const double scale = 1.0 / (4294967296.0 * (double)a.capacity);
    for (int d = 0; d < 3; ++d) {
      const long long v = (long long)atomicExch(&acc[d], 0ull);
      a.com_out[d] = (float)((double)v * scale);
    }
    a.ctr->done[a.com_slot] = 0u;
  }
}

// Bin key and tentative rank of a freshly written cell for the next rebuild
// (what k_count does, fused into the state write).
template <int D>
__device__ __forceinline__ void count_cell(const GridP& g, const PassArgs& a, unsigned slot, const float* x) {
  int c[3] = {0, 0, 0};
  bin_coords_div<D>(g, x, c);
  const unsigned b = flatten<D>(g, c);
  a.key[slot] = b;
  a.rank[slot] = count_bin(a.cnt, a.part, b);
}

// ---------------------------------------------------------------------------
// division: decide (RNG keyed by cell id and step), append daughter at A[n + k]

template <int D>
__device__ __forceinline__ void maybe_divide(const GridP& g, const PassArgs& a, unsigned n, unsigned id,
                                             const float* xnew, float2 pnew, unsigned long long step,
                                             unsigned parent_slot) {
  if (!a.div_enabled) return;
  if ((hash64(a.seed, step, id, 0) >> 11) > a.div_thresh) return;
  unsigned k = atomicAdd(&a.ctr->div_count, 1u);
  unsigned slot = n + k;
  if (slot >= a.capacity) { atomicOr(&a.ctr->error, 1u); return; }
  double th = acos(2.0 * u01(hash64(a.seed, step, id, 1)) - 1.0);
  double ph = u01(hash64(a.seed, step, id, 2)) * 2.0 * 3.14159265358979323846;
  float v[3];
  pol_to_vec3((float)th, (float)ph, v);
  float4 o = make_float4(0.f, 0.f, 0.f, __uint_as_float(0xffffffffu));
  o.x = xnew[0] + a.div_offset * v[0];
  if (D >= 2) o.y = xnew[1] + a.div_offset * v[1];
  if (D >= 3) o.z = xnew[2] + a.div_offset * v[2];
  a.A[slot] = o;
  if (a.PA) a.PA[slot] = pnew;
  // the daughter takes the parent's new extra fields (written before this)
  for (unsigned c = 0; c < a.E; ++c) a.EA[c * (size_t)a.capacity + slot] = a.EA[c * (size_t)a.capacity + parent_slot];
  a.div_parent[k] = id;
  a.div_slot[k] = slot;
  if (a.count_next) {
    const float xd[3] = {o.x, o.y, o.z};
    count_cell<D>(g, a, slot, xd);
  }
}

// Daughter ids: n + rank of the parent id among this step's parents, then
// (last block) n += daughters.  Deterministic: ids depend only on parent ids.
static __global__ void k_divide_commit(Counters* __restrict__ ctr, unsigned capacity, const unsigned* __restrict__ parent,
                                const unsigned* __restrict__ slot, float4* __restrict__ A) {
  __shared__ bool last;
  const unsigned n = ctr->n;
  unsigned k = ctr->div_count;
  if (k > capacity - n) k = capacity - n;
  for (unsigned d = blockIdx.x * blockDim.x + threadIdx.x; d < k; d += gridDim.x * blockDim.x) {
    const unsigned p = parent[d];
    unsigned r = 0;
    for (unsigned e = 0; e < k; ++e) r += parent[e] < p ? 1u : 0u;
    A[slot[d]].w = __uint_as_float(n + r);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    last = atomicAdd(&ctr->done_div, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (last && threadIdx.x == 0) {
    ctr->n = n + k;
    ctr->div_count = 0u;
    ctr->step += 1ull;
    ctr->done_div = 0u;
  }
}
static __global__ void k_step_commit(Counters* __restrict__ ctr) { ctr->step += 1ull; }

// ---------------------------------------------------------------------------
// the force pass

// Gabriel witness test over the bins that overlap the ball around the
// midpoint (binned_gabriel.hpp:133-209).  true = some k blocks the pair.
template <int D>
__device__ __forceinline__ bool gabriel_blocked(const GridP& g, const ForceP& fp, const float4* __restrict__ X,
                                                const unsigned* __restrict__ off, unsigned i, unsigned j,
                                                const float* xi, const float* disp, float d2) {
  float m[3];
#pragma unroll
  for (int d = 0; d < D; ++d) m[d] = xi[d] - disp[d] * 0.5f;
  const float rsq = d2 * fp.gab_factor;
  const float r = sqrtf(rsq);
  int mn[3] = {0, 0, 0}, mx[3] = {0, 0, 0};
#pragma unroll
  for (int d = 0; d < D; ++d) {
    mn[d] = clampi((int)floorf((m[d] - r - g.mn[d]) * g.inv_bin), g.ext[d] - 1);
    mx[d] = clampi((int)floorf((m[d] + r - g.mn[d]) * g.inv_bin), g.ext[d] - 1);
  }
  const int z0 = D >= 3 ? mn[2] : 0, z1 = D >= 3 ? mx[2] : 0;
  for (int z = z0; z <= z1; ++z) {
    for (int y = mn[1]; y <= mx[1]; ++y) {
      // a row of bins along x is one contiguous segment in sorted order
      int c0[3] = {mn[0], y, z}, c1[3] = {mx[0], y, z};
      const unsigned lo = off[flatten<D>(g, c0)], hi = off[flatten<D>(g, c1) + 1];
      for (unsigned k = lo; k < hi; ++k) {
        if (k == i || k == j) continue;
        const float4 v = X[k];
        const float e0 = v.x - m[0], e1 = v.y - m[1];
        float s = e0 * e0 + e1 * e1;
        if (D >= 3) { const float e2 = v.z - m[2]; s = s + e2 * e2; }
        if (s < rsq) return true;
      }
    }
  }
  return false;
}

// naive_gabriel.hpp:71-80: every k, radius (d2 * 0.25) * c^2
template <int D>
__device__ __forceinline__ bool gabriel_blocked_naive(const ForceP& fp, const float4* __restrict__ X, unsigned n,
                                                      unsigned i, unsigned j, const float* xi, const float* disp,
                                                      float d2) {
  float m[3];
#pragma unroll
  for (int d = 0; d < D; ++d) m[d] = xi[d] - disp[d] * 0.5f;
  const float rsq = d2 * 0.25f * fp.gab_csq;
  for (unsigned k = 0; k < n; ++k) {
    if (k == i || k == j) continue;
    const float4 v = X[k];
    const float e0 = v.x - m[0], e1 = v.y - m[1];
    float s = e0 * e0 + e1 * e1;
    if (D >= 3) { const float e2 = v.z - m[2]; s = s + e2 * e2; }
    if (s < rsq) return true;
  }
  return false;
}

// ---------------------------------------------------------------------------
// Naive Delaunay (naive_delaunay.hpp).  The reference applies the pair (i, j)
// once per accepted simplex: in 2-D per third point k whose circumcircle
// through i, j, k is non-degenerate (|den| > FLT_EPSILON) and holds no other
// point (distance^2 <= r^2 rejects); in 3-D per third point k for which some
// l > k spans a non-degenerate tetrahedron with an empty circumsphere (a point
// outside the axis-aligned box |p - c| <= r is skipped before its distance
// test).  k_delaunay_mult counts the applications of every in-cutoff pair,
// one block per cell i with the threads spread over k; the force pass then
// adds the pair's force that many times, in j order -- the Serial order.
template <int D>
__device__ __forceinline__ float sq_len(const float4& v) {
  float s = v.x * v.x + v.y * v.y;
  if (D >= 3) s = s + v.z * v.z;
  return s;
}

template <int D>
__device__ __forceinline__ float sq_dist(const float4& v, const float* c) {
  const float e0 = v.x - c[0], e1 = v.y - c[1];
  float s = e0 * e0 + e1 * e1;
  if (D >= 3) { const float e2 = v.z - c[2]; s = s + e2 * e2; }
  return s;
}

__device__ __forceinline__ bool delaunay_triangle_empty(const float4* __restrict__ X, unsigned n, unsigned i,
                                                        unsigned j, unsigned k, const float4& pi, const float4& pj,
                                                        float li, float lj) {
  const float4 pk = __ldg(&X[k]);
  const float den = 2.0f * (pi.x * (pj.y - pk.y) + pj.x * (pk.y - pi.y) + pk.x * (pi.y - pj.y));
  if (fabsf(den) <= FLT_EPSILON) return false;
  const float lk = sq_len<2>(pk);
  float c[2];
  c[0] = (li * (pj.y - pk.y) + lj * (pk.y - pi.y) + lk * (pi.y - pj.y)) / den;
  c[1] = (li * (pk.x - pj.x) + lj * (pi.x - pk.x) + lk * (pj.x - pi.x)) / den;
  const float r2 = sq_dist<2>(pi, c);
  for (unsigned m = 0; m < n; ++m) {
    if (m == i || m == j || m == k) continue;
    if (sq_dist<2>(__ldg(&X[m]), c) <= r2) return false;
  }
  return true;
}

__device__ __forceinline__ bool delaunay_any_tetrahedron(const float4* __restrict__ X, unsigned n, unsigned i,
                                                         unsigned j, unsigned k, const float4& pi, const float4& pj,
                                                         float li, float lj) {
  const float4 pk = __ldg(&X[k]);
  const float lk = sq_len<3>(pk);
  for (unsigned l = k + 1; l < n; ++l) {
    if (l == i || l == j) continue;
    const float4 pl = __ldg(&X[l]);
    const float e1[3] = {pj.x - pi.x, pj.y - pi.y, pj.z - pi.z};
    const float e2[3] = {pk.x - pi.x, pk.y - pi.y, pk.z - pi.z};
    const float e3[3] = {pl.x - pi.x, pl.y - pi.y, pl.z - pi.z};
    const float den = 2.0f * (e1[0] * (e2[1] * e3[2] - e2[2] * e3[1]) - e1[1] * (e2[0] * e3[2] - e2[2] * e3[0]) +
                              e1[2] * (e2[0] * e3[1] - e2[1] * e3[0]));
    if (fabsf(den) <= FLT_EPSILON) continue;
    const float b1 = lj - li, b2 = lk - li, b3 = sq_len<3>(pl) - li;
    float c[3];
    c[0] = pi.x + (b1 * (e2[1] * e3[2] - e2[2] * e3[1]) - e1[1] * (b2 * e3[2] - e2[2] * b3) +
                   e1[2] * (b2 * e3[1] - e2[1] * b3)) / den;
    c[1] = pi.y + (e1[0] * (b2 * e3[2] - e2[2] * b3) - b1 * (e2[0] * e3[2] - e2[2] * e3[0]) +
                   e1[2] * (e2[0] * b3 - b2 * e3[0])) / den;
    c[2] = pi.z + (e1[0] * (e2[1] * b3 - b2 * e3[1]) - e1[1] * (e2[0] * b3 - b2 * e3[0]) +
                   b1 * (e2[0] * e3[1] - e2[1] * e3[0])) / den;
    const float r2 = sq_dist<3>(pi, c);
    const float r = sqrtf(r2);
    bool ok = true;
    for (unsigned m = 0; m < n; ++m) {
      if (m == i || m == j || m == k || m == l) continue;
      const float4 pm = __ldg(&X[m]);
      if (fabsf(pm.x - c[0]) > r || fabsf(pm.y - c[1]) > r || fabsf(pm.z - c[2]) > r) continue;
      if (sq_dist<3>(pm, c) <= r2) { ok = false; break; }
    }
    if (ok) return true;
  }
  return false;
}

constexpr int kDelaunayThreads = 128;
constexpr unsigned kDelaunayMaxCells = 4096;  // the pair-count table is capacity^2 x 2 bytes

template <int D>
static __global__ void __launch_bounds__(kDelaunayThreads)
k_delaunay_mult(const float4* __restrict__ X, const Counters* __restrict__ ctr, float rc2, unsigned stride,
                unsigned short* __restrict__ mult) {
  __shared__ unsigned cnt;
  const unsigned n = ctr->n;
  const unsigned i = blockIdx.x;
  if (i >= n) return;
  const float4 pi = __ldg(&X[i]);
  const float li = sq_len<D>(pi);
  for (unsigned j = 0; j < n; ++j) {
    if (j == i) continue;
    const float4 pj = __ldg(&X[j]);
    const float e0 = pi.x - pj.x, e1 = pi.y - pj.y;
    float d2 = e0 * e0 + e1 * e1;
    if (D >= 3) { const float e2 = pi.z - pj.z; d2 = d2 + e2 * e2; }
    if (d2 >= rc2) continue;  // the same test, on the same values, in every thread
    if (threadIdx.x == 0) cnt = 0u;
    __syncthreads();
    const float lj = sq_len<D>(pj);
    unsigned local = 0;
    for (unsigned k = threadIdx.x; k < n; k += kDelaunayThreads) {
      if (k == i || k == j) continue;
      local += (D == 2 ? delaunay_triangle_empty(X, n, i, j, k, pi, pj, li, lj)
                       : delaunay_any_tetrahedron(X, n, i, j, k, pi, pj, li, lj)) ? 1u : 0u;
    }
    if (local) atomicAdd(&cnt, local);
    __syncthreads();
    if (threadIdx.x == 0) mult[(size_t)i * stride + j] = (unsigned short)cnt;
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Delaunay finder for any capacity (tecs/device/delaunay_star.cuh).  Before
// each pass: the bounding box of the pass's positions, a bin grid of about
// two cells per bin, a counting sort into it, then each cell's partners and
// multiplicities (k_dl_mult, one thread per cell).  The pass applies each
// listed pair reps times in ascending j, as FINDER 4 does.
constexpr unsigned kDlRow = 64;  // partners per cell
constexpr int kDlThreads = 64;

struct DlState {
  unsigned mm[6];  // ordered-integer min (0..2) and max (3..5) of the coordinates
  double lo[3];
  double h, inv;
  int dims[3];
  unsigned nbins;
};

__device__ __forceinline__ unsigned f2ord(float f) {
  const unsigned u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord2f(unsigned u) {
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

static __global__ void k_dl_reset(DlState* st) {
  if (threadIdx.x < 3) { st->mm[threadIdx.x] = 0xffffffffu; st->mm[3 + threadIdx.x] = 0u; }
}

template <int D>
static __global__ void k_dl_bounds(const float4* __restrict__ X, const Counters* __restrict__ ctr, DlState* st) {
  const unsigned n = ctr->n;
  unsigned lo[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu}, hi[3] = {0u, 0u, 0u};
  for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float4 v = X[i];
    const float c[3] = {v.x, v.y, v.z};
#pragma unroll
    for (int d = 0; d < D; ++d) {
      const unsigned o = f2ord(c[d]);
      lo[d] = min(lo[d], o);
      hi[d] = max(hi[d], o);
    }
  }
#pragma unroll
  for (int d = 0; d < D; ++d) {
    for (int sh = 16; sh > 0; sh >>= 1) {
      lo[d] = min(lo[d], __shfl_xor_sync(0xffffffffu, lo[d], sh));
      hi[d] = max(hi[d], __shfl_xor_sync(0xffffffffu, hi[d], sh));
    }
    if ((threadIdx.x & 31) == 0) { atomicMin(&st->mm[d], lo[d]); atomicMax(&st->mm[3 + d], hi[d]); }
  }
}

template <int D>
static __global__ void k_dl_plan(const Counters* __restrict__ ctr, unsigned max_bins, DlState* st) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const unsigned n = ctr->n;
  double mn[3] = {0.0, 0.0, 0.0}, mx[3] = {0.0, 0.0, 0.0};
  if (n > 0)
    for (int d = 0; d < D; ++d) { mn[d] = ord2f(st->mm[d]); mx[d] = ord2f(st->mm[3 + d]); }
  dl::Grid g{};
  dl::plan_grid<D>(g, mn, mx, n, max_bins);
  for (int d = 0; d < 3; ++d) { st->lo[d] = g.lo[d]; st->dims[d] = g.dims[d]; }
  st->h = g.h;
  st->inv = g.inv;
  st->nbins = g.nbins;
}

__device__ __forceinline__ dl::Grid dl_view(const DlState* st) {
  dl::Grid g{};
  for (int d = 0; d < 3; ++d) { g.lo[d] = st->lo[d]; g.dims[d] = st->dims[d]; }
  g.h = st->h;
  g.inv = st->inv;
  g.nbins = st->nbins;
  return g;
}

template <int D>
__device__ __forceinline__ unsigned dl_bin(const dl::Grid& g, const float4& v) {
  const double q[3] = {v.x, v.y, v.z};
  int b[3];
  dl::bin_of<D>(g, q, b);
  return dl::flat(g, b[0], b[1], b[2]);
}

template <int D>
static __global__ void k_dl_count(const float4* __restrict__ X, const Counters* __restrict__ ctr,
                                  const DlState* __restrict__ st, unsigned* __restrict__ cnt) {
  const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ctr->n) return;
  const dl::Grid g = dl_view(st);
  atomicAdd(&cnt[dl_bin<D>(g, X[i])], 1u);
}

// exclusive scan of the bin counts into off (off[nbins] = cells), one block;
// the counts are cleared for the scatter's cursors
static __global__ void __launch_bounds__(1024) k_dl_scan(const DlState* __restrict__ st, unsigned* __restrict__ cnt,
                                                         unsigned* __restrict__ off) {
  __shared__ unsigned part[1024];
  const unsigned nb = st->nbins, t = threadIdx.x;
  const unsigned per = (nb + 1023u) / 1024u, b0 = min(nb, t * per), b1 = min(nb, b0 + per);
  unsigned sum = 0;
  for (unsigned b = b0; b < b1; ++b) sum += cnt[b];
  part[t] = sum;
  __syncthreads();
  for (unsigned sh = 1; sh < 1024u; sh <<= 1) {
    const unsigned v = t >= sh ? part[t - sh] : 0u;
    __syncthreads();
    part[t] += v;
    __syncthreads();
  }
  unsigned run = part[t] - sum;
  for (unsigned b = b0; b < b1; ++b) {
    const unsigned c = cnt[b];
    off[b] = run;
    run += c;
    cnt[b] = 0u;
  }
  if (t == 1023u) off[nb] = part[1023];
}

template <int D>
static __global__ void k_dl_scatter(const float4* __restrict__ X, const Counters* __restrict__ ctr,
                                    const DlState* __restrict__ st, unsigned* __restrict__ cnt,
                                    const unsigned* __restrict__ off, unsigned* __restrict__ idx,
                                    float4* __restrict__ sp) {
  const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ctr->n) return;
  const dl::Grid g = dl_view(st);
  const float4 v = X[i];
  const unsigned b = dl_bin<D>(g, v);
  const unsigned at = off[b] + atomicAdd(&cnt[b], 1u);
  idx[at] = i;
  sp[at] = v;
}

// one warp per cell: the lanes share each search's entries (dl::Warp)
template <int D>
static __global__ void __launch_bounds__(kDlThreads) k_dl_mult(const float4* __restrict__ X, Counters* __restrict__ ctr,
                                                               const DlState* __restrict__ st,
                                                               const unsigned* __restrict__ off,
                                                               const unsigned* __restrict__ idx,
                                                               const float4* __restrict__ sp, float rc2,
                                                               uint2* __restrict__ row, unsigned* __restrict__ len) {
  const unsigned n = ctr->n;
  const unsigned i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;  // the same in every lane of the warp
  if (i >= n) return;
  dl::Grid g = dl_view(st);
  g.off = off;
  g.idx = idx;
  g.sp = reinterpret_cast<const dl::Pt*>(sp);
  g.P = reinterpret_cast<const dl::Pt*>(X);
  g.n = n;
  g.rc2 = rc2;
  // the warp's star and candidate lists: one copy, in shared memory
  __shared__ __align__(16) unsigned char scratch[(kDlThreads / 32) * sizeof(dl::Scratch)];
  dl::Scratch& sc = reinterpret_cast<dl::Scratch*>(scratch)[threadIdx.x >> 5];
  unsigned oj[kDlRow], orp[kDlRow], err = 0;
  const dl::Warp lanes;
  const unsigned m = dl::cell_mult<D>(lanes, g, i, oj, orp, kDlRow, &err, sc);
  if (lanes.lane() != 0u) return;
  for (unsigned t = 0; t < m; ++t) row[(size_t)i * kDlRow + t] = make_uint2(oj[t], orp[t]);
  len[i] = m;
  // a full near-circle list keeps the points nearest the circle (no error);
  // any other overflow leaves the row incomplete
  if (err & (dl::kErrStar | dl::kErrPairs | dl::kErrList)) atomicOr(&ctr->error, 4u);
}

template <int D, int FINDER, int FORCE>
__device__ __forceinline__ void visit(const GridP& g, const ForceP& fp, const PassArgs& a, unsigned n, unsigned i,
                                      unsigned j, const float* xi, float2 pi, Acc& acc, unsigned idi,
                                      unsigned reps5 = 1u) {
  const float4 vj = a.X[j];
  float disp[3];
  disp[0] = xi[0] - vj.x;
  if (D >= 2) disp[1] = xi[1] - vj.y;
  if (D >= 3) disp[2] = xi[2] - vj.z;
  float d2 = disp[0] * disp[0] + disp[1] * disp[1];
  if (D >= 3) d2 = d2 + disp[2] * disp[2];
  if (d2 >= fp.rc2) return;
  if (FINDER == 3 && gabriel_blocked<D>(g, fp, a.X, a.off, i, j, xi, disp, d2)) return;
  if (FINDER == 2 && gabriel_blocked_naive<D>(fp, a.X, n, i, j, xi, disp, d2)) return;
  unsigned reps = FINDER == 5 ? reps5 : 1u;
  if (FINDER == 4 && (reps = a.dmult[(size_t)i * a.capacity + j]) == 0u) return;
  if (a.pairs) {
    unsigned long long s = atomicAdd(&a.ctr->pair_count, (unsigned long long)reps);
    for (unsigned r = 0; r < reps; ++r)
      if (s + r < a.pair_cap) a.pairs[s + r] = make_uint2(idi, id_at(a.X, a.Bid, j));
  }
  const float dist = sqrtf(d2);
  const float2 pj = (FORCE == 2 && a.P) ? a.P[j] : make_float2(0.f, 0.f);
  for (unsigned r = 0; r < reps; ++r) pair_force<D, FORCE>(fp, disp, dist, pi, pj, acc);
}

// Commit of one cell: out(i) = 0 + sum (views(i) += values on cleared stage
// buffers); the drag term adds exactly zero for the built-in laws
// (pairwise_drag = 0).  Then the fused integrator epilogue of the mode.
// One link's force on this cell, added after the pairwise sum: the
// constant-pull law of examples/intercalation.cpp:65-71 -- cell a gets
// k*(x_b - x_a)/|x_b - x_a|, cell b its negative -- in the Serial order of
// integrators/base.hpp:205-233 (link order, each term from a zero accumulator).
// A link to an id beyond the active cells sees the zero position of an unused
// view slot.
template <int D>
__device__ __forceinline__ void add_link(const PassArgs& a, unsigned n, const float* xs, unsigned e, float* s) {
  const uint2 le = a.link_ent[e];
  const bool b_end = (le.y & 1u) != 0u;
  float xo[3] = {0.f, 0.f, 0.f};
  if (le.x < n) {
    const float4 v = a.X[a.slot_of ? a.slot_of[le.x] : le.x];
    xo[0] = v.x; xo[1] = v.y; xo[2] = v.z;
  }
  float disp[3] = {0.f, 0.f, 0.f};
#pragma unroll
  for (int d = 0; d < D; ++d) disp[d] = b_end ? xs[d] - xo[d] : xo[d] - xs[d];
  float d2 = disp[0] * disp[0] + disp[1] * disp[1];
  if (D >= 3) d2 = d2 + disp[2] * disp[2];
  const float dist = sqrtf(d2);
  const float k = b_end ? -a.link_k : a.link_k;
#pragma unroll
  for (int d = 0; d < D; ++d) s[d] = s[d] + (0.0f + (k * disp[d]) / dist);
}

// One extra component's update, in double for Scalar fields (the reference's
// float += float * double) and in float otherwise.
__device__ __forceinline__ float ex_update(float x, float d, float dt, double dt64, bool dbl) {
  return dbl ? (float)((double)x + (double)d * dt64) : x + d * dt;
}

// The extra fields of one active cell (slot i): the mode's delta store and
// state update, as cell_commit does for the position.  exd: the cell's extra
// deltas, 0 + its sums (null: zero).
__device__ __forceinline__ void commit_extras(const PassArgs& a, unsigned i, const float* exd) {
  const size_t C = a.capacity;
  for (unsigned k = 0; k < a.E; ++k) {
    const float d = exd ? exd[k] : 0.0f;
    const bool dbl = (a.ex_dbl >> k) & 1u;
    const size_t at = k * C + i;
    if (a.mode == kStore) {
      a.ed_out[at] = d;
    } else if (a.mode == kHeun1Fused) {
      a.ed_out[at] = d;
      a.Et[at] = ex_update(a.EX[at], d, a.dt, a.dt64, dbl);
    } else if (a.mode == kEulerFused) {
      a.EA[at] = ex_update(a.EBx[at], d, a.dt, a.dt64, dbl);
    } else {
      // Heun: x += (d1 + d2) * 0.5 * dt (heun.hpp:89-90)
      const float h = a.ed1[at] + d;
      const float xb = a.EBx[at];
      a.EA[at] = dbl ? (float)((double)xb + ((double)h * 0.5) * a.dt64) : xb + (h * 0.5f) * a.dt;
    }
  }
}

// The library's link law: the constant pull (add_link).  A user LINK_FORCE
// law takes its place in the user-law pass (tecs/pairwise.cuh).
struct BuiltinLinks {
  template <int D>
  __device__ __forceinline__ void add(const PassArgs& a, unsigned n, unsigned id, const float* xs, float2 ps,
                                      unsigned e, float* s, float* sp, float* se) const {
    add_link<D>(a, n, xs, e, s);
  }
};

// The write of one active cell: links, then the mode's store or fused
// integrator update, the next rebuild's bin count and division.  s receives
// the cell's position delta (for the COM partials).
// NE: the extra components the pass carries (the user-law pass of a config
// with extra fields; the built-in passes carry none and leave the extra
// fields to k_predict / k_finish, see enqueue_step).
template <int D, class Links = BuiltinLinks, unsigned NE = 0>
__device__ __forceinline__ void cell_commit(const GridP& g, const PassArgs& a, unsigned n, unsigned i,
                                            const float* xi, const float4& vi, const float2& pi, const Acc& acc,
                                            float* s, const Links& links = Links{}, const float* exd = nullptr) {
#pragma unroll
  for (int d = 0; d < 3; ++d) s[d] = 0.0f + acc.x[d];
  float sp[2] = {0.0f + acc.p[0], 0.0f + acc.p[1]};
  float se[NE > 0 ? NE : 1];
  if constexpr (NE > 0) {
#pragma unroll
    for (unsigned k = 0; k < NE; ++k) se[k] = 0.0f + exd[k];
  }
  if (a.link_off) {
    const unsigned id = a.Bid ? a.Bid[i] : id_of(vi);
    const unsigned e1 = a.link_off[id + 1];
    for (unsigned e = a.link_off[id]; e < e1; ++e) links.template add<D>(a, n, id, xi, pi, e, s, sp, se);
  }
  if constexpr (NE > 0) commit_extras(a, i, se);
  const float sp0 = sp[0], sp1 = sp[1];
  if (a.mode == kStore) {
    a.d_out[i] = make_float4(s[0], s[1], s[2], 0.f);
    if (a.dp_out) a.dp_out[i] = make_float2(sp0, sp1);
    return;
  }
  const float dt = a.dt;
  if (a.mode == kHeun1Fused) {
    a.d_out[i] = make_float4(s[0], s[1], s[2], 0.f);
    a.Xt[i] = make_float4(xi[0] + s[0] * dt, xi[1] + s[1] * dt, xi[2] + s[2] * dt, vi.w);
    if (a.P) {
      a.dp_out[i] = make_float2(sp0, sp1);
      a.Pt[i] = make_float2(pi.x + sp0 * dt, pi.y + sp1 * dt);
    }
    return;
  }
  // kEulerFused / kHeun2Fused: write the next state into A (w = cell id)
  const float4 xb = a.Bx[i];
  const unsigned idb = a.Bid ? a.Bid[i] : id_of(xb);
  float xn[3];
  float2 pn = make_float2(0.f, 0.f);
  if (a.mode == kEulerFused) {
    xn[0] = xb.x + s[0] * dt; xn[1] = xb.y + s[1] * dt; xn[2] = xb.z + s[2] * dt;
    if (a.P) { const float2 pb = a.Bp[i]; pn = make_float2(pb.x + sp0 * dt, pb.y + sp1 * dt); }
  } else {
    const float4 d1 = a.d1[i];
    const float h0 = d1.x + s[0], h1 = d1.y + s[1], h2 = d1.z + s[2];
    xn[0] = xb.x + (h0 * 0.5f) * dt; xn[1] = xb.y + (h1 * 0.5f) * dt; xn[2] = xb.z + (h2 * 0.5f) * dt;
    if (a.P) {
      const float2 pb = a.Bp[i], q1 = a.dp1[i];
      const float g0 = q1.x + sp0, g1 = q1.y + sp1;
      pn = make_float2(pb.x + (g0 * 0.5f) * dt, pb.y + (g1 * 0.5f) * dt);
    }
  }
  if (D < 3) xn[2] = 0.f;
  a.A[i] = make_float4(xn[0], xn[1], xn[2], __uint_as_float(idb));
  if (a.PA) a.PA[i] = pn;
  if (a.count_next) count_cell<D>(g, a, i, xn);
  maybe_divide<D>(g, a, n, idb, xn, pn, a.ctr->step, i);
}

// cell_commit for an active cell, then (every thread of the block) the COM
// partials of kStore.
template <int D, class Links = BuiltinLinks, unsigned NE = 0>
__device__ __forceinline__ void pass_epilogue(const GridP& g, const PassArgs& a, bool active, unsigned n, unsigned i,
                                              const float* xi, const float4& vi, const float2& pi, const Acc& acc,
                                              const Links& links = Links{}, const float* exd = nullptr) {
  float s[3] = {0.f, 0.f, 0.f};
  if (active) cell_commit<D, Links, NE>(g, a, n, i, xi, vi, pi, acc, s, links, exd);
  if (a.mode == kStore && a.com_part)
    com_reduce_block(a, active ? com_fixed(s[0]) : 0ll, active ? com_fixed(s[1]) : 0ll,
                     active ? com_fixed(s[2]) : 0ll);
}


// ---------------------------------------------------------------------------
// Gabriel fast path.
//
// A witness k that blocks the pair (i, j) lies inside the ball of radius
// r = c*d/2 around the midpoint m, and |x_i - m| = d/2, so |x_k - x_i| < d(1+c)/2.
// For c <= 0.9 and d < cutoff that is < 0.95 * cutoff: every witness is itself
// one of i's in-cutoff neighbours, found in i's 27 candidate bins.  The pass
// therefore collects i's in-cutoff neighbours (candidate order = the
// reference's summation order) into shared memory and tests each pair against
// the others, keeping the reference's bin-range restriction on k exactly
// (binned_gabriel.hpp:142-207).  If a cell has more than kMaxNb neighbours, or
// a ball's bin range leaves i's 3x3x3 block, the cell takes the general path.
constexpr int kMaxNb = 16;
// Threads (cells) per block of the cooperative passes: three warps.  The
// block's shared memory (about 30 KB) then lets seven blocks share an SM, 672
// cells, so that a 100k-cell pass runs in a single wave on 152 SMs.
constexpr int kPassThreads = 96;
// Position arrays that the cooperative pass scans hold this many float4 past
// their capacity: the candidate scan reads whole rounds past a row's end (at
// most 31 slots) and masks the extra slots off.
constexpr unsigned kRowPad = 64;

// nb: room for MAXN neighbours at a stride of STRIDE (the block size)
template <int D, int FORCE, int MAXN = kMaxNb, int STRIDE = kPassThreads>
__device__ __forceinline__ bool gabriel_cell_fast(const GridP& g, const ForceP& fp, const PassArgs& a, unsigned i,
                                                  const float* xi, float2 pi, unsigned idi, Acc& acc,
                                                  float4* nb) {
  int bc[3] = {0, 0, 0};
  bin_coords_div<D>(g, xi, bc);
  int cnt = 0;
  const int z0 = D >= 3 ? -1 : 0, z1 = D >= 3 ? 1 : 0;
  for (int dz = z0; dz <= z1; ++dz) {
    const int cz = D >= 3 ? bc[2] + dz : 0;
    if (D >= 3 && (cz < 0 || cz >= g.ext[2])) continue;
    for (int dy = -1; dy <= 1; ++dy) {
      const int cy = bc[1] + dy;
      if (cy < 0 || cy >= g.ext[1]) continue;
      const int x0 = max(bc[0] - 1, 0), x1 = min(bc[0] + 1, g.ext[0] - 1);
      int c0[3] = {x0, cy, cz};
      const unsigned b0 = flatten<D>(g, c0);
      // boundaries of the (up to) three bins of this row
      const unsigned o0 = __ldg(&a.off[b0]);
      const unsigned o1 = __ldg(&a.off[b0 + 1]);
      const unsigned o2 = x1 >= x0 + 1 ? __ldg(&a.off[b0 + 2]) : o1;
      const unsigned o3 = x1 >= x0 + 2 ? __ldg(&a.off[b0 + 3]) : o2;
      for (unsigned j = o0; j < o3; ++j) {
        if (j == i) continue;
        const float4 vj = __ldg(&a.X[j]);
        const float e0 = xi[0] - vj.x, e1 = xi[1] - vj.y;
        float d2 = e0 * e0 + e1 * e1;
        if (D >= 3) { const float e2 = xi[2] - vj.z; d2 = d2 + e2 * e2; }
        if (d2 >= fp.rc2) continue;
        if (cnt == MAXN) return false;
        const int rx = x0 + (j >= o1 ? 1 : 0) + (j >= o2 ? 1 : 0) - bc[0];
        const unsigned code = (unsigned)(rx + 1) | ((unsigned)(dy + 1) << 2) | ((unsigned)(dz + 1) << 4);
        nb[cnt * STRIDE] = make_float4(vj.x, vj.y, vj.z, __uint_as_float((j << 6) | code));
        ++cnt;
      }
    }
  }
  // pass over the pairs: Gabriel test against the other neighbours
  unsigned accepted = 0u;
  for (int q = 0; q < cnt; ++q) {
    const float4 vj = nb[q * STRIDE];
    float disp[3];
    disp[0] = xi[0] - vj.x;
    disp[1] = xi[1] - vj.y;
    disp[2] = D >= 3 ? xi[2] - vj.z : 0.f;
    float d2 = disp[0] * disp[0] + disp[1] * disp[1];
    if (D >= 3) d2 = d2 + disp[2] * disp[2];
    // midpoint ball and its bin range, relative to i's bin
    float m[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int d = 0; d < D; ++d) m[d] = xi[d] - disp[d] * 0.5f;
    const float rsq = d2 * fp.gab_factor;
    const float r = sqrtf(rsq);
    int lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
#pragma unroll
    for (int d = 0; d < D; ++d) {
      lo[d] = clampi((int)floorf((m[d] - r - g.mn[d]) * g.inv_bin), g.ext[d] - 1) - bc[d];
      hi[d] = clampi((int)floorf((m[d] + r - g.mn[d]) * g.inv_bin), g.ext[d] - 1) - bc[d];
      if (lo[d] < -1 || hi[d] > 1) return false;
    }
    bool blocked = false;
    for (int w = 0; w < cnt && !blocked; ++w) {
      if (w == q) continue;
      const float4 vk = nb[w * STRIDE];
      const unsigned code = __float_as_uint(vk.w) & 63u;
      const int rx = (int)(code & 3u) - 1, ry = (int)((code >> 2) & 3u) - 1, rz = (int)((code >> 4) & 3u) - 1;
      if (rx < lo[0] || rx > hi[0] || ry < lo[1] || ry > hi[1]) continue;
      if (D >= 3 && (rz < lo[2] || rz > hi[2])) continue;
      const float f0 = vk.x - m[0], f1 = vk.y - m[1];
      float s = f0 * f0 + f1 * f1;
      if (D >= 3) { const float f2 = vk.z - m[2]; s = s + f2 * f2; }
      if (s < rsq) blocked = true;
    }
    if (!blocked) accepted |= 1u << q;
  }
  // forces of the accepted pairs, in candidate (= reference summation) order
  Acc loc = {{0.f, 0.f, 0.f}, {0.f, 0.f}};
  while (accepted) {
    const int q = __ffs(accepted) - 1;
    accepted &= accepted - 1u;
    const float4 vj = nb[q * STRIDE];
    const unsigned j = __float_as_uint(vj.w) >> 6;
    float disp[3];
    disp[0] = xi[0] - vj.x;
    disp[1] = xi[1] - vj.y;
    disp[2] = D >= 3 ? xi[2] - vj.z : 0.f;
    float d2 = disp[0] * disp[0] + disp[1] * disp[1];
    if (D >= 3) d2 = d2 + disp[2] * disp[2];
    if (a.pairs) {
      unsigned long long s = atomicAdd(&a.ctr->pair_count, 1ull);
      if (s < a.pair_cap) a.pairs[s] = make_uint2(idi, id_at(a.X, a.Bid, j));
    }
    const float dist = sqrtf(d2);
    const float2 pj = (FORCE == 2 && a.P) ? __ldg(&a.P[j]) : make_float2(0.f, 0.f);
    pair_force<D, FORCE>(fp, disp, dist, pi, pj, loc);
  }
  acc = loc;
  return true;
}

template <int D, int FINDER, int FORCE>
__device__ __forceinline__ void cell_general(const GridP& g, const ForceP& fp, const PassArgs& a, unsigned n, unsigned i,
                                          const float* xi, float2 pi, unsigned idi, Acc& acc);

template <int D, int FINDER, int FORCE>
static __global__ void __launch_bounds__(kPassThreads) k_pass(GridP g, ForceP fp, PassArgs a) {
  const unsigned n = a.ctr->n;
  const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = i < n;
  Acc acc = {{0.f, 0.f, 0.f}, {0.f, 0.f}};
  float xi[3] = {0.f, 0.f, 0.f};
  float4 vi = make_float4(0.f, 0.f, 0.f, 0.f);
  float2 pi = make_float2(0.f, 0.f);
  if (active) {
    vi = a.X[i];
    xi[0] = vi.x; xi[1] = vi.y; xi[2] = vi.z;
    if (a.P) pi = a.P[i];
    const unsigned idi = id_at(a.X, a.Bid, i);
    if (FINDER == 3 && a.gabriel_fast) {
      __shared__ float4 nbuf[kMaxNb * kPassThreads];
      if (!gabriel_cell_fast<D, FORCE>(g, fp, a, i, xi, pi, idi, acc, &nbuf[threadIdx.x])) {
        // nothing was recorded or accumulated yet: redo the cell the general way
        cell_general<D, FINDER, FORCE>(g, fp, a, n, i, xi, pi, idi, acc);
      }
    } else {
      cell_general<D, FINDER, FORCE>(g, fp, a, n, i, xi, pi, idi, acc);
    }
  }
  pass_epilogue<D>(g, a, active, n, i, xi, vi, pi, acc);
}

// The general path: the reference's loops (27 bins, then the ball's bins per pair).
template <int D, int FINDER, int FORCE>
__device__ __forceinline__ void cell_general(const GridP& g, const ForceP& fp, const PassArgs& a, unsigned n, unsigned i,
                                          const float* xi, float2 pi, unsigned idi, Acc& acc) {
    if (FINDER == 1 || FINDER == 3) {
      int bc[3] = {0, 0, 0};
      if (FINDER == 1) bin_coords_mul<D>(g, xi, bc);
      else bin_coords_div<D>(g, xi, bc);
      // neighbour bins in the reference's task order (x fastest); each row of
      // bins along x is one contiguous range of the sorted arrays
      const int R = g.R;
      const int z0 = D >= 3 ? -R : 0, z1 = D >= 3 ? R : 0;
      for (int dz = z0; dz <= z1; ++dz) {
        const int cz = D >= 3 ? bc[2] + dz : 0;
        if (D >= 3 && (cz < 0 || cz >= g.ext[2])) continue;
        for (int dy = -R; dy <= R; ++dy) {
          const int cy = bc[1] + dy;
          if (cy < 0 || cy >= g.ext[1]) continue;
          const int x0 = max(bc[0] - R, 0), x1 = min(bc[0] + R, g.ext[0] - 1);
          int c0[3] = {x0, cy, cz}, c1[3] = {x1, cy, cz};
          const unsigned lo = a.off[flatten<D>(g, c0)], hi = a.off[flatten<D>(g, c1) + 1];
          for (unsigned j = lo; j < hi; ++j) {
            if (j == i) continue;
            visit<D, FINDER, FORCE>(g, fp, a, n, i, j, xi, pi, acc, idi);
          }
        }
      }
    } else if (FINDER == 5) {
      // the cell's Delaunay partners, ascending j, each applied reps times
      const unsigned m = a.dl_len[i];
      for (unsigned t = 0; t < m; ++t) {
        const uint2 e = a.dl_row[(size_t)i * kDlRow + t];
        visit<D, FINDER, FORCE>(g, fp, a, n, i, e.x, xi, pi, acc, idi, e.y);
      }
    } else {
      for (unsigned j = 0; j < n; ++j) {
        if (j == i) continue;
        visit<D, FINDER, FORCE>(g, fp, a, n, i, j, xi, pi, acc, idi);
      }
    }
}

// ---------------------------------------------------------------------------
// User pairwise laws: a PAIRWISE_FORCE lambda or functor compiled into the
// calling program (include/tecs/pairwise.cuh) takes pair_force's place in the
// general pass.  Candidate order, pair predicates, per-cell sums and the
// epilogues (COM, links, fused integrator modes, division) are those of
// k_pass, so a law written like a built-in one gives the built-in's bits.
// Law is a device callable adding the pair (self = i, other = j) to acc:
//   law(a, id_i, id_j, x_i, x_j (w = key or id), displacement x_i - x_j, distance, p_i, p_j, acc)
// with displacement[2] = 0 in 2-D and p = 0 without polarity.  With
// Law::kGeneric it also carries a per-cell (GENERIC_FORCE) law,
//   law.generic(a, id_i, x_i, p_i, g)
// adding to a zero g; the reference evaluates it before the pairwise forces
// (integrators/base.hpp:116-142, kernel_fuser.hpp:148-156), into the cleared
// stage buffer that the pair sums are then added to, so the cell's delta is
// 0 + (g + pair sum) -- the reference's ((0 + g) + pair sum) + 0 bit for bit.

template <int D, int FINDER, class Law>
__device__ __forceinline__ void visit_law(const GridP& g, const ForceP& fp, const PassArgs& a, unsigned n, unsigned i,
                                          unsigned j, const float* xi, float2 pi, Acc& acc,
                                          typename Law::Cell& dacc, unsigned idi, const Law& law,
                                          unsigned reps5 = 1u) {
  const float4 vj = a.X[j];
  float disp[3] = {xi[0] - vj.x, xi[1] - vj.y, D >= 3 ? xi[2] - vj.z : 0.f};
  float d2 = disp[0] * disp[0] + disp[1] * disp[1];
  if (D >= 3) d2 = d2 + disp[2] * disp[2];
  if (d2 >= fp.rc2) return;
  if (FINDER == 3 && gabriel_blocked<D>(g, fp, a.X, a.off, i, j, xi, disp, d2)) return;
  if (FINDER == 2 && gabriel_blocked_naive<D>(fp, a.X, n, i, j, xi, disp, d2)) return;
  // Delaunay: the law is called once per accepted simplex, in j order
  unsigned reps = FINDER == 5 ? reps5 : 1u;
  if (FINDER == 4 && (reps = a.dmult[(size_t)i * a.capacity + j]) == 0u) return;
  const unsigned idj = id_at(a.X, a.Bid, j);
  if (a.pairs) {
    const unsigned long long s = atomicAdd(&a.ctr->pair_count, (unsigned long long)reps);
    for (unsigned r = 0; r < reps; ++r)
      if (s + r < a.pair_cap) a.pairs[s + r] = make_uint2(idi, idj);
  }
  const float dist = sqrtf(d2);
  const float2 pj = a.P ? a.P[j] : make_float2(0.f, 0.f);
  for (unsigned r = 0; r < reps; ++r) law(a, idi, idj, j, xi, vj, disp, dist, pi, pj, acc, dacc);
}

// cell_general's loops with a user law
template <int D, int FINDER, class Law>
__device__ __forceinline__ void cell_law(const GridP& g, const ForceP& fp, const PassArgs& a, unsigned n, unsigned i,
                                         const float* xi, float2 pi, unsigned idi, Acc& acc,
                                         typename Law::Cell& dacc, const Law& law) {
  if (FINDER == 1 || FINDER == 3) {
    int bc[3] = {0, 0, 0};
    if (FINDER == 1) bin_coords_mul<D>(g, xi, bc);
    else bin_coords_div<D>(g, xi, bc);
    const int R = g.R;
    const int z0 = D >= 3 ? -R : 0, z1 = D >= 3 ? R : 0;
    for (int dz = z0; dz <= z1; ++dz) {
      const int cz = D >= 3 ? bc[2] + dz : 0;
      if (D >= 3 && (cz < 0 || cz >= g.ext[2])) continue;
      for (int dy = -R; dy <= R; ++dy) {
        const int cy = bc[1] + dy;
        if (cy < 0 || cy >= g.ext[1]) continue;
        const int x0 = max(bc[0] - R, 0), x1 = min(bc[0] + R, g.ext[0] - 1);
        int c0[3] = {x0, cy, cz}, c1[3] = {x1, cy, cz};
        const unsigned lo = a.off[flatten<D>(g, c0)], hi = a.off[flatten<D>(g, c1) + 1];
        for (unsigned j = lo; j < hi; ++j) {
          if (j == i) continue;
          visit_law<D, FINDER>(g, fp, a, n, i, j, xi, pi, acc, dacc, idi, law);
        }
      }
    }
  } else if (FINDER == 5) {
    const unsigned m = a.dl_len[i];
    for (unsigned t = 0; t < m; ++t) {
      const uint2 e = a.dl_row[(size_t)i * kDlRow + t];
      visit_law<D, FINDER>(g, fp, a, n, i, e.x, xi, pi, acc, dacc, idi, law, e.y);
    }
  } else {
    for (unsigned j = 0; j < n; ++j) {
      if (j == i) continue;
      visit_law<D, FINDER>(g, fp, a, n, i, j, xi, pi, acc, dacc, idi, law);
    }
  }
}

template <int D, int FINDER, class Law>
static __global__ void __launch_bounds__(kPassThreads) k_pass_law(GridP g, ForceP fp, PassArgs a,
                                                                  const Law* __restrict__ lawp) {
  const Law& law = *lawp;
  constexpr unsigned NE = Law::kExtra;
  const unsigned n = a.ctr->n;
  const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = i < n;
  Acc acc = {{0.f, 0.f, 0.f}, {0.f, 0.f}};
  typename Law::Cell cell;
  float xi[3] = {0.f, 0.f, 0.f};
  float4 vi = make_float4(0.f, 0.f, 0.f, 0.f);
  float2 pi = make_float2(0.f, 0.f);
  if (active) {
    vi = a.X[i];
    xi[0] = vi.x; xi[1] = vi.y; xi[2] = vi.z;
    if (a.P) pi = a.P[i];
    const unsigned idi = id_at(a.X, a.Bid, i);
    cell.drag = 0.f;
#pragma unroll
    for (int d = 0; d < 3; ++d) cell.v[d] = 0.f;
    if constexpr (NE > 0) {
#pragma unroll
      for (unsigned k = 0; k < NE; ++k) {
        cell.ex_self[k] = a.EX[k * (size_t)a.capacity + i];
        cell.ex_delta[k] = 0.f;
      }
    }
    cell_law<D, FINDER>(g, fp, a, n, i, xi, pi, idi, acc, cell, law);
    if constexpr (Law::kGeneric) {
      Acc gen = {{0.f, 0.f, 0.f}, {0.f, 0.f}};
      float gex[NE > 0 ? NE : 1] = {};
      law.generic(a, idi, xi, pi, gen, cell.ex_self, gex);
#pragma unroll
      for (int d = 0; d < 3; ++d) acc.x[d] = gen.x[d] + acc.x[d];
      acc.p[0] = gen.p[0] + acc.p[0];
      acc.p[1] = gen.p[1] + acc.p[1];
      if constexpr (NE > 0) {
#pragma unroll
        for (unsigned k = 0; k < NE; ++k) cell.ex_delta[k] = gex[k] + cell.ex_delta[k];
      }
    }
    // out(i) += total_velocity / fmax(total_drag, epsilon), after the pair
    // sums (binned_gabriel.hpp:356-357); with no drag this adds +0
    if constexpr (Law::kPairwise) {
      const float den = fmaxf(cell.drag, FLT_EPSILON);
#pragma unroll
      for (int d = 0; d < D; ++d) acc.x[d] = acc.x[d] + cell.v[d] / den;
    }
  }
  // a LINK_FORCE law evaluates the cell's links in place of the built-in pull
  if constexpr (NE > 0) {
    if constexpr (Law::kLink) pass_epilogue<D, Law, NE>(g, a, active, n, i, xi, vi, pi, acc, law, cell.ex_delta);
    else pass_epilogue<D, BuiltinLinks, NE>(g, a, active, n, i, xi, vi, pi, acc, BuiltinLinks{}, cell.ex_delta);
  } else {
    if constexpr (Law::kLink) pass_epilogue<D>(g, a, active, n, i, xi, vi, pi, acc, law);
    else pass_epilogue<D>(g, a, active, n, i, xi, vi, pi, acc);
  }
}

// One force evaluation handed to a user law's launcher (tecs_sim_set_pair_law).
// size is sizeof(UserPassCall) of the library that filled it: a program built
// against other headers is refused.
struct UserPassCall {
  unsigned size;
  int device;           // the simulation's GPU
  int dims;
  int finder;           // TECS_FINDER_NAIVE_ALL_PAIRS .. TECS_FINDER_DELAUNAY
  unsigned blocks;      // of kPassThreads threads
  GridP g;
  ForceP fp;
  PassArgs a;
};

// Launches the pass of one evaluation with the law, on the library's stream,
// for the finder and dimension count the program was compiled for.  0 on
// success; 1 the call's layout differs; 2 a launch error; 3 the simulation's
// finder or dimension count is not the program's.
// A program compiled for the naive Delaunay finder runs with the Delaunay
// finder of any capacity (FINDER 5) too: the library takes that one past the
// naive finder's capacity.
template <int D, int FINDER, class Law>
int launch_user_pass(const UserPassCall* c, cudaStream_t stream, const Law* law) {
  static_assert(FINDER >= 0 && FINDER <= 5, "user laws run with the all-pairs, Gabriel and Delaunay finders");
  if (!c || c->size != sizeof(UserPassCall)) return 1;
  const bool dl5 = FINDER == 4 && c->finder == 5;
  if (c->dims != D || (c->finder != FINDER && !dl5) || c->a.E != Law::kExtra) return 3;
  int cur = -1;
  if (cudaGetDevice(&cur) != cudaSuccess || (cur != c->device && cudaSetDevice(c->device) != cudaSuccess)) return 2;
  if (dl5) k_pass_law<D, 5, Law><<<c->blocks, kPassThreads, 0, stream>>>(c->g, c->fp, c->a, law);
  else k_pass_law<D, FINDER, Law><<<c->blocks, kPassThreads, 0, stream>>>(c->g, c->fp, c->a, law);
  return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

// Loads the law's pass on the device before the library first launches it,
// which may be while it captures a step graph: 0 on success.
template <int D, int FINDER, class Law>
int prepare_user_pass(int device) {
  cudaFuncAttributes fa;
  if (cudaSetDevice(device) != cudaSuccess) return 2;
  if (FINDER == 4 && cudaFuncGetAttributes(&fa, k_pass_law<D, 5, Law>) != cudaSuccess) return 2;
  return cudaFuncGetAttributes(&fa, k_pass_law<D, FINDER, Law>) == cudaSuccess ? 0 : 2;
}

// ---------------------------------------------------------------------------
// Warp-cooperative Gabriel pass (spring laws and the 3-D polarity law).
//
// Same pair semantics as gabriel_cell_fast, reorganised so that the lanes stay
// busy: (1) each thread collects its cell's in-cutoff neighbours into shared
// memory, in candidate order; (2) each warp lists every (cell, neighbour)
// pair of its 32 cells -- sorted by the cell's neighbour count, so the
// Gabriel loops of a round of pairs run the same length -- and its lanes take
// pairs round-robin for the Gabriel test, setting accept bits per cell; (3)
// the same for the pair forces, each written over its candidate slot; (4) each thread
// adds its cell's accepted contributions in candidate order -- the
// reference's summation order, so the sums stay bit-identical.  Cells with
// more neighbours than the slots, or whose witness ball leaves the 3x3x3 bin
// block, take the general path in phase 4.
// Candidate slot (q, cell c) in shared memory, XOR-swizzled so that threads
// reading different q of the same cell hit different banks.
__device__ __forceinline__ int cix(int q, int c) { return q * kPassThreads + (c ^ q); }

// FINDER 3: binned Gabriel; FINDER 1: binned all-pairs (i's bin by
// multiplication, binned_all_pairs.hpp:103-109, and every in-cutoff pair
// accepted: no phase 2).
// The grid pass: block blockIdx.x's cells.
template <int D, int FORCE, int FINDER = 3>
static __global__ void __launch_bounds__(kPassThreads) k_pass_gabriel(GridP g, ForceP fp, PassArgs a) {
#define TECS_PASS_BLOCK blockIdx.x
#include "pass_gabriel_body.inc"
#undef TECS_PASS_BLOCK
}

// One block's cells blk * kPassThreads .. (only warp-level synchronisation,
// so a kernel may run several blocks' cells one after another).
template <int D, int FORCE, int FINDER = 3>
__device__ __forceinline__ void pass_gabriel_block(const GridP& g, const ForceP& fp, const PassArgs& a,
                                                   const unsigned blk) {
#define TECS_PASS_BLOCK blk
#include "pass_gabriel_body.inc"
#undef TECS_PASS_BLOCK
}

// Symmetric finders (…_symmetric.hpp): only j with a smaller id, +delta to the
// evaluating cell and -delta to j for every field.  Float atomics: the
// accumulation order is not fixed, results agree to rounding.
template <int D, int FINDER, int FORCE>
static __global__ void __launch_bounds__(128) k_pass_sym(GridP g, ForceP fp, PassArgs a) {
  const unsigned n = a.ctr->n;
  const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 vi = a.X[i];
  const float xi[3] = {vi.x, vi.y, vi.z};
  const float2 pi = a.P ? a.P[i] : make_float2(0.f, 0.f);
  const unsigned idi = id_at(a.X, a.Bid, i);
  auto one = [&](unsigned j) {
    if (id_at(a.X, a.Bid, j) >= idi) return;
    Acc acc = {{0.f, 0.f, 0.f}, {0.f, 0.f}};
    const unsigned long long before = a.pairs ? 1ull : 0ull;
    (void)before;
    // pair (self = i, other = j)
    const float4 vj = a.X[j];
    float disp[3];
    disp[0] = xi[0] - vj.x;
    disp[1] = xi[1] - vj.y;
    disp[2] = D >= 3 ? xi[2] - vj.z : 0.f;
    float d2 = disp[0] * disp[0] + disp[1] * disp[1];
    if (D >= 3) d2 = d2 + disp[2] * disp[2];
    if (d2 >= fp.rc2) return;
    if (FINDER == 3 && gabriel_blocked<D>(g, fp, a.X, a.off, i, j, xi, disp, d2)) return;
    if (FINDER == 2 && gabriel_blocked_naive<D>(fp, a.X, n, i, j, xi, disp, d2)) return;
    if (a.pairs) {
      unsigned long long s = atomicAdd(&a.ctr->pair_count, 1ull);
      if (s < a.pair_cap) a.pairs[s] = make_uint2(idi, id_at(a.X, a.Bid, j));
    }
    const float dist = sqrtf(d2);
    const float2 pj = (FORCE == 2 && a.P) ? a.P[j] : make_float2(0.f, 0.f);
    pair_force<D, FORCE>(fp, disp, dist, pi, pj, acc);
    for (int d = 0; d < D; ++d) {
      atomicAdd(&((float*)&a.d_out[i])[d], acc.x[d]);
      atomicAdd(&((float*)&a.d_out[j])[d], -acc.x[d]);
    }
    if (a.dp_out) {
      atomicAdd(&a.dp_out[i].x, acc.p[0]); atomicAdd(&a.dp_out[i].y, acc.p[1]);
      atomicAdd(&a.dp_out[j].x, -acc.p[0]); atomicAdd(&a.dp_out[j].y, -acc.p[1]);
    }
  };
  if (FINDER == 1 || FINDER == 3) {
    int bc[3] = {0, 0, 0};
    bin_coords_div<D>(g, xi, bc);
    const int R = g.R;
    const int z0 = D >= 3 ? -R : 0, z1 = D >= 3 ? R : 0;
    for (int dz = z0; dz <= z1; ++dz) {
      const int cz = D >= 3 ? bc[2] + dz : 0;
      if (D >= 3 && (cz < 0 || cz >= g.ext[2])) continue;
      for (int dy = -R; dy <= R; ++dy) {
        const int cy = bc[1] + dy;
        if (cy < 0 || cy >= g.ext[1]) continue;
        const int x0 = max(bc[0] - R, 0), x1 = min(bc[0] + R, g.ext[0] - 1);
        int c0[3] = {x0, cy, cz}, c1[3] = {x1, cy, cz};
        const unsigned lo = a.off[flatten<D>(g, c0)], hi = a.off[flatten<D>(g, c1) + 1];
        for (unsigned j = lo; j < hi; ++j) one(j);
      }
    }
  } else {
    for (unsigned j = 0; j < n; ++j) one(j);
  }
}

// ---------------------------------------------------------------------------
// One Euler step of a small simulation in one cluster of kSmallCtas blocks
// (up to kSmallCells = 1536 cells and kSmallBins bins; the binned finders on
// the geometry of the cooperative pass, no COM fix, no division, no extra
// fields, built-in laws): the bin counts (made by the previous step's
// epilogue, or here), their scan, the scatter, the in-bin id order, then the
// pass -- what the rebuild kernels and the fused pass do over the grid, for a
// step whose launches would otherwise each cost more than their work.
// The phases are separated by cluster barriers (release/acquire at cluster
// scope); every block scans all the counts into its own shared memory, so the
// scan needs no barrier of its own; each block runs the cooperative pass
// (pass_gabriel_block) over blocks of cells blockIdx.x, + kSmallCtas, ...  The
// arithmetic is that of the passes over the grid, so runs are bit-identical.
// The cluster size is set at launch (16 blocks: past the portable 8, opted
// into per kernel).
constexpr int kSmallCtas = 16;
// one block of cells per block of the cluster: past that the blocks run
// their cells' blocks in turn, and the grid path spreads them over more SMs
constexpr unsigned kSmallCells = kSmallCtas * kPassThreads;
constexpr unsigned kSmallBins = 16384;
constexpr size_t kSmallSmem = (kSmallBins + 1) * sizeof(unsigned);

__device__ __forceinline__ void cluster_barrier() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

template <int D, int FINDER, int FORCE>
static __global__ void __launch_bounds__(kPassThreads)
    k_step_small(GridP g, ForceP fp, PassArgs p1, int run_count, const float4* A, const float2* PA, float4* B,
                 float2* PB, unsigned* Bid, unsigned* off, unsigned* src, unsigned part_words) {
  extern __shared__ unsigned offs[];  // the exclusive scan of the counts, nbins + 1 words
  __shared__ unsigned wsum[kPassThreads / 32];
  const unsigned n = p1.ctr->n, t = threadIdx.x;
  const unsigned g0 = blockIdx.x * kPassThreads + t, gs = kSmallCtas * kPassThreads;
  const int lane = t & 31, warp = t >> 5;
  const unsigned len = g.nbins + 1;
  // 1. bin counts of A (the previous step's epilogue made them unless run_count)
  if (run_count) {
    for (unsigned c = g0; c < n; c += gs) {
      const float4 v = A[c];
      const float q[3] = {v.x, v.y, v.z};
      int b3[3] = {0, 0, 0};
      bin_coords_div<D>(g, q, b3);
      const unsigned b = flatten<D>(g, b3);
      p1.key[c] = b;
      p1.rank[c] = atomicAdd(&p1.cnt[b], 1u);
    }
    cluster_barrier();
  }
  // 2. every block: the exclusive scan of all the counts (offs[nbins] = n);
  // block 0 also writes it to off for the pass; then the scatter of the
  // block's own cells
  {
    const unsigned per = (len + kPassThreads - 1) / kPassThreads;
    const unsigned b0 = min(len, t * per), b1 = min(len, b0 + per);
    unsigned sum = 0;
    for (unsigned b = b0; b < b1; ++b) sum += p1.cnt[b];
    unsigned incl = sum;
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    if (lane == 31) wsum[warp] = incl;
    __syncthreads();
    unsigned before = 0;
    for (int w = 0; w < warp; ++w) before += wsum[w];
    unsigned run = before + incl - sum;
    for (unsigned b = b0; b < b1; ++b) {
      const unsigned c = p1.cnt[b];
      offs[b] = run;
      if (blockIdx.x == 0) off[b] = run;
      run += c;
    }
  }
  __syncthreads();
  for (unsigned c = g0; c < n; c += gs) src[offs[p1.key[c]] + p1.rank[c]] = c;
  cluster_barrier();
  // 3. the counts cleared for the next step's epilogue (and chunk totals that
  // the counting formed on a sparse grid), each bin in ascending id
  // (k_order_gather)
  for (unsigned b = g0; b < len; b += gs) p1.cnt[b] = 0u;
  for (unsigned w = g0; w < part_words; w += gs) p1.part[w] = 0u;
  for (unsigned u = g0; u < n; u += gs) {
    const unsigned c = src[u], b = p1.key[c], lo = offs[b], hi = offs[b + 1];
    const float4 v = A[c];
    unsigned dst = u;
    if (hi - lo > 1u) {
      const unsigned me = id_of(v);
      unsigned r = 0;
      for (unsigned k = lo; k < hi; ++k) r += id_of(A[src[k]]) < me ? 1u : 0u;
      dst = lo + r;
    }
    B[dst] = make_float4(v.x, v.y, v.z, __uint_as_float(b));
    Bid[dst] = id_of(v);
    if (PB) PB[dst] = PA[c];
  }
  cluster_barrier();
  // 4. the Euler pass
  for (unsigned blk = blockIdx.x; blk * kPassThreads < n; blk += kSmallCtas)
    pass_gabriel_block<D, FORCE, FINDER>(g, fp, p1, blk);
}

// Plain COM reduction over a delta buffer (used after the symmetric pass).
static __global__ void k_com(const float4* __restrict__ d, PassArgs a) {
  const unsigned n = a.ctr->n;
  long long x = 0, y = 0, z = 0;
  for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float4 v = d[i];
    x += com_fixed(v.x); y += com_fixed(v.y); z += com_fixed(v.z);
  }
  com_reduce_block(a, x, y, z);
}

// ---------------------------------------------------------------------------
// integrator epilogues when the COM fix (or the symmetric finder) forbids
// fusing them into the pass

// heun.hpp:54-68: d1' = d1 - c1; x~ = x + d1' * dt (every field).  d1' is not
// stored: the corrector forms it again with the same operations.
static __global__ void k_predict(const Counters* __restrict__ ctr, const float* __restrict__ com, float dt,
                          const float4* __restrict__ B, const float2* __restrict__ PB, const float4* __restrict__ d1,
                          const float2* __restrict__ dp1, float4* __restrict__ Xt, float2* __restrict__ Pt,
                          PassArgs ex) {
  const unsigned n = ctr->n;
  const float c0 = com[0], c1 = com[1], c2 = com[2];
  for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    // the extra fields' predictor: x~ = x + d1 * dt (no COM fix: it acts on
    // the first field only)
    for (unsigned k = 0; k < ex.E; ++k) {
      const size_t at = k * (size_t)ex.capacity + i;
      ex.Et[at] = ex_update(ex.EBx[at], ex.ed1[at], dt, ex.dt64, (ex.ex_dbl >> k) & 1u);
    }
    float4 v = d1[i];
    v.x = v.x - c0; v.y = v.y - c1; v.z = v.z - c2;  // d1 - c1 (re-formed by k_finish)
    const float4 x = B[i];
    Xt[i] = make_float4(x.x + v.x * dt, x.y + v.y * dt, x.z + v.z * dt, x.w);
    if (Pt) {
      const float2 p = PB[i], q = dp1[i];
      Pt[i] = make_float2(p.x + q.x * dt, p.y + q.y * dt);
    }
  }
}

// heun.hpp:78-98 (corrector) and euler.hpp:49-69 with the COM subtraction,
// the old velocities when the simulation keeps them, plus division.  Heun: s = d1 + (d2 - c); x += (s * 0.5) * dt.
// Euler:  s = d1 - c; x += s * dt.
template <int D>
static __global__ void k_finish(int heun, GridP g, PassArgs a, const float* __restrict__ com, const float4* __restrict__ d2,
                         const float2* __restrict__ dp2) {
  const unsigned n = a.ctr->n;
  // Euler: com = c (slot 0).  Heun: com = c1 (slot 0), com + 4 = c2 (slot 1)
  const float c0 = com[heun ? 4 : 0], c1 = com[heun ? 5 : 1], c2 = com[heun ? 6 : 2];
  const float p0 = com[0], p1 = com[1], p2 = com[2];
  const float dt = a.dt;
  const unsigned long long step = a.ctr->step;
  for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float4 xb = a.Bx[i];
    const float4 v1 = a.d1[i];
    float xn[3];
    float2 pn = make_float2(0.f, 0.f);
    if (heun) {
      const float4 v2 = d2[i];
      const float f0 = v1.x - p0, f1 = v1.y - p1, f2 = v1.z - p2;  // d1 - c1 (predictor)
      const float e0 = v2.x - c0, e1 = v2.y - c1, e2 = v2.z - c2;  // d2 - c2 (corrector)
      const float h0 = f0 + e0, h1 = f1 + e1, h2 = f2 + e2;
      xn[0] = xb.x + (h0 * 0.5f) * dt; xn[1] = xb.y + (h1 * 0.5f) * dt; xn[2] = xb.z + (h2 * 0.5f) * dt;
      // old_velocities(i) = (d1' + d2') * 0.5 (heun.hpp:87)
      if (a.old_vel) a.old_vel[a.Bid ? a.Bid[i] : id_of(xb)] = make_float4(h0 * 0.5f, h1 * 0.5f, h2 * 0.5f, 0.f);
      if (a.PA) {
        const float2 pb = a.Bp[i], q1 = a.dp1[i], q2 = dp2[i];
        const float g0 = q1.x + q2.x, g1 = q1.y + q2.y;
        pn = make_float2(pb.x + (g0 * 0.5f) * dt, pb.y + (g1 * 0.5f) * dt);
      }
    } else {
      const float e0 = v1.x - c0, e1 = v1.y - c1, e2 = v1.z - c2;
      xn[0] = xb.x + e0 * dt; xn[1] = xb.y + e1 * dt; xn[2] = xb.z + e2 * dt;
      // old_velocities(i) = d1' (euler.hpp:59)
      if (a.old_vel) a.old_vel[a.Bid ? a.Bid[i] : id_of(xb)] = make_float4(e0, e1, e2, 0.f);
      if (a.PA) {
        const float2 pb = a.Bp[i], q1 = a.dp1[i];
        pn = make_float2(pb.x + q1.x * dt, pb.y + q1.y * dt);
      }
    }
    if (D < 3) xn[2] = 0.f;
    const unsigned idb = a.Bid ? a.Bid[i] : id_of(xb);
    a.A[i] = make_float4(xn[0], xn[1], xn[2], __uint_as_float(idb));
    if (a.PA) a.PA[i] = pn;
    // the extra fields: Euler x + d1 dt, Heun x + (d1 + d2) * 0.5 * dt
    for (unsigned k = 0; k < a.E; ++k) {
      const size_t at = k * (size_t)a.capacity + i;
      const bool dbl = (a.ex_dbl >> k) & 1u;
      const float xe = a.EBx[at];
      if (heun) {
        const float h = a.ed1[at] + a.ed2[at];
        a.EA[at] = dbl ? (float)((double)xe + ((double)h * 0.5) * a.dt64) : xe + (h * 0.5f) * dt;
      } else {
        a.EA[at] = ex_update(xe, a.ed1[at], dt, a.dt64, dbl);
      }
    }
    if (a.count_next) count_cell<D>(g, a, i, xn);
    maybe_divide<D>(g, a, n, idb, xn, pn, step, i);
  }
}

}  // namespace tecs
