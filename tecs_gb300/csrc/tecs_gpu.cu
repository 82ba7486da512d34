// tecs_gpu.cu -- C ABI of the GB300 cell-step library (include/tecs_gpu.h).
//
// One tecs_sim owns the device state of one simulation and a CUDA stream.
// tecs_sim_step queues one integrator step as a fixed kernel sequence:
//
//   rebuild   [k_count] -> k_scan_reduce -> k_scan_apply -> k_scatter -> k_order_gather
//             (k_count is fused into the previous step's state write when every
//              step rebuilds)
//   Euler     k_pass(kEulerFused)                                   [no COM]
//             k_pass(kStore + COM) -> k_finish                      [COM]
//   Heun      k_pass(kHeun1Fused) -> k_pass(kHeun2Fused)            [no COM]
//             k_pass(kStore + COM) -> k_predict -> k_pass(kStore + COM) -> k_finish
//   division  k_divide_commit
//
// and, by default, captures that sequence once as a CUDA graph and replays it.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstddef>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/tecs_gpu.h"
#include "../../include/tecs/device/kernels.cuh"

using namespace tecs;

namespace {
thread_local std::string g_last_error;

int fail(const std::string& m) {
  g_last_error = m;
  return -1;
}
#define CK(call)                                                                              \
  do {                                                                                        \
    cudaError_t e_ = (call);                                                                  \
    if (e_ != cudaSuccess) return fail(std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

unsigned ceil_div(unsigned long long a, unsigned b) { return (unsigned)((a + b - 1) / b); }
}  // namespace

// shared with engine.cu: the thread's last error message
namespace tecs {
int set_last_error(const std::string& m) { return fail(m); }
}  // namespace tecs

namespace {

// pack AoS float[n][dims] into float4 (x, y, z, id)
__global__ void k_pack(const float* __restrict__ in, unsigned n, int dims, float4* __restrict__ A) {
  for (unsigned s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
    float4 v = make_float4(0.f, 0.f, 0.f, __uint_as_float(s));
    v.x = in[(size_t)s * dims];
    if (dims >= 2) v.y = in[(size_t)s * dims + 1];
    if (dims >= 3) v.z = in[(size_t)s * dims + 2];
    A[s] = v;
  }
}
// id -> slot map of the sorted copy, from its slot -> id array
__global__ void k_slot_map(const Counters* __restrict__ ctr, const unsigned* __restrict__ Bid, unsigned capacity,
                           unsigned* __restrict__ slot_of) {
  const unsigned n = ctr->n;
  for (unsigned s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
    const unsigned id = Bid[s];
    if (id < capacity) slot_of[id] = s;
  }
}

// scatter slot-ordered float4 values into cell-id order AoS float[n][dims]
__global__ void k_unpack(const float4* __restrict__ idw, const unsigned* __restrict__ ids,
                         const float4* __restrict__ val, unsigned n, int dims, float* __restrict__ out) {
  for (unsigned s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
    const unsigned id = ids ? ids[s] : id_of(idw[s]);
    const float4 v = val[s];
    out[(size_t)id * dims] = v.x;
    if (dims >= 2) out[(size_t)id * dims + 1] = v.y;
    if (dims >= 3) out[(size_t)id * dims + 2] = v.z;
  }
}
__global__ void k_unpack2(const float4* __restrict__ idw, const unsigned* __restrict__ ids,
                          const float2* __restrict__ val, unsigned n, float2* __restrict__ out) {
  for (unsigned s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x)
    out[ids ? ids[s] : id_of(idw[s])] = val[s];
}

// The upload of a state in one pass: positions packed as (x, y, z, id) and
// polarities copied -- read straight from the caller's page-locked host
// buffers when they are mapped (on GB300 a kernel reaches host memory over
// NVLink-C2C at the link's rate, so no staging copy is needed) -- the
// counters reset (all but the step index, which keys the division stream),
// and, when the first rebuild expects them, the cells counted per bin.
__global__ void k_upload(const float* __restrict__ pos, const float2* __restrict__ pol, unsigned n, int dims,
                         float4* __restrict__ A, float2* __restrict__ PA, Counters* __restrict__ ctr, GridP g,
                         unsigned* __restrict__ key, unsigned* __restrict__ rank, unsigned* __restrict__ cnt,
                         unsigned* __restrict__ part) {
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    ctr->n = n;
    ctr->div_count = 0u;
    ctr->done[0] = ctr->done[1] = 0u;
    ctr->error = 0u;
    ctr->done_div = 0u;
    ctr->pair_count = 0ull;
  }
  for (unsigned s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
    float4 v = make_float4(0.f, 0.f, 0.f, __uint_as_float(s));
    v.x = pos[(size_t)s * dims];
    if (dims >= 2) v.y = pos[(size_t)s * dims + 1];
    if (dims >= 3) v.z = pos[(size_t)s * dims + 2];
    A[s] = v;
    if (pol) PA[s] = pol[s];
    if (cnt) {
      float p[3] = {v.x, v.y, v.z};
      int c[3] = {0, 0, 0};
      unsigned b;
      if (dims == 3) { bin_coords_div<3>(g, p, c); b = flatten<3>(g, c); }
      else { bin_coords_div<2>(g, p, c); b = flatten<2>(g, c); }
      key[s] = b;
      rank[s] = count_bin(cnt, part, b);
    }
  }
}

// download helpers that take the agent count from the device counters, so
// that a download needs no host round trip before its copies
__global__ void k_unpack_dev(const float4* __restrict__ A, const Counters* __restrict__ ctr, int dims,
                             float* __restrict__ out) {
  const unsigned n = ctr->n;
  for (unsigned s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
    const float4 v = A[s];
    const size_t o = (size_t)id_of(v) * dims;
    out[o] = v.x;
    if (dims >= 2) out[o + 1] = v.y;
    if (dims >= 3) out[o + 2] = v.z;
  }
}
__global__ void k_unpack2_dev(const float4* __restrict__ A, const Counters* __restrict__ ctr,
                              const float2* __restrict__ val, float2* __restrict__ out) {
  const unsigned n = ctr->n;
  for (unsigned s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x)
    out[id_of(A[s])] = val[s];
}
// copy the first n * per floats of src to dst (a mapped host buffer), four at
// a time when dst is 16-byte aligned
__global__ void k_copy_out(const float* __restrict__ src, const Counters* __restrict__ ctr, unsigned per,
                           float* __restrict__ dst) {
  const size_t total = (size_t)ctr->n * per;
  const size_t stride = (size_t)gridDim.x * blockDim.x, t0 = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  size_t done = 0;
  if ((reinterpret_cast<uintptr_t>(dst) & 15u) == 0) {
    const size_t q = total / 4;
    for (size_t k = t0; k < q; k += stride)
      reinterpret_cast<float4*>(dst)[k] = reinterpret_cast<const float4*>(src)[k];
    done = q * 4;
  }
  for (size_t k = done + t0; k < total; k += stride) dst[k] = src[k];
}

// The device address of a page-locked host buffer mapped into the device's
// address space, or null for any other pointer.
const void* mapped_host(const void* p) {
  if (!p) return nullptr;
  cudaPointerAttributes at{};
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}
}  // namespace

struct tecs_sim {
  tecs_sim_desc d{};
  GridP g{};
  ForceP fp{};
  cudaStream_t stream = nullptr;
  bool binned = false;
  float4 *A = nullptr, *B = nullptr, *Xt = nullptr, *d1 = nullptr, *d2 = nullptr;
  float2 *PA = nullptr, *PB = nullptr, *Pt = nullptr, *dp1 = nullptr, *dp2 = nullptr;
  unsigned *key = nullptr, *rank = nullptr, *src = nullptr, *cnt = nullptr, *off = nullptr, *part = nullptr;
  unsigned *div_parent = nullptr, *div_slot = nullptr;
  unsigned* Bid = nullptr;  // cell ids of B's slots (B.w holds the bin key)
  unsigned short* dmult = nullptr;  // naive Delaunay: applications per directed pair, capacity x capacity
  // Delaunay of any capacity: the pass's bin grid (state, counts, offsets,
  // sorted slots and positions) and each cell's partner row
  DlState* dl_st = nullptr;
  unsigned *dl_cnt = nullptr, *dl_off = nullptr, *dl_idx = nullptr, *dl_len = nullptr;
  float4* dl_sp = nullptr;
  uint2* dl_row = nullptr;
  unsigned dl_maxbins = 0;
  // links: per-cell entries in link order, and the id -> slot map of the sorted copy
  unsigned* link_off = nullptr;
  uint2* link_ent = nullptr;
  unsigned* slot_of = nullptr;
  // the integrator's old velocities by cell id (float4, capacity), when kept
  float4* ov = nullptr;
  // extra fields: E components per cell, component-major ([k * capacity +
  // slot]); EA in A's slot order, EB in B's, Et the predictor, ed1 / ed2 the
  // passes' deltas; ex_dbl marks the components of Scalar fields
  unsigned E = 0, ex_dbl = 0;
  float *EA = nullptr, *EB = nullptr, *Et = nullptr, *ed1 = nullptr, *ed2 = nullptr;
  unsigned n_links = 0;
  float link_k = 0.f;
  // B and Bid hold a sort of the current cells (false from an upload until the
  // next rebuild, which the first step after an upload always does)
  bool sorted = false;
  Counters* ctr = nullptr;
  double* com_part = nullptr;
  float* com = nullptr;  // [0..2] pass 1, [4..6] pass 2
  float* stage = nullptr;
  unsigned n_host = 0;
  int step_count = 0;
  bool use_graph = true;
  cudaGraphExec_t gexec[2] = {nullptr, nullptr};
  double gdt[2] = {0.0, 0.0};
  int kernels[2] = {0, 0};
  int last_kernels = 0;
  // the next rebuild's bin count is done by the state-writing kernel
  bool fuse_count = false;
  bool small_ok = true;  // small steps may take k_step_small (TECS_NO_SMALL_STEP=1: never)
  // sparse grids (bins > 4 x capacity): the counting also forms the scan's
  // chunk totals, and the rebuild needs no reduction pass over the bins
  bool fuse_part = false;
  Counters* hctr = nullptr;  // page-locked mirror of the device counters
  // a user pairwise law compiled into the calling program: launches each force pass in place of pass_fn's
  tecs_pair_law_fn law_fn = nullptr;
  void* law_user = nullptr;
  // per-kernel CUDA events (external event-record nodes when captured in a graph)
  bool profiling = false;
  static constexpr int kMaxProf = 32;
  cudaEvent_t ev[2 * kMaxProf] = {};
  const char* prof_name[kMaxProf] = {};
  int prof_n = 0;       // kernels marked while queueing the current step
  int prof_last = 0;    // kernels marked in the step that was last queued
};

namespace {

unsigned launch_count(const tecs_sim* s) {
  return s->d.division_probability > 0.0 ? s->d.capacity : s->n_host;
}

using PassFn = void (*)(GridP, ForceP, PassArgs);

thread_local bool g_capturing = false;

int prof_mark(tecs_sim* s, int which, const char* name) {
  if (!s->profiling) return 0;
  const int k = s->prof_n;
  if (k >= tecs_sim::kMaxProf) return 0;
  cudaEvent_t& e = s->ev[2 * k + which];
  if (!e) CK(cudaEventCreate(&e));
  if (g_capturing) CK(cudaEventRecordWithFlags(e, s->stream, cudaEventRecordExternal));
  else CK(cudaEventRecord(e, s->stream));
  if (which == 1) {
    s->prof_name[k] = name;
    s->prof_n = k + 1;
  }
  return 0;
}
#define PROF_BEGIN(s) \
  if (prof_mark((s), 0, nullptr)) return -1
#define PROF_END(s, name) \
  if (prof_mark((s), 1, (name))) return -1


// The cooperative Gabriel pass needs the fast-path geometry and packs bin
// coordinates in 10 bits and slots in 27 bits.
bool coop_geometry(const tecs_sim* s) {
  return s->g.R == 1 && s->g.bin_size >= s->d.cutoff && s->g.ext[0] <= 1024 && s->g.ext[1] <= 1024 &&
         s->g.ext[2] <= 1024 && s->d.capacity < (1u << 27);
}
// The built-in binned pass over the grid is the cooperative one
// (k_pass_gabriel): all-pairs on its geometry, Gabriel also with c <= 0.9.
bool coop_pass(const tecs_sim* s) {
  const bool geom = coop_geometry(s);
  if (s->d.finder == TECS_FINDER_BINNED_ALL_PAIRS) return geom;
  return s->d.finder == TECS_FINDER_BINNED_GABRIEL && geom && s->d.gabriel_coefficient <= 0.9f;
}

PassFn pass_fn(const tecs_sim* s, bool sym) {
  const int D = s->d.dims, F = s->d.finder, FO = s->d.force;
  const bool coop_geom = coop_geometry(s);
  const bool coop = coop_geom && s->d.gabriel_coefficient <= 0.9f;
#define PICK(DD, FF)                                                            \
  if (D == DD && F == FF) {                                                     \
    if (sym) {                                                                  \
      if (FO == 0) return k_pass_sym<DD, FF, 0>;                                \
      if (FO == 1) return k_pass_sym<DD, FF, 1>;                                \
      if (DD == 3) return k_pass_sym<DD, FF, 2>;                                \
    } else {                                                                    \
      if (FF == 3 && coop && FO == 0) return k_pass_gabriel<DD, 0>;             \
      if (FF == 3 && coop && FO == 1) return k_pass_gabriel<DD, 1>;             \
      if (FF == 3 && coop && FO == 2 && DD == 3) return k_pass_gabriel<3, 2>;   \
      if (FF == 1 && coop_geom && FO == 0) return k_pass_gabriel<DD, 0, 1>;     \
      if (FF == 1 && coop_geom && FO == 1) return k_pass_gabriel<DD, 1, 1>;     \
      if (FF == 1 && coop_geom && FO == 2 && DD == 3) return k_pass_gabriel<3, 2, 1>; \
      if (FO == 0) return k_pass<DD, FF, 0>;                                    \
      if (FO == 1) return k_pass<DD, FF, 1>;                                    \
      if (DD == 3) return k_pass<DD, FF, 2>;                                    \
    }                                                                           \
  }
  PICK(3, 0) PICK(3, 1) PICK(3, 2) PICK(3, 3) PICK(2, 0) PICK(2, 1) PICK(2, 2) PICK(2, 3)
#undef PICK
  if (F == TECS_FINDER_NAIVE_DELAUNAY && !sym) {
    if (D == 3 && FO == 0) return k_pass<3, 4, 0>;
    if (D == 3 && FO == 1) return k_pass<3, 4, 1>;
    if (D == 3 && FO == 2) return k_pass<3, 4, 2>;
    if (D == 2 && FO == 0) return k_pass<2, 4, 0>;
    if (D == 2 && FO == 1) return k_pass<2, 4, 1>;
  }
  if (F == TECS_FINDER_DELAUNAY && !sym) {
    if (D == 3 && FO == 0) return k_pass<3, 5, 0>;
    if (D == 3 && FO == 1) return k_pass<3, 5, 1>;
    if (D == 3 && FO == 2) return k_pass<3, 5, 2>;
    if (D == 2 && FO == 0) return k_pass<2, 5, 0>;
    if (D == 2 && FO == 1) return k_pass<2, 5, 1>;
  }
  return nullptr;
}


// the extra fields moved with A -> B
ExtraMove extra_move(const tecs_sim* s) { return ExtraMove{s->E, (size_t)s->d.capacity, s->EA, s->EB}; }

PassArgs base_args(const tecs_sim* s, float dt, double dt64 = 0.0) {
  PassArgs a{};
  a.off = s->off;
  a.ctr = s->ctr;
  a.dt = dt;
  a.capacity = s->d.capacity;
  a.div_enabled = s->d.division_probability > 0.0 ? 1 : 0;
  {
    const double p = s->d.division_probability;
    a.div_thresh = p >= 1.0 ? ~0ull : (p > 0.0 ? (unsigned long long)std::floor(p * 9007199254740992.0) : 0ull);
  }
  a.div_offset = s->d.division_offset;
  a.seed = s->d.seed;
  a.div_parent = s->div_parent;
  a.div_slot = s->div_slot;
  a.A = s->A;
  a.PA = s->d.has_polarity ? s->PA : nullptr;
  // the fast Gabriel path needs every witness inside i's cutoff ball and 3x3x3 bin block
  a.gabriel_fast = (s->d.gabriel_coefficient <= 0.9f && s->g.R == 1 && s->g.bin_size >= s->d.cutoff) ? 1 : 0;
  a.count_next = s->fuse_count ? 1 : 0;
  a.Bid = s->binned ? s->Bid : nullptr;
  a.key = s->key;
  a.rank = s->rank;
  a.cnt = s->cnt;
  a.part = s->fuse_part ? s->part : nullptr;
  a.dmult = s->dmult;
  a.dl_row = s->dl_row;
  a.dl_len = s->dl_len;
  a.link_off = s->n_links ? s->link_off : nullptr;
  a.link_ent = s->n_links ? s->link_ent : nullptr;
  a.slot_of = (s->n_links && s->binned) ? s->slot_of : nullptr;
  a.link_k = s->link_k;
  a.full_step = 1;
  a.old_vel = s->ov;
  a.dt64 = dt64;
  a.E = s->E;
  a.ex_dbl = s->ex_dbl;
  a.EA = s->EA;
  return a;
}

// Rebuild B (working copy) from A: bins sorted by (bin, id), or id order for naive finders.
// With run_count false the bin counts of A were already made by the kernel that wrote A.
int enqueue_rebuild(tecs_sim* s, int& K, bool run_count) {
  const unsigned L = launch_count(s);
  const unsigned gb = ceil_div(L ? L : 1, 256);
  float2* PA = s->d.has_polarity ? s->PA : nullptr;
  float2* PB = s->d.has_polarity ? s->PB : nullptr;
  if (s->binned) {
    const unsigned len = s->g.nbins + 1;
    const unsigned chunks = ceil_div(len, kScanChunk);
    const unsigned pw = (unsigned)scan_part_words(len);
    unsigned* part = s->fuse_part ? s->part : nullptr;
    if (run_count) {
      PROF_BEGIN(s);
      if (part) CK(cudaMemsetAsync(part, 0, (size_t)pw * 4, s->stream));
      k_count<<<gb, 256, 0, s->stream>>>(s->A, s->ctr, s->g, s->d.dims, s->key, s->rank, s->cnt, part);
      PROF_END(s, "k_count");
      K += 1;
    }
    if (part) {
      // sparse grid: the counting formed the chunk totals (count_bin); the
      // super-chunk totals are needed past kScanSuper chunks only
      if (chunks > kScanSuper) {
        PROF_BEGIN(s);
        k_scan_super<<<ceil_div(chunks, kScanSuper), kScanThreads, 0, s->stream>>>(part, chunks);
        PROF_END(s, "k_scan_super");
        K += 1;
      }
    } else if (chunks > 1) {
      // one chunk: its prefix needs no partial sums
      PROF_BEGIN(s);
      CK(cudaMemsetAsync(s->part + chunks, 0, (pw - chunks) * 4, s->stream));
      k_scan_reduce<<<chunks, kScanThreads, 0, s->stream>>>(s->cnt, len, s->part);
      PROF_END(s, "k_scan_reduce");
      K += 1;
    }
    PROF_BEGIN(s);
    k_scan_apply<<<chunks, kScanThreads, 0, s->stream>>>(s->cnt, len, s->part, s->off);
    PROF_END(s, "k_scan_apply");
    PROF_BEGIN(s);
    k_scatter<<<gb, 256, 0, s->stream>>>(s->ctr, s->key, s->rank, s->off, s->src, s->part, part ? pw : 0u);
    PROF_END(s, "k_scatter");
    PROF_BEGIN(s);
    k_order_gather<<<gb, 256, 0, s->stream>>>(s->ctr, s->key, s->off, s->src, s->A, PA, s->B, PB, s->Bid,
                                              s->n_links ? s->slot_of : nullptr, extra_move(s));
    PROF_END(s, "k_order_gather");
    K += 3;
  } else {
    PROF_BEGIN(s);
    k_id_scatter<<<gb, 256, 0, s->stream>>>(s->ctr, s->A, PA, s->B, PB, extra_move(s));
    PROF_END(s, "k_id_scatter");
    K += 1;
  }
  CK(cudaGetLastError());
  return 0;
}

// The Delaunay finder of any capacity: bin grid of the pass's positions, then
// every cell's partner row.
int enqueue_delaunay_star(tecs_sim* s, const PassArgs& a, int& K) {
  const unsigned L = launch_count(s);
  const unsigned gb = ceil_div(L ? L : 1, 256);
  const bool d3 = s->d.dims == 3;
  PROF_BEGIN(s);
  CK(cudaMemsetAsync(s->dl_cnt, 0, (size_t)s->dl_maxbins * 4, s->stream));
  k_dl_reset<<<1, 32, 0, s->stream>>>(s->dl_st);
  if (d3) k_dl_bounds<3><<<std::min(gb, 1216u), 256, 0, s->stream>>>(a.X, s->ctr, s->dl_st);
  else k_dl_bounds<2><<<std::min(gb, 1216u), 256, 0, s->stream>>>(a.X, s->ctr, s->dl_st);
  if (d3) k_dl_plan<3><<<1, 32, 0, s->stream>>>(s->ctr, s->dl_maxbins, s->dl_st);
  else k_dl_plan<2><<<1, 32, 0, s->stream>>>(s->ctr, s->dl_maxbins, s->dl_st);
  if (d3) k_dl_count<3><<<gb, 256, 0, s->stream>>>(a.X, s->ctr, s->dl_st, s->dl_cnt);
  else k_dl_count<2><<<gb, 256, 0, s->stream>>>(a.X, s->ctr, s->dl_st, s->dl_cnt);
  k_dl_scan<<<1, 1024, 0, s->stream>>>(s->dl_st, s->dl_cnt, s->dl_off);
  if (d3) k_dl_scatter<3><<<gb, 256, 0, s->stream>>>(a.X, s->ctr, s->dl_st, s->dl_cnt, s->dl_off, s->dl_idx, s->dl_sp);
  else k_dl_scatter<2><<<gb, 256, 0, s->stream>>>(a.X, s->ctr, s->dl_st, s->dl_cnt, s->dl_off, s->dl_idx, s->dl_sp);
  PROF_END(s, "k_dl_grid");
  K += 6;
  const unsigned mb = ceil_div(L ? L : 1, kDlThreads / 32);  // one warp per cell
  PROF_BEGIN(s);
  if (d3) k_dl_mult<3><<<mb, kDlThreads, 0, s->stream>>>(a.X, s->ctr, s->dl_st, s->dl_off, s->dl_idx, s->dl_sp,
                                                         s->fp.rc2, s->dl_row, s->dl_len);
  else k_dl_mult<2><<<mb, kDlThreads, 0, s->stream>>>(a.X, s->ctr, s->dl_st, s->dl_off, s->dl_idx, s->dl_sp,
                                                      s->fp.rc2, s->dl_row, s->dl_len);
  PROF_END(s, "k_dl_mult");
  K += 1;
  CK(cudaGetLastError());
  return 0;
}

int enqueue_delaunay_mult(tecs_sim* s, const PassArgs& a, int& K) {
  if (s->d.finder == TECS_FINDER_DELAUNAY) return enqueue_delaunay_star(s, a, K);
  const unsigned L = launch_count(s);
  // applications per pair on this pass's positions, before the pass
  PROF_BEGIN(s);
  if (s->d.dims == 3) k_delaunay_mult<3><<<L ? L : 1, kDelaunayThreads, 0, s->stream>>>(a.X, s->ctr, s->fp.rc2,
                                                                                       s->d.capacity, s->dmult);
  else k_delaunay_mult<2><<<L ? L : 1, kDelaunayThreads, 0, s->stream>>>(a.X, s->ctr, s->fp.rc2, s->d.capacity,
                                                                           s->dmult);
  PROF_END(s, "k_delaunay_mult");
  K += 1;
  return 0;
}

int enqueue_pass(tecs_sim* s, PassArgs a, int& K) {
  const bool sym = s->d.symmetric != 0;
  const unsigned L = launch_count(s);
  const unsigned blocks = ceil_div(L ? L : 1, kPassThreads);
  if (s->law_fn) {
    if (s->d.finder >= TECS_FINDER_NAIVE_DELAUNAY && enqueue_delaunay_mult(s, a, K)) return -1;
    UserPassCall c{};
    c.size = sizeof(UserPassCall);
    c.device = s->d.device;
    c.dims = s->d.dims;
    c.finder = s->d.finder;
    c.blocks = blocks;
    c.g = s->g;
    c.fp = s->fp;
    c.a = a;
    PROF_BEGIN(s);
    const int r = s->law_fn(s->law_user, &c, s->stream);
    PROF_END(s, "k_pass_law");
    K += 1;
    if (r) return fail("the user pairwise law's launcher failed (code " + std::to_string(r) + ")");
    CK(cudaGetLastError());
    return 0;
  }
  const PassFn fn = pass_fn(s, sym);
  if (!fn) return fail("unsupported finder/force/dims combination");
  if (s->d.finder >= TECS_FINDER_NAIVE_DELAUNAY && enqueue_delaunay_mult(s, a, K)) return -1;
  PROF_BEGIN(s);
  fn<<<ceil_div(L ? L : 1, kPassThreads), kPassThreads, 0, s->stream>>>(s->g, s->fp, a);
  PROF_END(s, a.mode == kStore ? "k_pass_store" : a.mode == kEulerFused ? "k_pass_euler"
              : a.mode == kHeun1Fused ? "k_pass_heun1" : "k_pass_heun2");
  K += 1;
  CK(cudaGetLastError());
  return 0;
}

// One integrator step (plus division), queued on the stream.
// A step small enough for one cluster (k_step_small): Euler, binned,
// non-symmetric, built-in laws, no COM fix, no division, no links, no extra
// fields, no old velocities.  (Heun's two passes in one cluster, with a
// barrier between them, were slower than over the grid.)
bool small_step_ok(const tecs_sim* s) {
  return s->d.integrator == TECS_EULER && s->binned && !s->d.symmetric && !s->d.com_fix && s->d.division_probability <= 0.0 && !s->n_links &&
         !s->E && !s->ov && !s->law_fn && s->small_ok && s->d.capacity <= kSmallCells && s->g.nbins <= kSmallBins &&
         coop_pass(s);
}

using SmallFn = void (*)(GridP, ForceP, PassArgs, int, const float4*, const float2*, float4*, float2*, unsigned*,
                         unsigned*, unsigned*, unsigned);

SmallFn small_fn_of(const tecs_sim* s) {
  const int D = s->d.dims, F = s->d.finder, FO = s->d.force;
  if (F != TECS_FINDER_BINNED_ALL_PAIRS && F != TECS_FINDER_BINNED_GABRIEL) return nullptr;
  const bool gab = F == TECS_FINDER_BINNED_GABRIEL;
  if (D == 3) {
    if (FO == 0) return gab ? k_step_small<3, 3, 0> : k_step_small<3, 1, 0>;
    if (FO == 1) return gab ? k_step_small<3, 3, 1> : k_step_small<3, 1, 1>;
    if (FO == 2) return gab ? k_step_small<3, 3, 2> : k_step_small<3, 1, 2>;
  } else {
    if (FO == 0) return gab ? k_step_small<2, 3, 0> : k_step_small<2, 1, 0>;
    if (FO == 1) return gab ? k_step_small<2, 3, 1> : k_step_small<2, 1, 1>;
  }
  return nullptr;
}

// Every instantiation of the kernel (the force may change after creation,
// tecs_sim_set_force), allowed a cluster of kSmallCtas blocks (past the
// portable 8) and shared memory for the scan of up to kSmallBins + 1 counts
// past the default 48 KB; set once per device, at the first creation, outside
// any stream capture.  False if such a cluster cannot be placed on the GPU
// (steps then run over the grid).
bool small_prepare_one(SmallFn fn) {
  if (cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess ||
      cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmallSmem) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = kSmallCtas;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.gridDim = dim3(kSmallCtas);
  cfg.blockDim = dim3(kPassThreads);
  cfg.dynamicSmemBytes = kSmallSmem;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  int clusters = 0;
  if (cudaOccupancyMaxActiveClusters(&clusters, fn, &cfg) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return clusters >= 1;
}

constexpr int kMaxDevices = 64;

bool small_prepare(int device) {
  static std::atomic<int> state[kMaxDevices];  // 0 not yet, 1 ready, 2 unavailable
  if (device < 0 || device >= kMaxDevices) return false;
  if (const int v = state[device].load()) return v == 1;
  const SmallFn fns[] = {k_step_small<3, 1, 0>, k_step_small<3, 1, 1>, k_step_small<3, 1, 2>,
                         k_step_small<3, 3, 0>, k_step_small<3, 3, 1>, k_step_small<3, 3, 2>,
                         k_step_small<2, 1, 0>, k_step_small<2, 1, 1>, k_step_small<2, 3, 0>,
                         k_step_small<2, 3, 1>};
  bool ok = true;
  for (const SmallFn fn : fns) ok = ok && small_prepare_one(fn);
  state[device].store(ok ? 1 : 2);
  return ok;
}

int launch_small(tecs_sim* s, SmallFn fn, const PassArgs& p1, bool pol) {
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = kSmallCtas;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.gridDim = dim3(kSmallCtas);
  cfg.blockDim = dim3(kPassThreads);
  cfg.dynamicSmemBytes = (s->g.nbins + 1) * sizeof(unsigned);
  cfg.stream = s->stream;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  const unsigned part_words = s->fuse_part ? (unsigned)scan_part_words(s->g.nbins + 1) : 0u;
  CK(cudaLaunchKernelEx(&cfg, fn, s->g, s->fp, p1, s->fuse_count ? 0 : 1, (const float4*)s->A, (const float2*)(pol ? s->PA : nullptr), s->B,
                        pol ? s->PB : nullptr, s->Bid, s->off, s->src, part_words));
  return 0;
}

int enqueue_step(tecs_sim* s, double dt64, bool rebuild, int& K) {
  const float dt = (float)dt64;  // VectorN * Scalar narrows dt (vector.hpp:264-267)
  const bool pol = s->d.has_polarity != 0;
  const bool sym = s->d.symmetric != 0;
  const bool com = s->d.com_fix != 0;
  // the old velocities are written by k_finish, after every pass that reads
  // them; the extra fields are updated there (the built-in passes carry none)
  const bool fused = !com && !sym && !s->ov && !s->E;
  const unsigned L = launch_count(s);
  const unsigned gb = ceil_div(L ? L : 1, 256);
  const int D = s->d.dims;
  if (rebuild && small_step_ok(s)) {
    // k_step_small below sorts the cells itself
  } else if (rebuild || !s->binned) {
    if (enqueue_rebuild(s, K, !s->fuse_count)) return -1;
  } else {
    PROF_BEGIN(s);
    k_refresh<<<gb, 256, 0, s->stream>>>(s->ctr, s->A, pol ? s->PA : nullptr, s->B, pol ? s->PB : nullptr,
                                         extra_move(s));
    PROF_END(s, "k_refresh");
    K += 1;
  }
  PassArgs a = base_args(s, dt, dt64);
  if (rebuild && small_step_ok(s)) {
    // the whole step in one cluster (k_step_small)
    PassArgs p1 = a;
    p1.X = s->B;
    p1.P = pol ? s->PB : nullptr;
    p1.Bx = s->B;
    p1.Bp = p1.P;
    p1.mode = kEulerFused;
    p1.count_next = s->fuse_count ? 1 : 0;
    const SmallFn fn = small_fn_of(s);
    if (!fn) return fail("unsupported finder/force/dims combination");
    PROF_BEGIN(s);
    if (launch_small(s, fn, p1, pol)) return -1;
    PROF_END(s, "k_step_small");
    K += 1;
    return 0;
  }
  auto store_args = [&](PassArgs& p, float4* dout, float2* dpout, int slot) {
    p.mode = kStore;
    p.d_out = dout;
    p.dp_out = pol ? dpout : nullptr;
    p.ed_out = slot == 0 ? s->ed1 : s->ed2;
    p.EX = slot == 0 ? s->EB : s->Et;
    p.com_part = (com && !sym) ? s->com_part : nullptr;
    p.com_out = s->com + 4 * slot;
    p.com_slot = slot;
  };
  auto sym_zero = [&](float4* dout, float2* dpout) -> int {
    if (!sym) return 0;
    CK(cudaMemsetAsync(dout, 0, sizeof(float4) * s->d.capacity, s->stream));
    if (pol) CK(cudaMemsetAsync(dpout, 0, sizeof(float2) * s->d.capacity, s->stream));
    return 0;
  };
  auto sym_com = [&](const float4* dout, int slot) {
    if (!(sym && com)) return;
    PassArgs c = base_args(s, dt);
    c.com_part = s->com_part;
    c.com_out = s->com + 4 * slot;
    c.com_slot = slot;
    prof_mark(s, 0, nullptr);
    k_com<<<ceil_div(L ? L : 1, 128), 128, 0, s->stream>>>(dout, c);
    prof_mark(s, 1, "k_com");
    K += 1;
  };
  PassArgs fin = base_args(s, dt, dt64);
  fin.Bx = s->B;
  fin.Bp = pol ? s->PB : nullptr;
  fin.d1 = s->d1;
  fin.dp1 = pol ? s->dp1 : nullptr;
  fin.EBx = s->EB;
  fin.ed1 = s->ed1;
  fin.ed2 = s->d.integrator == TECS_HEUN ? s->ed2 : nullptr;
  fin.Et = s->Et;

  if (s->d.integrator == TECS_EULER) {
    PassArgs p = a;
    p.X = s->B;
    p.P = pol ? s->PB : nullptr;
    if (fused) {
      p.mode = kEulerFused;
      p.Bx = s->B;
      p.Bp = p.P;
      if (enqueue_pass(s, p, K)) return -1;
    } else {
      store_args(p, s->d1, s->dp1, 0);
      if (sym_zero(s->d1, s->dp1)) return -1;
      if (enqueue_pass(s, p, K)) return -1;
      sym_com(s->d1, 0);
      PROF_BEGIN(s);
      if (D == 3) k_finish<3><<<gb, 256, 0, s->stream>>>(0, s->g, fin, s->com, nullptr, nullptr);
      else k_finish<2><<<gb, 256, 0, s->stream>>>(0, s->g, fin, s->com, nullptr, nullptr);
      PROF_END(s, "k_finish");
      K += 1;
    }
  } else {
    PassArgs p1 = a;
    p1.X = s->B;
    p1.P = pol ? s->PB : nullptr;
    if (fused) {
      p1.mode = kHeun1Fused;
      p1.d_out = s->d1;
      p1.dp_out = pol ? s->dp1 : nullptr;
      p1.Xt = s->Xt;
      p1.Pt = pol ? s->Pt : nullptr;
      if (enqueue_pass(s, p1, K)) return -1;
    } else {
      store_args(p1, s->d1, s->dp1, 0);
      if (sym_zero(s->d1, s->dp1)) return -1;
      if (enqueue_pass(s, p1, K)) return -1;
      sym_com(s->d1, 0);
      PROF_BEGIN(s);
      k_predict<<<gb, 256, 0, s->stream>>>(s->ctr, s->com, dt, s->B, pol ? s->PB : nullptr, s->d1,
                                           pol ? s->dp1 : nullptr, s->Xt, pol ? s->Pt : nullptr, fin);
      PROF_END(s, "k_predict");
      K += 1;
    }
    PassArgs p2 = a;
    p2.X = s->Xt;
    p2.P = pol ? s->Pt : nullptr;
    p2.full_step = 0;  // heun.hpp:117
    if (fused) {
      p2.mode = kHeun2Fused;
      p2.Bx = s->B;
      p2.Bp = pol ? s->PB : nullptr;
      p2.d1 = s->d1;
      p2.dp1 = pol ? s->dp1 : nullptr;
      if (enqueue_pass(s, p2, K)) return -1;
    } else {
      store_args(p2, s->d2, s->dp2, 1);
      if (sym_zero(s->d2, s->dp2)) return -1;
      if (enqueue_pass(s, p2, K)) return -1;
      sym_com(s->d2, 1);
      PROF_BEGIN(s);
      if (D == 3) k_finish<3><<<gb, 256, 0, s->stream>>>(1, s->g, fin, s->com, s->d2, pol ? s->dp2 : nullptr);
      else k_finish<2><<<gb, 256, 0, s->stream>>>(1, s->g, fin, s->com, s->d2, pol ? s->dp2 : nullptr);
      PROF_END(s, "k_finish");
      K += 1;
    }
  }
  if (s->d.division_probability > 0.0) {
    PROF_BEGIN(s);
    k_divide_commit<<<32, 256, 0, s->stream>>>(s->ctr, s->d.capacity, s->div_parent, s->div_slot, s->A);
    PROF_END(s, "k_divide_commit");
    K += 1;
  }
  CK(cudaGetLastError());
  return 0;
}

void drop_graphs(tecs_sim* s) {
  for (int k = 0; k < 2; ++k) {
    if (s->gexec[k]) cudaGraphExecDestroy(s->gexec[k]);
    s->gexec[k] = nullptr;
  }
}

}  // namespace

extern "C" {

const char* tecs_last_error(void) { return g_last_error.c_str(); }

int tecs_sim_desc_default(tecs_sim_desc* d) {
  if (!d) return fail("null desc");
  std::memset(d, 0, sizeof *d);
  d->dims = 3;
  d->finder = TECS_FINDER_BINNED_GABRIEL;
  d->cutoff = 1.0f;
  d->gabriel_coefficient = 0.8f;
  for (int k = 0; k < 3; ++k) { d->min_bounds[k] = -20.f; d->max_bounds[k] = 20.f; }
  d->bin_size_scale = 1.0f;
  d->integrator = TECS_HEUN;
  d->force = TECS_FORCE_SPRING2R;
  d->k_rep = 2.0f; d->r_rep = 0.7f; d->k_adh = 0.5f; d->r_adh = 0.8f;
  d->division_offset = 0.25f;
  d->seed = 2807;
  return 0;
}

int tecs_sim_create(const tecs_sim_desc* desc, tecs_sim** out) {
  if (!desc || !out) return fail("null argument");
  *out = nullptr;
  if (desc->dims != 2 && desc->dims != 3) return fail("dims must be 2 or 3");
  if (desc->capacity == 0) return fail("capacity must be > 0");
  if (desc->finder < 0 || desc->finder > TECS_FINDER_DELAUNAY) return fail("unknown finder");
  if (desc->finder >= TECS_FINDER_NAIVE_DELAUNAY && desc->symmetric)
    return fail("the Delaunay finder has no symmetric variant");
  if (desc->finder == TECS_FINDER_DELAUNAY && desc->capacity >= (1u << 30))
    return fail("the Delaunay finder holds fewer than 2^30 cells");
  if (desc->finder == TECS_FINDER_NAIVE_DELAUNAY && desc->capacity > kDelaunayMaxCells)
    return fail("the naive Delaunay finder holds at most 4096 cells");
  if (desc->force < 0 || desc->force > 2) return fail("unknown force");
  if (desc->force == TECS_FORCE_POLARITY && (desc->dims != 3 || !desc->has_polarity))
    return fail("the polarity force needs dims 3 and a polarity field");
  if (!(desc->cutoff > 0.f) || !(desc->bin_size_scale > 0.f)) return fail("cutoff and bin_size_scale must be > 0");
  tecs_sim* s = new tecs_sim();
  s->d = *desc;
  int dev_count = 0;
  if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count == 0) {
    delete s;
    return fail("no CUDA device");
  }
  if (cudaSetDevice(desc->device) != cudaSuccess) {
    delete s;
    return fail("cudaSetDevice failed");
  }
  // grid: binned_gabriel.hpp:28-42, grid.hpp:201-215
  GridP& g = s->g;
  g.bin_size = desc->bin_size_scale * desc->cutoff;
  g.inv_bin = 1.0f / g.bin_size;
  g.R = (int)std::ceil(desc->cutoff * g.inv_bin);
  unsigned long long nb = 1;
  for (int k = 0; k < 3; ++k) { g.mn[k] = 0.f; g.ext[k] = 1; }
  for (int k = 0; k < desc->dims; ++k) {
    g.mn[k] = desc->min_bounds[k];
    g.ext[k] = (int)std::ceil((desc->max_bounds[k] - desc->min_bounds[k]) / g.bin_size);
    if (g.ext[k] < 1) { delete s; return fail("max_bounds must exceed min_bounds"); }
    nb *= (unsigned long long)g.ext[k];
  }
  // the naive and Delaunay finders do not use this grid
  const bool binned_finder = desc->finder == TECS_FINDER_BINNED_ALL_PAIRS || desc->finder == TECS_FINDER_BINNED_GABRIEL;
  if (binned_finder && nb > (1ull << 31)) { delete s; return fail("bin grid too large"); }
  if (!binned_finder && nb > (1ull << 31)) nb = 1ull << 31;
  g.nbins = (unsigned)nb;
  grid_set_pow2(g);
  ForceP& f = s->fp;
  f.force = desc->force;
  f.k_rep = desc->k_rep; f.r_rep = desc->r_rep; f.k_adh = desc->k_adh; f.r_adh = desc->r_adh; f.k_pol = desc->k_pol;
  f.rc2 = desc->cutoff * desc->cutoff;
  f.gab_factor = desc->gabriel_coefficient * desc->gabriel_coefficient * 0.25f;
  f.gab_csq = desc->gabriel_coefficient * desc->gabriel_coefficient;
  s->binned = desc->finder == TECS_FINDER_BINNED_ALL_PAIRS || desc->finder == TECS_FINDER_BINNED_GABRIEL;
  s->fuse_count = s->binned && (desc->division_probability > 0.0 || desc->rebuild_every_n <= 1);
  s->fuse_part = s->binned && (double)g.nbins > 4.0 * (double)desc->capacity;
  {
    const char* e = std::getenv("TECS_NO_SMALL_STEP");
    s->small_ok = !(e && e[0] == '1') && s->binned && small_prepare(s->d.device);
  }

  const size_t cap = desc->capacity;
  auto alloc = [&](void** p, size_t bytes) -> bool { return cudaMalloc(p, bytes ? bytes : 16) == cudaSuccess; };
  bool ok = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) == cudaSuccess;
  // the sorted position arrays carry kRowPad zeroed float4 past the capacity
  const size_t xcap = cap + kRowPad;
  ok = ok && alloc((void**)&s->A, xcap * 16) && alloc((void**)&s->B, xcap * 16) && alloc((void**)&s->Xt, xcap * 16) &&
       alloc((void**)&s->d1, cap * 16) && alloc((void**)&s->d2, cap * 16);
  // every clear is queued on the simulation's own stream: the stream is
  // non-blocking, so work on it is not ordered after the legacy default
  // stream, which a plain cudaMemset would use
  ok = ok && cudaMemsetAsync(s->A, 0, xcap * 16, s->stream) == cudaSuccess &&
       cudaMemsetAsync(s->B, 0, xcap * 16, s->stream) == cudaSuccess &&
       cudaMemsetAsync(s->Xt, 0, xcap * 16, s->stream) == cudaSuccess;
  if (desc->has_polarity)
    ok = ok && alloc((void**)&s->PA, cap * 8) && alloc((void**)&s->PB, cap * 8) && alloc((void**)&s->Pt, cap * 8) &&
         alloc((void**)&s->dp1, cap * 8) && alloc((void**)&s->dp2, cap * 8);
  ok = ok && alloc((void**)&s->key, cap * 4) && alloc((void**)&s->rank, cap * 4) && alloc((void**)&s->src, cap * 4);
  ok = ok && alloc((void**)&s->div_parent, cap * 4) && alloc((void**)&s->div_slot, cap * 4);
  if (s->binned) ok = ok && alloc((void**)&s->Bid, cap * 4);
  if (desc->finder == TECS_FINDER_NAIVE_DELAUNAY) ok = ok && alloc((void**)&s->dmult, cap * cap * 2);
  if (desc->finder == TECS_FINDER_DELAUNAY) {
    // about two cells per bin: capacity / 2 bins suffice (dl::plan_grid)
    s->dl_maxbins = (unsigned)(cap / 2 + 64);
    ok = ok && alloc((void**)&s->dl_st, sizeof(DlState)) && alloc((void**)&s->dl_cnt, (size_t)s->dl_maxbins * 4) &&
         alloc((void**)&s->dl_off, ((size_t)s->dl_maxbins + 1) * 4) && alloc((void**)&s->dl_idx, cap * 4) &&
         alloc((void**)&s->dl_sp, cap * 16) && alloc((void**)&s->dl_row, cap * kDlRow * 8) &&
         alloc((void**)&s->dl_len, cap * 4);
    if (ok) ok = cudaMemsetAsync(s->dl_len, 0, cap * 4, s->stream) == cudaSuccess;
  }
  if (s->binned) {
    const size_t len = (size_t)g.nbins + 1;
    ok = ok && alloc((void**)&s->cnt, len * 4) && alloc((void**)&s->off, len * 4) &&
         alloc((void**)&s->part, scan_part_words(len) * 4);
  }
  // COM accumulators: 3 per reduction slot, two slots (Heun's two passes)
  const size_t pass_blocks = std::max<size_t>(ceil_div(cap, 128), 2);
  ok = ok && cudaMallocHost((void**)&s->hctr, sizeof(Counters)) == cudaSuccess;
  ok = ok && alloc((void**)&s->ctr, sizeof(Counters)) && alloc((void**)&s->com_part, pass_blocks * 3 * 8) &&
       alloc((void**)&s->com, 8 * 4) && alloc((void**)&s->stage, cap * 4 * 4);
  if (ok && s->cnt) ok = cudaMemsetAsync(s->cnt, 0, ((size_t)g.nbins + 1) * 4, s->stream) == cudaSuccess;
  if (ok)
    ok = cudaMemsetAsync(s->ctr, 0, sizeof(Counters), s->stream) == cudaSuccess &&
         cudaMemsetAsync(s->com, 0, 32, s->stream) == cudaSuccess &&
         cudaMemsetAsync(s->com_part, 0, pass_blocks * 3 * 8, s->stream) == cudaSuccess &&
         cudaStreamSynchronize(s->stream) == cudaSuccess;
  if (!ok) {
    std::string m = std::string("device allocation failed: ") + cudaGetErrorString(cudaGetLastError());
    tecs_sim_destroy(s);
    return fail(m);
  }
  *out = s;
  return 0;
}

int tecs_sim_destroy(tecs_sim* s) {
  if (!s) return 0;
  cudaSetDevice(s->d.device);
  if (s->stream) cudaStreamSynchronize(s->stream);
  drop_graphs(s);
  for (auto& e : s->ev)
    if (e) cudaEventDestroy(e);
  if (s->hctr) cudaFreeHost(s->hctr);
  void* ptrs[] = {s->A, s->B, s->Xt, s->d1, s->d2, s->PA, s->PB, s->Pt, s->dp1, s->dp2, s->key, s->rank, s->src,
                  s->cnt, s->off, s->part, s->div_parent, s->div_slot, s->ctr, s->com_part, s->com, s->stage,
                  s->Bid, s->dmult, s->link_off, s->link_ent, s->slot_of, s->ov, s->EA, s->EB, s->Et,
                  s->ed1, s->ed2, s->dl_st, s->dl_cnt, s->dl_off, s->dl_idx, s->dl_sp, s->dl_row, s->dl_len};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (s->stream) cudaStreamDestroy(s->stream);
  delete s;
  return 0;
}

// A new state from positions (and polarities) the device can read: one
// k_upload pass.  The delta buffers need no reset: every pass writes the
// deltas of all active cells before they are read.
namespace {
// the extra fields of the n_old current cells into cell-id order (the upload
// puts cell i at slot i): EA -> Et by A's ids, then back
__global__ void k_extra_to_id(const float4* __restrict__ A, unsigned n_old, unsigned E, size_t C,
                              const float* __restrict__ EA, float* __restrict__ tmp) {
  for (unsigned s = blockIdx.x * blockDim.x + threadIdx.x; s < n_old; s += gridDim.x * blockDim.x) {
    const unsigned id = id_of(A[s]);
    for (unsigned k = 0; k < E; ++k) tmp[k * C + id] = EA[k * C + s];
  }
}
}  // namespace

static int upload_common(tecs_sim* s, const float* pos, const float2* pol, unsigned n) {
  if (s->E && s->n_host) {
    // Xt is free between steps; its extras partner Et takes the copy
    k_extra_to_id<<<ceil_div(s->n_host, 256), 256, 0, s->stream>>>(s->A, s->n_host, s->E, s->d.capacity, s->EA,
                                                                   s->Et);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(s->EA, s->Et, (size_t)s->E * s->d.capacity * 4, cudaMemcpyDeviceToDevice, s->stream));
  }
  // the first rebuild expects the bin counts of A, and their chunk totals,
  // to be made already
  const unsigned len = s->g.nbins + 1;
  if (s->fuse_count) {
    CK(cudaMemsetAsync(s->cnt, 0, (size_t)len * 4, s->stream));
    if (s->fuse_part) CK(cudaMemsetAsync(s->part, 0, scan_part_words(len) * 4, s->stream));
  }
  k_upload<<<std::max(1u, ceil_div(n, 256)), 256, 0, s->stream>>>(
      pos, s->d.has_polarity ? pol : nullptr, n, s->d.dims, s->A, s->PA, s->ctr, s->g, s->key, s->rank,
      s->fuse_count ? s->cnt : nullptr, (s->fuse_count && s->fuse_part) ? s->part : nullptr);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(s->stream));
  // the captured step graphs depend on the state only through their grid
  // size: keep them unless that changes
  const unsigned old_launch = launch_count(s);
  s->n_host = n;
  s->step_count = 0;
  s->sorted = false;
  if (launch_count(s) != old_launch) drop_graphs(s);
  return 0;
}

int tecs_sim_upload(tecs_sim* s, const float* pos, const float* pol, unsigned n) {
  if (!s || (!pos && n)) return fail("null argument");
  if (n > s->d.capacity) return fail("agent count exceeds capacity");
  if (s->d.has_polarity && n && !pol) return fail("simulation has a polarity field: polarity required");
  CK(cudaSetDevice(s->d.device));
  const int D = s->d.dims;
  // page-locked host buffers are read by k_upload itself; other host memory
  // is copied to the device first
  const float* src = static_cast<const float*>(mapped_host(pos));
  const float2* psrc = static_cast<const float2*>(mapped_host(pol));
  if (n && !src) {
    CK(cudaMemcpyAsync(s->stage, pos, (size_t)n * D * 4, cudaMemcpyHostToDevice, s->stream));
    src = s->stage;
  }
  if (n && s->d.has_polarity && !psrc) {
    CK(cudaMemcpyAsync(s->Pt, pol, (size_t)n * 8, cudaMemcpyHostToDevice, s->stream));
    psrc = s->Pt;
  }
  return upload_common(s, src, psrc, n);
}

int tecs_sim_upload_device(tecs_sim* s, const float* dpos, const float* dpol, unsigned n) {
  if (!s || (!dpos && n)) return fail("null argument");
  if (n > s->d.capacity) return fail("agent count exceeds capacity");
  if (s->d.has_polarity && n && !dpol) return fail("simulation has a polarity field: polarity required");
  CK(cudaSetDevice(s->d.device));
  return upload_common(s, dpos, reinterpret_cast<const float2*>(dpol), n);
}

int tecs_sim_step(tecs_sim* s, double dt, int n_steps) {
  if (!s) return fail("null simulation");
  if (n_steps < 0) return fail("negative step count");
  CK(cudaSetDevice(s->d.device));
  for (int it = 0; it < n_steps; ++it) {
    // binned_gabriel.hpp:83-89: rebuild when step_count == 0 || step_count >= rebuild_every_n;
    // division resets the counter every step (set_agent_count, :61-64)
    const bool rebuild = s->step_count == 0 || s->step_count >= s->d.rebuild_every_n;
    const int gk = rebuild ? 0 : 1;
    if (rebuild) s->step_count = 0;
    s->step_count++;
    if (s->d.division_probability > 0.0) s->step_count = 0;
    if (!s->use_graph) {
      int K = 0;
      s->prof_n = 0;
      if (enqueue_step(s, dt, rebuild, K)) return -1;
      s->last_kernels = K;
      s->prof_last = s->prof_n;
      if (rebuild) s->sorted = true;
      continue;
    }
    if (!s->gexec[gk] || s->gdt[gk] != dt) {
      if (s->gexec[gk]) { cudaGraphExecDestroy(s->gexec[gk]); s->gexec[gk] = nullptr; }
      cudaGraph_t graph;
      CK(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
      int K = 0;
      s->prof_n = 0;
      g_capturing = true;
      int rc = enqueue_step(s, dt, rebuild, K);
      g_capturing = false;
      s->prof_last = s->prof_n;
      cudaError_t e = cudaStreamEndCapture(s->stream, &graph);
      if (rc) return -1;
      if (e != cudaSuccess) return fail(std::string("graph capture: ") + cudaGetErrorString(e));
      e = cudaGraphInstantiate(&s->gexec[gk], graph, 0);
      cudaGraphDestroy(graph);
      if (e != cudaSuccess) return fail(std::string("graph instantiate: ") + cudaGetErrorString(e));
      s->gdt[gk] = dt;
      s->kernels[gk] = K;
    }
    CK(cudaGraphLaunch(s->gexec[gk], s->stream));
    s->last_kernels = s->kernels[gk];
    if (rebuild) s->sorted = true;
  }
  return 0;
}

int tecs_sim_synchronize(tecs_sim* s) {
  if (!s) return fail("null simulation");
  CK(cudaStreamSynchronize(s->stream));
  return 0;
}

int tecs_sim_count(tecs_sim* s, unsigned* n) {
  if (!s || !n) return fail("null argument");
  CK(cudaMemcpyAsync(s->hctr, s->ctr, sizeof(Counters), cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  if (s->hctr->error & 1u) return fail("capacity exceeded by cell division");
  if (s->hctr->error & 2u) return fail("a user pairwise law set drag in a simulation that keeps no old velocities");
  if (s->hctr->error & 4u)
    return fail("the Delaunay finder met a cell with more partners or star simplices than its arrays hold");
  *n = s->hctr->n;
  return 0;
}

int tecs_sim_download(tecs_sim* s, float* pos, float* pol, unsigned* n_out) {
  if (!s || !pos) return fail("null argument");
  float* dst = static_cast<float*>(const_cast<void*>(mapped_host(pos)));
  float* pdst = (pol && s->d.has_polarity) ? static_cast<float*>(const_cast<void*>(mapped_host(pol))) : nullptr;
  if (dst && (pdst || !(pol && s->d.has_polarity))) {
    // page-locked host buffers: unpack in id order on the device and write
    // them from kernels, the count taken on the device; one synchronisation
    CK(cudaSetDevice(s->d.device));
    const unsigned gb = std::max(1u, ceil_div((unsigned)s->d.capacity, 256));
    const int D = s->d.dims;
    k_unpack_dev<<<gb, 256, 0, s->stream>>>(s->A, s->ctr, D, (float*)s->Xt);
    k_copy_out<<<gb, 256, 0, s->stream>>>((const float*)s->Xt, s->ctr, (unsigned)D, dst);
    if (pdst) {
      k_unpack2_dev<<<gb, 256, 0, s->stream>>>(s->A, s->ctr, s->PA, s->Pt);
      k_copy_out<<<gb, 256, 0, s->stream>>>((const float*)s->Pt, s->ctr, 2u, pdst);
    }
    CK(cudaGetLastError());
    unsigned n = 0;
    if (tecs_sim_count(s, &n)) return -1;
    if (n_out) *n_out = n;
    return 0;
  }
  unsigned n = 0;
  if (tecs_sim_count(s, &n)) return -1;
  const int D = s->d.dims;
  if (n) {
    // Xt is free between steps; unpack into it in id order
    k_unpack<<<ceil_div(n, 256), 256, 0, s->stream>>>(s->A, nullptr, s->A, n, D, (float*)s->Xt);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(pos, s->Xt, (size_t)n * D * 4, cudaMemcpyDeviceToHost, s->stream));
    if (pol && s->d.has_polarity) {
      k_unpack2<<<ceil_div(n, 256), 256, 0, s->stream>>>(s->A, nullptr, s->PA, n, s->Pt);
      CK(cudaGetLastError());
      CK(cudaMemcpyAsync(pol, s->Pt, (size_t)n * 8, cudaMemcpyDeviceToHost, s->stream));
    }
    CK(cudaStreamSynchronize(s->stream));
  }
  if (n_out) *n_out = n;
  return 0;
}

int tecs_sim_evaluate(tecs_sim* s, float* dpos, float* dpol, uint32_t* pairs, size_t pair_cap, size_t* n_pairs) {
  if (!s) return fail("null simulation");
  CK(cudaSetDevice(s->d.device));
  unsigned n = 0;
  if (tecs_sim_count(s, &n)) return -1;
  const bool pol = s->d.has_polarity != 0;
  int K = 0;
  if (enqueue_rebuild(s, K, !s->fuse_count)) return -1;
  uint2* dpairs = nullptr;
  if (pairs && pair_cap) CK(cudaMalloc(&dpairs, pair_cap * sizeof(uint2)));
  CK(cudaMemsetAsync(&s->ctr->pair_count, 0, 8, s->stream));
  if (s->d.symmetric) {
    CK(cudaMemsetAsync(s->d1, 0, sizeof(float4) * s->d.capacity, s->stream));
    if (pol) CK(cudaMemsetAsync(s->dp1, 0, sizeof(float2) * s->d.capacity, s->stream));
  }
  PassArgs a = base_args(s, 0.f);
  a.X = s->B;
  a.P = pol ? s->PB : nullptr;
  a.mode = kStore;
  a.d_out = s->d1;
  a.dp_out = pol ? s->dp1 : nullptr;
  a.pairs = dpairs;
  a.pair_cap = dpairs ? pair_cap : 0;
  a.count_next = 0;
  int rc = enqueue_pass(s, a, K);
  if (rc == 0 && s->binned) s->sorted = true;  // the rebuild above sorted the current cells
  if (rc == 0 && s->fuse_count && n) {
    // A is unchanged: count it again for the next step's rebuild
    k_count<<<ceil_div(n, 256), 256, 0, s->stream>>>(s->A, s->ctr, s->g, s->d.dims, s->key, s->rank, s->cnt,
                                                     s->fuse_part ? s->part : nullptr);
  }
  if (rc == 0 && n) {
    if (dpos) {
      k_unpack<<<ceil_div(n, 256), 256, 0, s->stream>>>(s->B, s->binned ? s->Bid : nullptr, s->d1, n, s->d.dims,
                                                         (float*)s->Xt);
      cudaMemcpyAsync(dpos, s->Xt, (size_t)n * s->d.dims * 4, cudaMemcpyDeviceToHost, s->stream);
    }
    if (dpol && pol) {
      k_unpack2<<<ceil_div(n, 256), 256, 0, s->stream>>>(s->B, s->binned ? s->Bid : nullptr, s->dp1, n, s->Pt);
      cudaMemcpyAsync(dpol, s->Pt, (size_t)n * 8, cudaMemcpyDeviceToHost, s->stream);
    }
  }
  unsigned long long cnt = 0;
  cudaMemcpyAsync(&cnt, &s->ctr->pair_count, 8, cudaMemcpyDeviceToHost, s->stream);
  cudaError_t e = cudaStreamSynchronize(s->stream);
  if (rc == 0 && e == cudaSuccess && dpairs) {
    size_t m = cnt < pair_cap ? (size_t)cnt : pair_cap;
    e = cudaMemcpyAsync(pairs, dpairs, m * sizeof(uint2), cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  }
  if (dpairs) cudaFree(dpairs);
  if (rc) return rc;
  if (e != cudaSuccess) return fail(std::string("evaluate: ") + cudaGetErrorString(e));
  if (n_pairs) *n_pairs = (size_t)cnt;
  return 0;
}

void* tecs_sim_stream(tecs_sim* s) { return s ? (void*)s->stream : nullptr; }

int tecs_sim_download_device(tecs_sim* s, float* d_positions, float* d_polarity, unsigned* n_out) {
  if (!s || !d_positions) return fail("null argument");
  CK(cudaSetDevice(s->d.device));
  const unsigned gb = std::max(1u, ceil_div((unsigned)s->d.capacity, 256));
  // the unpack takes the agent count from the device counters
  k_unpack_dev<<<gb, 256, 0, s->stream>>>(s->A, s->ctr, s->d.dims, d_positions);
  if (d_polarity && s->d.has_polarity)
    k_unpack2_dev<<<gb, 256, 0, s->stream>>>(s->A, s->ctr, s->PA, reinterpret_cast<float2*>(d_polarity));
  CK(cudaGetLastError());
  unsigned n = 0;
  if (tecs_sim_count(s, &n)) return -1;
  if (n_out) *n_out = n;
  return 0;
}

namespace {
// old velocities (float4 by id) <-> D floats per cell
__global__ void k_vel_out(const float4* __restrict__ ov, unsigned n, int D, float* __restrict__ out) {
  for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float4 v = ov[i];
    const float c[3] = {v.x, v.y, v.z};
    for (int d = 0; d < D; ++d) out[(size_t)i * D + d] = c[d];
  }
}
__global__ void k_vel_in(const float* __restrict__ in, unsigned n, int D, float4* __restrict__ ov) {
  for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    float c[3] = {0.f, 0.f, 0.f};
    for (int d = 0; d < D; ++d) c[d] = in[(size_t)i * D + d];
    ov[i] = make_float4(c[0], c[1], c[2], 0.f);
  }
}
}  // namespace

int tecs_sim_keep_old_velocities(tecs_sim* s, int keep) {
  if (!s) return fail("null simulation");
  if (keep && s->d.symmetric) return fail("old velocities are kept with the non-symmetric finders");
  if ((keep != 0) == (s->ov != nullptr)) return 0;
  CK(cudaSetDevice(s->d.device));
  CK(cudaStreamSynchronize(s->stream));
  drop_graphs(s);
  if (!keep) {
    CK(cudaFree(s->ov));
    s->ov = nullptr;
    return 0;
  }
  CK(cudaMalloc(&s->ov, sizeof(float4) * s->d.capacity));
  CK(cudaMemsetAsync(s->ov, 0, sizeof(float4) * s->d.capacity, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  return 0;
}

int tecs_sim_old_velocities(tecs_sim* s, float* out, unsigned* n_out) {
  if (!s || !out) return fail("null argument");
  if (!s->ov) return fail("the simulation keeps no old velocities");
  CK(cudaSetDevice(s->d.device));
  unsigned n = 0;
  if (tecs_sim_count(s, &n)) return -1;
  if (n_out) *n_out = n;
  if (!n) return 0;
  const int D = s->d.dims;
  // Xt is free between steps
  k_vel_out<<<ceil_div(n, 256), 256, 0, s->stream>>>(s->ov, n, D, reinterpret_cast<float*>(s->Xt));
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(out, s->Xt, (size_t)n * D * 4, cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  return 0;
}

int tecs_sim_set_old_velocities(tecs_sim* s, const float* v, unsigned n) {
  if (!s || (!v && n)) return fail("null argument");
  if (!s->ov) return fail("the simulation keeps no old velocities");
  if (n > s->d.capacity) return fail("agent count exceeds capacity");
  if (!n) return 0;
  CK(cudaSetDevice(s->d.device));
  const int D = s->d.dims;
  CK(cudaMemcpyAsync(s->Xt, v, (size_t)n * D * 4, cudaMemcpyHostToDevice, s->stream));
  k_vel_in<<<ceil_div(n, 256), 256, 0, s->stream>>>(reinterpret_cast<const float*>(s->Xt), n, D, s->ov);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(s->stream));
  return 0;
}

namespace {
// one extra field (components [offset, offset + width)) of the n active
// cells, by cell id: device block <-> AoS rows of width floats
__global__ void k_extra_out(const float4* __restrict__ A, unsigned n, size_t C, const float* __restrict__ EA,
                            unsigned offset, unsigned width, float* __restrict__ out) {
  for (unsigned s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
    const unsigned id = id_of(A[s]);
    for (unsigned c = 0; c < width; ++c) out[(size_t)id * width + c] = EA[(offset + c) * C + s];
  }
}
__global__ void k_extra_in(const float4* __restrict__ A, unsigned n, size_t C, float* __restrict__ EA,
                           unsigned offset, unsigned width, const float* __restrict__ in) {
  for (unsigned s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
    const unsigned id = id_of(A[s]);
    for (unsigned c = 0; c < width; ++c) EA[(offset + c) * C + s] = in[(size_t)id * width + c];
  }
}
}  // namespace

int tecs_sim_set_extra_fields(tecs_sim* s, unsigned components, uint32_t double_mask) {
  if (!s) return fail("null simulation");
  if (components > kMaxExtra) return fail("at most 8 extra components per cell");
  if (components && s->d.symmetric) return fail("extra fields are carried with the non-symmetric finders");
  if (components == s->E && double_mask == s->ex_dbl) return 0;
  CK(cudaSetDevice(s->d.device));
  CK(cudaStreamSynchronize(s->stream));
  drop_graphs(s);
  for (float** p : {&s->EA, &s->EB, &s->Et, &s->ed1, &s->ed2}) {
    if (*p) CK(cudaFree(*p));
    *p = nullptr;
  }
  s->E = components;
  s->ex_dbl = components ? double_mask & ((1u << components) - 1u) : 0u;
  if (!components) return 0;
  const size_t bytes = (size_t)components * s->d.capacity * 4;
  for (float** p : {&s->EA, &s->EB, &s->Et, &s->ed1, &s->ed2}) {
    CK(cudaMalloc(p, bytes));
    CK(cudaMemsetAsync(*p, 0, bytes, s->stream));
  }
  CK(cudaStreamSynchronize(s->stream));
  return 0;
}

static int extra_check(tecs_sim* s, unsigned offset, unsigned width) {
  if (!s) return fail("null simulation");
  if (!width || offset + width > s->E) return fail("extra field outside the extra components");
  return 0;
}

int tecs_sim_upload_extra(tecs_sim* s, unsigned offset, unsigned width, const float* values, unsigned n) {
  if (extra_check(s, offset, width)) return -1;
  if (!values && n) return fail("null argument");
  if (n > s->n_host) return fail("more rows than active cells");
  if (!n) return 0;
  CK(cudaSetDevice(s->d.device));
  const size_t bytes = (size_t)n * width * 4;
  const float* src = values;
  cudaPointerAttributes pa{};
  const bool on_device = cudaPointerGetAttributes(&pa, values) == cudaSuccess && pa.type == cudaMemoryTypeDevice;
  cudaGetLastError();
  if (!on_device) {
    // the predictor's extras are free between steps (E x capacity floats)
    CK(cudaMemcpyAsync(s->Et, values, bytes, cudaMemcpyHostToDevice, s->stream));
    src = s->Et;
  }
  k_extra_in<<<ceil_div(n, 256), 256, 0, s->stream>>>(s->A, n, s->d.capacity, s->EA, offset, width, src);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(s->stream));
  return 0;
}

int tecs_sim_download_extra(tecs_sim* s, unsigned offset, unsigned width, float* out, unsigned* n_out) {
  if (extra_check(s, offset, width)) return -1;
  if (!out) return fail("null argument");
  CK(cudaSetDevice(s->d.device));
  unsigned n = 0;
  if (tecs_sim_count(s, &n)) return -1;
  if (n_out) *n_out = n;
  if (!n) return 0;
  cudaPointerAttributes pa{};
  const bool on_device = cudaPointerGetAttributes(&pa, out) == cudaSuccess && pa.type == cudaMemoryTypeDevice;
  cudaGetLastError();
  float* dst = on_device ? out : s->Et;
  k_extra_out<<<ceil_div(n, 256), 256, 0, s->stream>>>(s->A, n, s->d.capacity, s->EA, offset, width, dst);
  CK(cudaGetLastError());
  if (!on_device) CK(cudaMemcpyAsync(out, s->Et, (size_t)n * width * 4, cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  return 0;
}

int tecs_device_alloc(int device, size_t bytes, void** out) {
  if (!out) return fail("null argument");
  *out = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
    cudaGetLastError();
    return fail("no CUDA device");
  }
  CK(cudaSetDevice(device));
  CK(cudaMalloc(out, bytes ? bytes : 16));
  return 0;
}

int tecs_device_free(void* p) {
  if (p) CK(cudaFree(p));
  return 0;
}

int tecs_device_copy(void* dst, const void* src, size_t bytes) {
  if (!bytes) return 0;
  if (!dst || !src) return fail("null argument");
  // after the device's queued work (a step on a simulation's own stream may
  // be writing what is read here)
  CK(cudaDeviceSynchronize());
  CK(cudaMemcpy(dst, src, bytes, cudaMemcpyDefault));
  return 0;
}

int tecs_sim_set_graph(tecs_sim* s, int enable) {
  if (!s) return fail("null simulation");
  s->use_graph = enable != 0;
  if (!s->use_graph) drop_graphs(s);
  return 0;
}

int tecs_sim_set_force(tecs_sim* s, int force, float k_rep, float r_rep, float k_adh, float r_adh, float k_pol) {
  if (!s) return fail("null simulation");
  if (force < 0 || force > 2) return fail("unknown force");
  if (force == TECS_FORCE_POLARITY && (s->d.dims != 3 || !s->d.has_polarity))
    return fail("the polarity force needs dims 3 and a polarity field");
  ForceP& f = s->fp;
  if (f.force == force && f.k_rep == k_rep && f.r_rep == r_rep && f.k_adh == k_adh && f.r_adh == r_adh &&
      f.k_pol == k_pol)
    return 0;
  // queued steps read the old constants through their graph's kernel arguments
  CK(cudaStreamSynchronize(s->stream));
  s->d.force = force;
  s->d.k_rep = k_rep; s->d.r_rep = r_rep; s->d.k_adh = k_adh; s->d.r_adh = r_adh; s->d.k_pol = k_pol;
  f.force = force;
  f.k_rep = k_rep; f.r_rep = r_rep; f.k_adh = k_adh; f.r_adh = r_adh; f.k_pol = k_pol;
  drop_graphs(s);
  return 0;
}

int tecs_sim_set_pair_law(tecs_sim* s, tecs_pair_law_fn fn, void* user) {
  if (!s) return fail("null simulation");
  if (fn && s->d.symmetric)
    return fail("user pairwise laws run with the non-symmetric all-pairs, Gabriel and Delaunay finders");
  if (fn == s->law_fn && user == s->law_user) return 0;
  CK(cudaSetDevice(s->d.device));
  // queued steps launched the old law from their graphs
  CK(cudaStreamSynchronize(s->stream));
  s->law_fn = fn;
  s->law_user = fn ? user : nullptr;
  drop_graphs(s);
  // the built-in passes write no extra deltas: clear the user law's
  if (s->E) {
    CK(cudaMemsetAsync(s->ed1, 0, (size_t)s->E * s->d.capacity * 4, s->stream));
    CK(cudaMemsetAsync(s->ed2, 0, (size_t)s->E * s->d.capacity * 4, s->stream));
    CK(cudaStreamSynchronize(s->stream));
  }
  return 0;
}

int tecs_sim_set_links(tecs_sim* s, const uint32_t* links, unsigned n_links, float strength) {
  if (!s || (n_links && !links)) return fail("null argument");
  if (n_links && s->d.symmetric) return fail("links are served with the non-symmetric finders");
  if (n_links >= (1u << 31)) return fail("too many links");
  const unsigned cap = s->d.capacity;
  for (size_t l = 0; l < 2 * (size_t)n_links; ++l)
    if (links[l] >= cap) return fail("link endpoint beyond capacity");
  CK(cudaSetDevice(s->d.device));
  CK(cudaStreamSynchronize(s->stream));
  // per-cell entries, each cell's in link order (a counting sort by endpoint)
  std::vector<unsigned> off((size_t)cap + 1, 0u);
  for (unsigned l = 0; l < n_links; ++l) {
    const unsigned a = links[2 * l], b = links[2 * l + 1];
    if (a == b) continue;  // skipped by the reference (integrators/base.hpp:211-212)
    ++off[a + 1];
    ++off[b + 1];
  }
  for (unsigned c = 0; c < cap; ++c) off[c + 1] += off[c];
  const unsigned entries = off[cap];
  std::vector<uint2> ent(entries ? entries : 1);
  std::vector<unsigned> fill(off.begin(), off.end() - 1);
  for (unsigned l = 0; l < n_links; ++l) {
    const unsigned a = links[2 * l], b = links[2 * l + 1];
    if (a == b) continue;
    ent[fill[a]++] = make_uint2(b, l << 1);
    ent[fill[b]++] = make_uint2(a, (l << 1) | 1u);
  }
  for (void* p : {(void*)s->link_off, (void*)s->link_ent, (void*)s->slot_of})
    if (p) CK(cudaFree(p));
  s->link_off = nullptr;
  s->link_ent = nullptr;
  s->slot_of = nullptr;
  s->n_links = 0;
  if (entries) {
    CK(cudaMalloc((void**)&s->link_off, ((size_t)cap + 1) * 4));
    CK(cudaMalloc((void**)&s->link_ent, (size_t)entries * sizeof(uint2)));
    CK(cudaMalloc((void**)&s->slot_of, (size_t)cap * 4));
    // on the simulation's stream, which the legacy default stream does not order
    CK(cudaMemcpyAsync(s->link_off, off.data(), ((size_t)cap + 1) * 4, cudaMemcpyHostToDevice, s->stream));
    CK(cudaMemcpyAsync(s->link_ent, ent.data(), (size_t)entries * sizeof(uint2), cudaMemcpyHostToDevice,
                       s->stream));
    CK(cudaStreamSynchronize(s->stream));
    s->n_links = n_links;
  }
  s->link_k = strength;
  // the id -> slot map of the current sorted order (every rebuild rewrites it);
  // the rebuild schedule itself is not touched, as in the reference
  if (s->n_links && s->binned && s->sorted) {
    k_slot_map<<<ceil_div(s->d.capacity, 256), 256, 0, s->stream>>>(s->ctr, s->Bid, s->d.capacity, s->slot_of);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(s->stream));
  }
  drop_graphs(s);
  return 0;
}

int tecs_sim_set_profiling(tecs_sim* s, int enable) {
  if (!s) return fail("null simulation");
  if ((enable != 0) != s->profiling) drop_graphs(s);
  s->profiling = enable != 0;
  return 0;
}

int tecs_sim_last_step_profile(tecs_sim* s, float* ms, int capacity, int* count) {
  if (!s || !count) return fail("null argument");
  if (!s->profiling) return fail("profiling is off");
  CK(cudaStreamSynchronize(s->stream));
  const int k = s->prof_last;
  *count = k;
  for (int i = 0; i < k && i < capacity; ++i) CK(cudaEventElapsedTime(&ms[i], s->ev[2 * i], s->ev[2 * i + 1]));
  return 0;
}

const char* tecs_sim_profile_name(tecs_sim* s, int index) {
  if (!s || index < 0 || index >= s->prof_last) return nullptr;
  return s->prof_name[index];
}

int tecs_sim_kernels_per_step(tecs_sim* s, int* kernels) {
  if (!s || !kernels) return fail("null argument");
  *kernels = s->last_kernels;
  return 0;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free force pass.
//
// Some callers cannot call cudaMalloc: code that hands this library a fixed
// device-memory budget and forbids allocation after start-up (a host runtime
// that owns the GPU's memory pool, a serving loop that must never stall on the
// allocator or fragment HBM between requests), or code already inside a region
// where allocating is not allowed.  For them, tecs_force_pass_noalloc runs the
// same one-pass force evaluation as tecs_sim_evaluate on caller-owned device
// buffers and takes all of its scratch from the file-scope array below.
//
// The array is part of the library's device image: every GPU that loads the
// library holds it (kNoallocScratchBytes) until the process exits.  All calls
// on one device share it and each call starts by clearing what must start at
// zero, so calls whose GPU work overlaps (two streams, two host threads) race
// on it and must be serialised by the caller.
namespace {
constexpr unsigned kNoallocMaxCells = TECS_NOALLOC_MAX_CELLS;
constexpr unsigned kNoallocMaxBins = TECS_NOALLOC_MAX_BINS;
constexpr size_t kNoallocAlign = 256;
constexpr size_t align_up(size_t v) { return (v + kNoallocAlign - 1) / kNoallocAlign * kNoallocAlign; }
// layout of the scratch array
constexpr size_t kOffCtr = 0;
constexpr size_t kOffA = align_up(kOffCtr + sizeof(Counters));
constexpr size_t kOffB = align_up(kOffA + (size_t)kNoallocMaxCells * sizeof(float4));
constexpr size_t kOffD = align_up(kOffB + ((size_t)kNoallocMaxCells + kRowPad) * sizeof(float4));
constexpr size_t kOffKey = align_up(kOffD + (size_t)kNoallocMaxCells * sizeof(float4));
constexpr size_t kOffRank = align_up(kOffKey + (size_t)kNoallocMaxCells * 4);
constexpr size_t kOffSrc = align_up(kOffRank + (size_t)kNoallocMaxCells * 4);
constexpr size_t kOffBid = align_up(kOffSrc + (size_t)kNoallocMaxCells * 4);
constexpr size_t kOffCnt = align_up(kOffBid + (size_t)kNoallocMaxCells * 4);
constexpr size_t kOffOff = align_up(kOffCnt + ((size_t)kNoallocMaxBins + 1) * 4);
constexpr size_t kOffPart = align_up(kOffOff + ((size_t)kNoallocMaxBins + 1) * 4);
constexpr size_t kNoallocScratchBytes =
    align_up(kOffPart + scan_part_words((size_t)kNoallocMaxBins + 1) * 4);

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];

__global__ void k_noalloc_reset(Counters* ctr, unsigned n) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    Counters c{};
    c.n = n;
    *ctr = c;
  }
}

// Device address of g_noalloc_scratch, looked up once per device with that
// device current.  The host-side name of the array is only a stand-in; kernels
// must be given this address.  The address is kept for the life of the
// process, so a device reset (cudaDeviceReset) between calls is not supported.
int noalloc_scratch(int device, unsigned char** out) {
  static std::mutex mu;
  static unsigned char* addr[64] = {};
  if (device < 0 || device >= 64) return fail("device ordinal out of range");
  std::lock_guard<std::mutex> lock(mu);
  if (!addr[device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return fail(std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
    addr[device] = (unsigned char*)p;
  }
  *out = addr[device];
  return 0;
}
}  // namespace

extern "C" int tecs_force_pass_noalloc(const tecs_sim_desc* desc, const float* d_positions, unsigned n,
                                       float* d_deltas, void* stream) {
  if (!desc || (n && (!d_positions || !d_deltas))) return fail("null argument");
  if (desc->dims != 2 && desc->dims != 3) return fail("dims must be 2 or 3");
  if (desc->finder != TECS_FINDER_BINNED_ALL_PAIRS && desc->finder != TECS_FINDER_BINNED_GABRIEL)
    return fail("the allocation-free pass serves the binned finders");
  if (desc->symmetric) return fail("the allocation-free pass serves the non-symmetric finders");
  if (desc->has_polarity || desc->force == TECS_FORCE_POLARITY)
    return fail("the allocation-free pass serves the spring laws without a polarity field");
  if (desc->force != TECS_FORCE_NONE && desc->force != TECS_FORCE_SPRING2R) return fail("unknown force");
  if (!(desc->cutoff > 0.f) || !(desc->bin_size_scale > 0.f)) return fail("cutoff and bin_size_scale must be > 0");
  if (n > kNoallocMaxCells)
    return fail("tecs_force_pass_noalloc: " + std::to_string(n) + " cells exceed the allocation-free limit of " +
                std::to_string(kNoallocMaxCells));
  // grid of binned_gabriel.hpp:28-42 / grid.hpp:201-215
  tecs_sim s;
  s.d = *desc;
  GridP& g = s.g;
  g.bin_size = desc->bin_size_scale * desc->cutoff;
  g.inv_bin = 1.0f / g.bin_size;
  g.R = (int)std::ceil(desc->cutoff * g.inv_bin);
  unsigned long long nb = 1;
  for (int k = 0; k < 3; ++k) { g.mn[k] = 0.f; g.ext[k] = 1; }
  for (int k = 0; k < desc->dims; ++k) {
    g.mn[k] = desc->min_bounds[k];
    g.ext[k] = (int)std::ceil((desc->max_bounds[k] - desc->min_bounds[k]) / g.bin_size);
    if (g.ext[k] < 1) return fail("max_bounds must exceed min_bounds");
    nb *= (unsigned long long)g.ext[k];
  }
  if (nb > kNoallocMaxBins)
    return fail("tecs_force_pass_noalloc: " + std::to_string(nb) + " bins exceed the allocation-free limit of " +
                std::to_string(kNoallocMaxBins));
  g.nbins = (unsigned)nb;
  grid_set_pow2(g);
  ForceP& f = s.fp;
  f.force = desc->force;
  f.k_rep = desc->k_rep; f.r_rep = desc->r_rep; f.k_adh = desc->k_adh; f.r_adh = desc->r_adh; f.k_pol = 0.f;
  f.rc2 = desc->cutoff * desc->cutoff;
  f.gab_factor = desc->gabriel_coefficient * desc->gabriel_coefficient * 0.25f;
  f.gab_csq = desc->gabriel_coefficient * desc->gabriel_coefficient;
  s.binned = true;
  s.fuse_count = false;
  // the device named by the description, as for every other entry point; its
  // scratch array is the one this call uses
  CK(cudaSetDevice(desc->device));
  unsigned char* base = nullptr;
  if (noalloc_scratch(desc->device, &base)) return -1;
  s.stream = (cudaStream_t)stream;
  s.d.capacity = n ? n : 1;
  s.d.division_probability = 0.0;
  s.n_host = n;
  s.ctr = (Counters*)(base + kOffCtr);
  s.A = (float4*)(base + kOffA);
  s.B = (float4*)(base + kOffB);
  s.d1 = (float4*)(base + kOffD);
  s.key = (unsigned*)(base + kOffKey);
  s.rank = (unsigned*)(base + kOffRank);
  s.src = (unsigned*)(base + kOffSrc);
  s.Bid = (unsigned*)(base + kOffBid);
  s.cnt = (unsigned*)(base + kOffCnt);
  s.off = (unsigned*)(base + kOffOff);
  s.part = (unsigned*)(base + kOffPart);
  // what must start at zero: the counters and the bin counts
  k_noalloc_reset<<<1, 32, 0, s.stream>>>(s.ctr, n);
  CK(cudaMemsetAsync(s.cnt, 0, ((size_t)g.nbins + 1) * 4, s.stream));
  if (n == 0) {
    CK(cudaGetLastError());
    return 0;
  }
  k_pack<<<ceil_div(n, 256), 256, 0, s.stream>>>(d_positions, n, desc->dims, s.A);
  int K = 0;
  if (enqueue_rebuild(&s, K, true)) return -1;
  PassArgs a = base_args(&s, 0.f);
  a.X = s.B;
  a.P = nullptr;
  a.mode = kStore;
  a.d_out = s.d1;
  a.dp_out = nullptr;
  a.count_next = 0;
  if (enqueue_pass(&s, a, K)) return -1;
  k_unpack<<<ceil_div(n, 256), 256, 0, s.stream>>>(s.B, s.Bid, s.d1, n, desc->dims, d_deltas);
  CK(cudaGetLastError());
  return 0;
}
