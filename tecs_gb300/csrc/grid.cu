// grid.cu -- the standalone bin grid of the C ABI (tecs_grid_*).
//
// The counterpart of the reference's acceleration::Grid
// (include/utils/grid.hpp:29-638): a uniform grid of bins over fixed bounds,
// rebuilt over a point set by the same counting sort as the force passes
// (k_count -> k_scan_* -> k_scatter -> k_order_gather: points sorted by
// (bin, index)), and queried on the device (tecs/device/grid_query.cuh).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>

#include "../../include/tecs_gpu.h"
#include "../../include/tecs/device/grid_query.cuh"
#include "../../include/tecs/device/kernels.cuh"

using namespace tecs;

namespace tecs {
int set_last_error(const std::string& m);
}

namespace {
#define GCK(call)                                                                                         \
  do {                                                                                                    \
    cudaError_t e_ = (call);                                                                              \
    if (e_ != cudaSuccess) return set_last_error(std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

unsigned cdiv(unsigned long long a, unsigned b) { return (unsigned)((a + b - 1) / b); }

__global__ void k_grid_pack(const float* __restrict__ in, unsigned n, int dims, float4* __restrict__ A,
                            Counters* __restrict__ ctr) {
  if (blockIdx.x == 0 && threadIdx.x == 0) ctr->n = n;
  for (unsigned s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
    float4 v = make_float4(0.f, 0.f, 0.f, __uint_as_float(s));
    v.x = in[(size_t)s * dims];
    if (dims >= 2) v.y = in[(size_t)s * dims + 1];
    if (dims >= 3) v.z = in[(size_t)s * dims + 2];
    A[s] = v;
  }
}

struct MaskFilter {
  const unsigned char* eligible;
  __device__ bool operator()(int j) const { return !eligible || eligible[j] != 0; }
};

__global__ void k_grid_query(GridDev G, int kind, const float* __restrict__ q, unsigned m, int radius_bins,
                             float radius, const unsigned* __restrict__ draws,
                             const unsigned char* __restrict__ eligible, int* __restrict__ out) {
  for (unsigned k = blockIdx.x * blockDim.x + threadIdx.x; k < m; k += gridDim.x * blockDim.x) {
    float p[3] = {0.f, 0.f, 0.f};
    for (int d = 0; d < G.dims; ++d) p[d] = q[(size_t)k * G.dims + d];
    int r = -1;
    if (kind == TECS_GRID_NEAREST) r = grid_nearest(G, p, radius_bins);
    else if (kind == TECS_GRID_RANDOM_IN_BINS) r = grid_random_in_bins(G, p, radius_bins, draws[k]);
    else r = grid_random_in_radius(G, p, radius, draws[k], MaskFilter{eligible});
    out[k] = r;
  }
}
}  // namespace

struct tecs_grid {
  int device = 0;
  int dims = 3;
  unsigned cap = 0;
  GridP g{};
  cudaStream_t stream = nullptr;
  float4 *A = nullptr, *B = nullptr;
  unsigned *Bid = nullptr, *key = nullptr, *rank = nullptr, *src = nullptr, *cnt = nullptr, *off = nullptr,
           *part = nullptr;
  Counters* ctr = nullptr;
  float* stage = nullptr;
  unsigned n = 0;
  bool built = false;
  // query buffers, grown on demand
  float* q = nullptr;
  unsigned* draws = nullptr;
  int* out = nullptr;
  unsigned char* eligible = nullptr;
  unsigned qcap = 0;
};

namespace {
int grid_free_queries(tecs_grid* G) {
  for (void* p : {(void*)G->q, (void*)G->draws, (void*)G->out, (void*)G->eligible})
    if (p) cudaFree(p);
  G->q = nullptr;
  G->draws = nullptr;
  G->out = nullptr;
  G->eligible = nullptr;
  G->qcap = 0;
  return 0;
}

int grid_rebuild_from_device(tecs_grid* G, const float* pts, unsigned n) {
  const unsigned gb = std::max(1u, cdiv(n, 256));
  k_grid_pack<<<gb, 256, 0, G->stream>>>(pts, n, G->dims, G->A, G->ctr);
  const unsigned len = G->g.nbins + 1;
  const unsigned chunks = cdiv(len, kScanChunk);
  const unsigned pw = (unsigned)scan_part_words(len);
  k_count<<<gb, 256, 0, G->stream>>>(G->A, G->ctr, G->g, G->dims, G->key, G->rank, G->cnt, nullptr);
  if (chunks > 1) {
    GCK(cudaMemsetAsync(G->part + chunks, 0, (size_t)(pw - chunks) * 4, G->stream));
    k_scan_reduce<<<chunks, kScanThreads, 0, G->stream>>>(G->cnt, len, G->part);
  }
  k_scan_apply<<<chunks, kScanThreads, 0, G->stream>>>(G->cnt, len, G->part, G->off);
  k_scatter<<<gb, 256, 0, G->stream>>>(G->ctr, G->key, G->rank, G->off, G->src, G->part, 0u);
  k_order_gather<<<gb, 256, 0, G->stream>>>(G->ctr, G->key, G->off, G->src, G->A, nullptr, G->B, nullptr, G->Bid,
                                            nullptr, ExtraMove{0, 0, nullptr, nullptr});
  GCK(cudaGetLastError());
  GCK(cudaStreamSynchronize(G->stream));
  G->n = n;
  G->built = true;
  return 0;
}
}  // namespace

extern "C" {

int tecs_grid_create(int dims, const float* min_bounds, const float* max_bounds, float bin_size, unsigned capacity,
                     int device, tecs_grid** out) {
  if (!min_bounds || !max_bounds || !out) return set_last_error("null argument");
  *out = nullptr;
  if (dims != 2 && dims != 3) return set_last_error("dims must be 2 or 3");
  if (!(bin_size > 0.f)) return set_last_error("bin size must be > 0");
  GCK(cudaSetDevice(device));
  tecs_grid* G = new tecs_grid();
  G->device = device;
  G->dims = dims;
  G->cap = capacity ? capacity : 1;
  GridP& g = G->g;
  g.bin_size = bin_size;
  g.inv_bin = 1.0f / bin_size;
  g.R = 1;
  unsigned long long nb = 1;
  for (int k = 0; k < 3; ++k) { g.mn[k] = 0.f; g.ext[k] = 1; }
  for (int k = 0; k < dims; ++k) {
    g.mn[k] = min_bounds[k];
    // grid.hpp:201-206: ceil((max - min) / bin_size)
    g.ext[k] = (int)std::ceil((max_bounds[k] - min_bounds[k]) / bin_size);
    if (g.ext[k] < 1) { delete G; return set_last_error("max_bounds must exceed min_bounds"); }
    nb *= (unsigned long long)g.ext[k];
  }
  if (nb > (1ull << 31)) { delete G; return set_last_error("bin grid too large"); }
  g.nbins = (unsigned)nb;
  grid_set_pow2(g);
  const size_t cap = G->cap, len = (size_t)g.nbins + 1;
  auto al = [](void** p, size_t b) { return cudaMalloc(p, b ? b : 16) == cudaSuccess; };
  bool ok = cudaStreamCreateWithFlags(&G->stream, cudaStreamNonBlocking) == cudaSuccess;
  ok = ok && al((void**)&G->A, cap * 16) && al((void**)&G->B, cap * 16) && al((void**)&G->Bid, cap * 4) &&
       al((void**)&G->key, cap * 4) && al((void**)&G->rank, cap * 4) && al((void**)&G->src, cap * 4) &&
       al((void**)&G->cnt, len * 4) && al((void**)&G->off, len * 4) &&
       al((void**)&G->part, scan_part_words(len) * 4) && al((void**)&G->ctr, sizeof(Counters)) &&
       al((void**)&G->stage, cap * (size_t)dims * 4);
  // the counts start at zero (each scan leaves them zero again); cleared on
  // the grid's own non-blocking stream, which later work is ordered after
  ok = ok && cudaMemsetAsync(G->cnt, 0, len * 4, G->stream) == cudaSuccess &&
       cudaMemsetAsync(G->off, 0, len * 4, G->stream) == cudaSuccess &&
       cudaMemsetAsync(G->ctr, 0, sizeof(Counters), G->stream) == cudaSuccess &&
       cudaStreamSynchronize(G->stream) == cudaSuccess;
  if (!ok) {
    const std::string m = std::string("grid allocation failed: ") + cudaGetErrorString(cudaGetLastError());
    tecs_grid_destroy(G);
    return set_last_error(m);
  }
  *out = G;
  return 0;
}

int tecs_grid_destroy(tecs_grid* G) {
  if (!G) return 0;
  cudaSetDevice(G->device);
  if (G->stream) cudaStreamSynchronize(G->stream);
  grid_free_queries(G);
  for (void* p : {(void*)G->A, (void*)G->B, (void*)G->Bid, (void*)G->key, (void*)G->rank, (void*)G->src,
                  (void*)G->cnt, (void*)G->off, (void*)G->part, (void*)G->ctr, (void*)G->stage})
    if (p) cudaFree(p);
  if (G->stream) cudaStreamDestroy(G->stream);
  delete G;
  return 0;
}

int tecs_grid_rebuild(tecs_grid* G, const float* points, unsigned n) {
  if (!G || (n && !points)) return set_last_error("null argument");
  if (n > G->cap) return set_last_error("point count exceeds the grid's capacity");
  GCK(cudaSetDevice(G->device));
  if (n) GCK(cudaMemcpyAsync(G->stage, points, (size_t)n * G->dims * 4, cudaMemcpyHostToDevice, G->stream));
  return grid_rebuild_from_device(G, G->stage, n);
}

int tecs_grid_rebuild_device(tecs_grid* G, const float* d_points, unsigned n) {
  if (!G || (n && !d_points)) return set_last_error("null argument");
  if (n > G->cap) return set_last_error("point count exceeds the grid's capacity");
  GCK(cudaSetDevice(G->device));
  return grid_rebuild_from_device(G, d_points, n);
}

int tecs_grid_query(tecs_grid* G, int kind, const float* queries, unsigned m, int radius_bins, float radius,
                    const uint32_t* draws, const uint8_t* eligible, int32_t* out) {
  if (!G || (m && (!queries || !out))) return set_last_error("null argument");
  if (kind < TECS_GRID_NEAREST || kind > TECS_GRID_RANDOM_IN_RADIUS) return set_last_error("unknown query kind");
  if (kind != TECS_GRID_NEAREST && m && !draws) return set_last_error("random queries need draws");
  if (kind != TECS_GRID_RANDOM_IN_RADIUS && radius_bins < 0) return set_last_error("radius_bins must be >= 0");
  if (kind == TECS_GRID_RANDOM_IN_RADIUS && !(radius >= 0.f)) return set_last_error("radius must be >= 0");
  if (!G->built) return set_last_error("the grid was never rebuilt");
  if (m == 0) return 0;
  GCK(cudaSetDevice(G->device));
  if (m > G->qcap) {
    grid_free_queries(G);
    const size_t qm = m;
    if (cudaMalloc((void**)&G->q, qm * G->dims * 4) != cudaSuccess ||
        cudaMalloc((void**)&G->draws, qm * 4) != cudaSuccess || cudaMalloc((void**)&G->out, qm * 4) != cudaSuccess ||
        cudaMalloc((void**)&G->eligible, (size_t)G->cap) != cudaSuccess) {
      grid_free_queries(G);
      return set_last_error("grid query allocation failed");
    }
    G->qcap = m;
  }
  GCK(cudaMemcpyAsync(G->q, queries, (size_t)m * G->dims * 4, cudaMemcpyHostToDevice, G->stream));
  if (draws) GCK(cudaMemcpyAsync(G->draws, draws, (size_t)m * 4, cudaMemcpyHostToDevice, G->stream));
  if (eligible && G->n)
    GCK(cudaMemcpyAsync(G->eligible, eligible, (size_t)G->n, cudaMemcpyHostToDevice, G->stream));
  GridDev D{G->g, G->dims, G->B, G->Bid, G->off};
  k_grid_query<<<std::max(1u, cdiv(m, 128)), 128, 0, G->stream>>>(D, kind, G->q, m, radius_bins, radius, G->draws,
                                                                  eligible ? G->eligible : nullptr, G->out);
  GCK(cudaGetLastError());
  GCK(cudaMemcpyAsync(out, G->out, (size_t)m * 4, cudaMemcpyDeviceToHost, G->stream));
  GCK(cudaStreamSynchronize(G->stream));
  return 0;
}

int tecs_grid_device_view(const tecs_grid* G, const void** sorted_positions, const unsigned** sorted_index,
                          const unsigned** bin_offsets) {
  if (!G || !sorted_positions || !sorted_index || !bin_offsets) return set_last_error("null argument");
  *sorted_positions = G->B;
  *sorted_index = G->Bid;
  *bin_offsets = G->off;
  return 0;
}

}  // extern "C"
