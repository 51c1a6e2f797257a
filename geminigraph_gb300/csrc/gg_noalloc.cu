// gg_active_edges_noalloc: the process_vertices reduction that feeds the
// sparse/dense switch (sum of out_degree over the set bits of a bitmap), for
// callers that must not allocate device memory.
//
// Some embedding applications cannot let a library call cudaMalloc: a
// serving process that reserves all of HBM for its own pool at start-up and
// hands out only pieces of it, or a caller on a latency-critical path where
// cudaMalloc/cudaFree would synchronise the device.  For them this entry
// point takes device inputs and a device output from the caller and uses, as
// its only scratch, the file-scope array below: GG_NOALLOC_MAX_SLICES uint64
// partial sums (32 KiB), which every GPU that loads the library holds until
// the process exits.  It calls no cudaMalloc, cudaFree or allocating library
// routine.
//
// Scratch use: slice s (vertices [s*65536, (s+1)*65536)) writes its partial
// sum to gg_noalloc_scratch[s]; the final kernel adds slots 0..slices-1 in
// order.  Every slot a call reads is written by the same call first, so
// nothing has to start at zero; the array keeps the last call's partials.
// All calls share the array: calls that overlap on the GPU (different
// streams, or host threads without ordering) race on it.
#include <mutex>

#include "gg_common.cuh"

namespace gg {

constexpr uint32_t NOALLOC_SLICE = 65536;  // vertices per partial sum
constexpr uint32_t NOALLOC_MAX_SLICES = GG_NOALLOC_MAX_VERTICES / NOALLOC_SLICE;
constexpr int NOALLOC_THREADS = 256;

static __device__ __align__(256) unsigned long long gg_noalloc_scratch[NOALLOC_MAX_SLICES];

// One block per slice; the block's partial is written (not added) to its slot.
__global__ void __launch_bounds__(NOALLOC_THREADS)
    noalloc_slice_sums(const uint32_t *__restrict__ bm, const uint32_t *__restrict__ deg, uint32_t V,
                       unsigned long long *__restrict__ partial) {
  __shared__ unsigned long long s_warp[NOALLOC_THREADS / 32];
  size_t v0 = (size_t)blockIdx.x * NOALLOC_SLICE;
  size_t v1 = v0 + NOALLOC_SLICE < V ? v0 + NOALLOC_SLICE : V;
  unsigned long long sum = 0;
  for (size_t wi = v0 / 32 + threadIdx.x; wi * 32 < v1; wi += NOALLOC_THREADS) {
    uint32_t w = bm[wi];
    while (w) {
      uint32_t b = __ffs(w) - 1;
      w &= w - 1;
      size_t v = wi * 32 + b;
      if (v < v1) sum += deg[v];
    }
  }
  sum = warp_sum(sum);
  if (lane_id() == 0) s_warp[threadIdx.x >> 5] = sum;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long t = 0;
    for (int i = 0; i < NOALLOC_THREADS / 32; i++) t += s_warp[i];
    partial[blockIdx.x] = t;
  }
}

__global__ void __launch_bounds__(NOALLOC_THREADS)
    noalloc_final(const unsigned long long *__restrict__ partial, uint32_t slices, unsigned long long *out) {
  __shared__ unsigned long long s_warp[NOALLOC_THREADS / 32];
  unsigned long long sum = 0;
  for (uint32_t i = threadIdx.x; i < slices; i += NOALLOC_THREADS) sum += partial[i];
  sum = warp_sum(sum);
  if (lane_id() == 0) s_warp[threadIdx.x >> 5] = sum;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long t = 0;
    for (int i = 0; i < NOALLOC_THREADS / 32; i++) t += s_warp[i];
    *out = t;
  }
}

// Device address of gg_noalloc_scratch per device, looked up once with that
// device current (in host code the symbol names a host-side stand-in).
static std::mutex g_noalloc_mu;
static unsigned long long *g_noalloc_ptr[64] = {};

static int noalloc_scratch(int device, unsigned long long **out) {
  if (device < 0 || device >= 64) {
    set_error("device %d out of range", device);
    return GG_ERR_INVALID;
  }
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_ptr[device]) {
    void *p = nullptr;
    GG_CUDA(cudaGetSymbolAddress(&p, gg_noalloc_scratch));
    g_noalloc_ptr[device] = (unsigned long long *)p;
  }
  *out = g_noalloc_ptr[device];
  return GG_OK;
}

}  // namespace gg

using namespace gg;

extern "C" int gg_active_edges_noalloc(const uint64_t *d_bitmap, const uint32_t *d_degree, uint32_t vertices,
                                       uint64_t *d_active_edges, void *stream) {
  if (!d_bitmap || !d_degree || !d_active_edges) {
    set_error("null argument");
    return GG_ERR_INVALID;
  }
  if (vertices > GG_NOALLOC_MAX_VERTICES) {
    set_error("gg_active_edges_noalloc: %u vertices exceed its fixed scratch (at most %u vertices)", vertices,
              (unsigned)GG_NOALLOC_MAX_VERTICES);
    return GG_ERR_LIMIT;
  }
  int device = 0;
  GG_CUDA(cudaGetDevice(&device));
  unsigned long long *partial = nullptr;
  GG_TRY(noalloc_scratch(device, &partial));
  cudaStream_t s = (cudaStream_t)stream;
  uint32_t slices = (uint32_t)(((uint64_t)vertices + NOALLOC_SLICE - 1) / NOALLOC_SLICE);
  if (slices)
    noalloc_slice_sums<<<slices, NOALLOC_THREADS, 0, s>>>((const uint32_t *)d_bitmap, d_degree, vertices, partial);
  noalloc_final<<<1, NOALLOC_THREADS, 0, s>>>(partial, slices, (unsigned long long *)d_active_edges);
  GG_CUDA(cudaGetLastError());
  GG_CUDA(cudaStreamSynchronize(s));
  return GG_OK;
}
