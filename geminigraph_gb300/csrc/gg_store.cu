// Graph store: edge list -> CSR (out) + CSC (in) on the device.
//
// Replaces Graph::load_directed (core/graph.hpp:771-1339) and
// Graph::load_undirected_from_directed (core/graph.hpp:349-757).  The
// reference makes five passes over the file with MPI self-shuffles and racing
// fetch_add fills; here every direction is one stable LSD radix sort of
// packed 64-bit (major << b | minor) keys on the device (b = bits of V-1),
// followed by a boundary pass that writes the offsets.  Lists come out sorted
// by neighbour id with duplicate edges in record order, so the build is
// deterministic.  Degrees are offset differences; symmetric graphs sort the
// records plus their reverses once and alias CSC = CSR (core/graph.hpp:733-738);
// their degree therefore counts both endpoints (core/graph.hpp:393-399).
#include <errno.h>
#include <fcntl.h>
#include <stdarg.h>
#include <string.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <chrono>
#include <thread>
#include <vector>

#include "gg_build.cuh"
#include "gg_common.cuh"
#include "gg_gen.h"
#include "gg_scan.cuh"

namespace gg {

// ------------------------------------------------------------------ errors
static thread_local char g_err[512] = "";

void set_error(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

int cuda_status(cudaError_t e, const char *what) {
  set_error("CUDA error %d (%s) in %s", (int)e, cudaGetErrorString(e), what);
  if (e == cudaErrorMemoryAllocation) return GG_ERR_NOMEM;
  return GG_ERR_CUDA;
}

size_t scan_scratch_elems(size_t n) { return scan_scratch_elems_impl(n) + 1; }

// ------------------------------------------------------------------ workspace
int ws_get(gg_graph *g, WsSlot slot, size_t bytes, void **out) {
  Workspace &w = g->ws;
  if (bytes == 0) bytes = 16;
  if (w.bytes[slot] < bytes) {
    if (w.ptr[slot]) GG_CUDA(cudaFree(w.ptr[slot]));
    w.ptr[slot] = nullptr;
    w.bytes[slot] = 0;
    GG_CUDA(cudaMalloc(&w.ptr[slot], bytes));
    w.bytes[slot] = bytes;
  }
  *out = w.ptr[slot];
  return GG_OK;
}

int ws_free_all(gg_graph *g) {
  Workspace &w = g->ws;
  for (int i = 0; i < WS_NSLOTS; i++) {
    if (w.ptr[i]) cudaFree(w.ptr[i]);
    w.ptr[i] = nullptr;
    w.bytes[i] = 0;
  }
  if (w.ctr) cudaFree(w.ctr);
  if (w.ctr_host) cudaFreeHost(w.ctr_host);
  if (w.stage) cudaFreeHost(w.stage);
  w.ctr = nullptr;
  w.ctr_host = nullptr;
  w.stage = nullptr;
  return GG_OK;
}

__global__ void copy_words_to_mapped(const uint32_t *__restrict__ src, uint32_t *dst, size_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    dst[i] = src[i];
}

int read_small(gg_graph *g, void *dst, const void *src, size_t bytes) {
  if (!g->ws.stage || bytes > STAGE_BYTES_HOST || (bytes & 3) || ((uintptr_t)src & 3)) {
    GG_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, g->stream));
    GG_CUDA(cudaStreamSynchronize(g->stream));
    return GG_OK;
  }
  copy_words_to_mapped<<<1, 256, 0, g->stream>>>((const uint32_t *)src, (uint32_t *)g->ws.stage, bytes / 4);
  GG_CUDA(cudaGetLastError());
  GG_CUDA(cudaStreamSynchronize(g->stream));
  memcpy(dst, g->ws.stage, bytes);
  return GG_OK;
}

int counters_reset(gg_graph *g) {
  GG_CUDA(cudaMemsetAsync(g->ws.ctr, 0, sizeof(Counters), g->stream));
  return GG_OK;
}

int counters_read(gg_graph *g, Counters *out) { return read_small(g, out, g->ws.ctr, sizeof(Counters)); }

int Trace::reserve_events(size_t n) {
  if (!st || !st->call_ms) return GG_OK;
  while (g->evpool.size() < ev.size() + n) {
    cudaEvent_t e;
    GG_CUDA(cudaEventCreate(&e));
    g->evpool.push_back(e);
  }
  return GG_OK;
}

// Inside a stream capture the record is made an external event node, which
// records the event when the graph runs (so that it can be timed); the flag
// is refused outside a capture.
int Trace::record(cudaEvent_t e) {
  if (capturing)
    GG_CUDA(cudaEventRecordWithFlags(e, g->stream, cudaEventRecordExternal));
  else
    GG_CUDA(cudaEventRecord(e, g->stream));
  return GG_OK;
}

int Trace::kbegin() {
  if (!timing()) return GG_OK;
  GG_TRY(reserve_events(2));
  cudaEvent_t e0 = g->evpool[ev.size()];
  ev.push_back(e0);
  ev_call.push_back(st->calls - 1);
  if (!replay) GG_TRY(record(e0));
  return GG_OK;
}

int Trace::kend() {
  if (!timing() || ev.size() % 2 == 0) return GG_OK;
  cudaEvent_t e1 = g->evpool[ev.size()];
  ev.push_back(e1);
  if (!replay) GG_TRY(record(e1));
  return GG_OK;
}

int Trace::collect() {
  if (!st || !st->call_ms) return GG_OK;
  for (size_t i = 0; i + 1 < ev.size(); i += 2) {
    float ms = 0;
    GG_CUDA(cudaEventSynchronize(ev[i + 1]));
    GG_CUDA(cudaEventElapsedTime(&ms, ev[i], ev[i + 1]));
    st->call_ms[ev_call[i / 2]] += ms;
  }
  ev.clear();
  ev_call.clear();
  return GG_OK;
}

// GG_CHECK builds: the run's bounds checks, read once it has finished.
int check_status(gg_graph *g) {
#if defined(GG_CHECK)
  static const char *const files[] = {"gg_engine.cuh", "gg_common.cuh", "gg_batched.cu", "gg_bc_batched.cu",
                                      "gg_store.cu",   "gg_bfs_pr.cu",  "gg_cc_sssp_bc.cu", "gg_partition.cu"};
  unsigned h[4] = {0, 0, 0, 0};
  GG_CUDA(cudaMemcpy(h, g->check_err, sizeof(h), cudaMemcpyDeviceToHost));
  if (h[0]) {
    const char *file = "?";
    for (const char *f : files)
      if (site_file_hash(f) == (h[0] >> 16)) file = f;
    GG_CUDA(cudaMemset(g->check_err, 0, sizeof(h)));
    set_error("device bounds check failed at %s:%u: index or vertex id %llu out of range (%u failures)", file,
              h[0] & 0xffffu, ((unsigned long long)h[2] << 32) | h[1], h[3]);
    return GG_ERR_CHECK;
  }
#else
  (void)g;
#endif
  return GG_OK;
}

int timed_begin(gg_graph *g) {
  GG_CUDA(cudaEventRecord(g->ev0, g->stream));
  return GG_OK;
}

int timed_end(gg_graph *g, gg_run_stats *st, int launches) {
  GG_CUDA(cudaEventRecord(g->ev1, g->stream));
  GG_CUDA(cudaEventSynchronize(g->ev1));
  GG_TRY(check_status(g));
  float ms = 0;
  GG_CUDA(cudaEventElapsedTime(&ms, g->ev0, g->ev1));
  if (st) {
    st->device_ms = ms;
    st->kernel_launches = launches;
  }
  return GG_OK;
}

// ------------------------------------------------------------------ radix sort
constexpr int RS_THREADS = 256;
constexpr int RS_ITEMS = 16;
constexpr int RS_TILE = RS_THREADS * RS_ITEMS;   // 4096 keys per tile
constexpr int RS_WARP_KEYS = 32 * RS_ITEMS;      // 512 consecutive keys per warp

__global__ void __launch_bounds__(RS_THREADS) rs_upsweep(const uint64_t *__restrict__ keys, size_t n, int shift,
                                                         uint32_t *__restrict__ counts, uint32_t ntiles) {
  __shared__ uint32_t hist[256];
  hist[threadIdx.x] = 0;
  __syncthreads();
  size_t base = (size_t)blockIdx.x * RS_TILE;
#pragma unroll 4
  for (int k = 0; k < RS_ITEMS; k++) {
    size_t idx = base + (size_t)k * RS_THREADS + threadIdx.x;
    if (idx < n) atomicAdd(&hist[(keys[idx] >> shift) & 255u], 1u);
  }
  __syncthreads();
  counts[(size_t)threadIdx.x * ntiles + blockIdx.x] = hist[threadIdx.x];
}

// Stable scatter of one tile.  Warp w ranks keys [w*512, w*512+512) of the
// tile in order (round r, lane) with __match_any_sync peer groups and a
// warp-private digit histogram; warps are then offset by the per-digit prefix
// over lower warps, and tiles by the digit-major scan of the upsweep counts.
__global__ void __launch_bounds__(RS_THREADS) rs_scatter(const uint64_t *__restrict__ kin,
                                                         const uint32_t *__restrict__ vin,
                                                         uint64_t *__restrict__ kout, uint32_t *__restrict__ vout,
                                                         size_t n, int shift, const uint32_t *__restrict__ scanned,
                                                         uint32_t ntiles) {
  __shared__ uint32_t whist[RS_THREADS / 32][256];
  __shared__ uint32_t gbase[256];
  for (int i = threadIdx.x; i < (RS_THREADS / 32) * 256; i += RS_THREADS) (&whist[0][0])[i] = 0;
  gbase[threadIdx.x] = scanned[(size_t)threadIdx.x * ntiles + blockIdx.x];
  __syncthreads();
  const unsigned w = threadIdx.x >> 5, lane = lane_id();
  const size_t base = (size_t)blockIdx.x * RS_TILE + (size_t)w * RS_WARP_KEYS;
  uint64_t key[RS_ITEMS];
  uint32_t val[RS_ITEMS];
  uint32_t rank[RS_ITEMS];
#pragma unroll
  for (int r = 0; r < RS_ITEMS; r++) {
    size_t idx = base + (size_t)r * 32 + lane;
    bool valid = idx < n;
    key[r] = valid ? kin[idx] : 0ull;
    val[r] = (vin && valid) ? vin[idx] : 0u;
    uint32_t d = valid ? (uint32_t)((key[r] >> shift) & 255u) : 256u + lane;
    unsigned peers = __match_any_sync(GG_FULL, d);
    unsigned leader = __ffs(peers) - 1;
    uint32_t cnt = valid ? whist[w][d] : 0u;
    __syncwarp();
    if (valid && lane == leader) whist[w][d] = cnt + __popc(peers);
    __syncwarp();
    rank[r] = cnt + __popc(peers & lanemask_lt());
  }
  __syncthreads();
  {
    uint32_t run = 0;
#pragma unroll
    for (int ww = 0; ww < RS_THREADS / 32; ww++) {
      uint32_t t = whist[ww][threadIdx.x];
      whist[ww][threadIdx.x] = run;
      run += t;
    }
  }
  __syncthreads();
#pragma unroll
  for (int r = 0; r < RS_ITEMS; r++) {
    size_t idx = base + (size_t)r * 32 + lane;
    if (idx < n) {
      uint32_t d = (uint32_t)((key[r] >> shift) & 255u);
      uint32_t pos = gbase[d] + whist[w][d] + rank[r];
      kout[pos] = key[r];
      if (vout) vout[pos] = val[r];
    }
  }
}

// Sorts n keys (and optional values) on the low `key_bits` bits.  Returns the
// buffers holding the result through *kres / *vres (either the inputs or the
// alternates).
int radix_sort(gg_graph *g, uint64_t *k0, uint32_t *v0, uint64_t *k1, uint32_t *v1, size_t n, int key_bits,
                      uint64_t **kres, uint32_t **vres) {
  *kres = k0;
  *vres = v0;
  if (n <= 1) return GG_OK;
  size_t ntiles = (n + RS_TILE - 1) / RS_TILE;
  size_t ncounts = 256 * ntiles;
  uint32_t *counts = nullptr, *scanned = nullptr, *scratch = nullptr;
  GG_CUDA(cudaMalloc(&counts, sizeof(uint32_t) * ncounts));
  GG_CUDA(cudaMalloc(&scanned, sizeof(uint32_t) * (ncounts + 1)));
  GG_CUDA(cudaMalloc(&scratch, sizeof(uint32_t) * scan_scratch_elems(ncounts)));
  uint64_t *ka = k0, *kb = k1;
  uint32_t *va = v0, *vb = v1;
  int status = GG_OK;
  for (int shift = 0; shift < key_bits; shift += 8) {
    rs_upsweep<<<(unsigned)ntiles, RS_THREADS, 0, g->stream>>>(ka, n, shift, counts, (uint32_t)ntiles);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess)
      e = exclusive_scan<uint32_t, ArrayIn<uint32_t>>(ArrayIn<uint32_t>{counts}, ncounts, scanned, scratch,
                                                      g->stream, nullptr);
    if (e == cudaSuccess) {
      rs_scatter<<<(unsigned)ntiles, RS_THREADS, 0, g->stream>>>(ka, va, kb, vb, n, shift, scanned,
                                                                 (uint32_t)ntiles);
      e = cudaGetLastError();
    }
    if (e != cudaSuccess) {
      status = cuda_status(e, "radix sort");
      break;
    }
    uint64_t *tk = ka; ka = kb; kb = tk;
    uint32_t *tv = va; va = vb; vb = tv;
  }
  cudaStreamSynchronize(g->stream);
  cudaFree(counts);
  cudaFree(scanned);
  cudaFree(scratch);
  *kres = ka;
  *vres = va;
  return status;
}

// ------------------------------------------------------------------ build kernels
// mode 0: key (src,dst); 1: key (dst,src); 2: both, records then reverses.
__global__ void make_keys(const uint32_t *__restrict__ rec, size_t E, int words, int mode, int bits, uint32_t V,
                          uint64_t *__restrict__ keys, uint32_t *__restrict__ vals, unsigned *err) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < E; i += (size_t)gridDim.x * blockDim.x) {
    uint32_t s = rec[i * words], d = rec[i * words + 1];
    uint32_t wb = words == 3 ? rec[i * words + 2] : 0u;
    if (s >= V || d >= V) {
      atomicOr(err, 1u);
      s = 0;
      d = 0;
    }
    uint64_t fwd = ((uint64_t)s << bits) | d, rev = ((uint64_t)d << bits) | s;
    if (mode == 0) {
      keys[i] = fwd;
    } else if (mode == 1) {
      keys[i] = rev;
    } else {
      keys[i] = fwd;
      keys[E + i] = rev;
    }
    if (vals) {
      vals[i] = wb;
      if (mode == 2) vals[E + i] = wb;
    }
  }
}

// off[v] = first position whose major id is >= v, for v in [0, V].
__global__ void offsets_from_keys(const uint64_t *__restrict__ keys, size_t n, int bits, uint32_t V,
                                  uint64_t *__restrict__ off, uint32_t *__restrict__ nbr) {
  const uint64_t mask = (bits >= 64) ? ~0ull : ((1ull << bits) - 1);
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    uint64_t k = keys[i];
    uint64_t maj = k >> bits;
    nbr[i] = (uint32_t)(k & mask);
    long long prev = i ? (long long)(keys[i - 1] >> bits) : -1ll;
    for (long long v = prev + 1; v <= (long long)maj; v++) off[v] = i;
    if (i == n - 1)
      for (uint64_t v = maj + 1; v <= V; v++) off[v] = n;
  }
}

// Bitmap of the vertices with deg > 0 (one warp per 32-bit word).
__global__ void nonzero_bitmap(const uint32_t *__restrict__ deg, uint32_t V, uint32_t *__restrict__ nz,
                               size_t words) {
  size_t nthreads = words * 32;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < nthreads; i += (size_t)gridDim.x * blockDim.x) {
    bool p = i < V && deg[i] > 0;
    unsigned b = __ballot_sync(GG_FULL, p);
    if ((threadIdx.x & 31) == 0) nz[i >> 5] = b;
  }
}

__global__ void degrees_from_offsets(const uint64_t *__restrict__ off, uint32_t V, uint32_t *__restrict__ deg) {
  for (size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (size_t)gridDim.x * blockDim.x)
    deg[v] = (uint32_t)(off[v + 1] - off[v]);
}

// 1 if LIGHT/HEAVY bin bounds lo < deg[i] <= hi.
struct DegInRange {
  const uint32_t *deg;
  uint32_t lo, hi;
  __device__ __forceinline__ uint32_t operator()(size_t i) const {
    uint32_t d = deg[i];
    return (d > lo && d <= hi) ? 1u : 0u;
  }
};

__global__ void compact_by_pos(const uint32_t *__restrict__ deg, uint32_t V, uint32_t lo, uint32_t hi,
                               const uint32_t *__restrict__ pos, uint32_t *__restrict__ out) {
  for (size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (size_t)gridDim.x * blockDim.x) {
    uint32_t d = deg[v];
    if (d > lo && d <= hi) out[pos[v]] = (uint32_t)v;
  }
}

struct ChunkCount {
  const uint32_t *list;
  const uint32_t *deg;
  uint32_t chunk;
  __device__ __forceinline__ uint32_t operator()(size_t i) const { return (deg[list[i]] + chunk - 1) / chunk; }
};

// Long lists are cut at absolute multiples of the chunk size in the adjacency
// array (so every chunk's 16-byte windows are aligned): a list [b, e) covers
// blocks b/chunk .. (e-1)/chunk.
struct AlignedChunkCount {
  const uint32_t *list;
  const uint64_t *off;
  uint32_t chunk;
  __device__ __forceinline__ uint32_t operator()(size_t i) const {
    const uint32_t v = list[i];
    const uint64_t b = off[v], e = off[v + 1];
    return e > b ? (uint32_t)((e - 1) / chunk - b / chunk + 1) : 0u;
  }
};

__global__ void fill_chunk_owner(const uint32_t *__restrict__ heavy_chunk, uint32_t nheavy,
                                 uint32_t *__restrict__ owner) {
  for (size_t h = (size_t)blockIdx.x * blockDim.x + threadIdx.x; h < nheavy; h += (size_t)gridDim.x * blockDim.x)
    for (uint32_t c = heavy_chunk[h]; c < heavy_chunk[h + 1]; c++) owner[c] = (uint32_t)h;
}

__global__ void gen_rmat_kernel(uint32_t *__restrict__ rec, uint64_t E, uint32_t scale, uint64_t key, int weighted) {
  int words = weighted ? 3 : 2;
  for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < E; e += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t s, d;
    gg_rmat_edge(key, scale, e, &s, &d);
    rec[e * words] = s;
    rec[e * words + 1] = d;
    if (weighted) rec[e * words + 2] = __float_as_uint(gg_gen_weight(key, e));
  }
}

__global__ void gen_grid_kernel(uint32_t *__restrict__ rec, uint64_t E, uint32_t n, uint64_t key, int weighted) {
  int words = weighted ? 3 : 2;
  for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < E; e += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t s, d;
    gg_grid_edge(n, e, &s, &d);
    rec[e * words] = s;
    rec[e * words + 1] = d;
    if (weighted) rec[e * words + 2] = __float_as_uint(gg_gen_weight(key, e));
  }
}

int bits_for(uint32_t V) {
  int b = 1;
  while (b < 32 && ((uint64_t)1 << b) < V) b++;
  return b;
}

// Ordered list of the vertices with lo < deg <= hi (scan + scatter).
static int bin_list(gg_graph *g, const Dir *d, uint32_t lo, uint32_t hi, uint32_t **list, uint32_t *count) {
  uint32_t V = g->V;
  uint32_t *pos = nullptr, *scratch = nullptr;
  GG_CUDA(cudaMalloc(&pos, sizeof(uint32_t) * ((size_t)V + 1)));
  GG_CUDA(cudaMalloc(&scratch, sizeof(uint32_t) * scan_scratch_elems(V)));
  GG_CUDA((exclusive_scan<uint32_t, DegInRange>(DegInRange{d->deg, lo, hi}, V, pos, scratch, g->stream, nullptr)));
  uint32_t n = 0;
  GG_CUDA(cudaMemcpyAsync(&n, pos + V, sizeof(uint32_t), cudaMemcpyDeviceToHost, g->stream));
  GG_CUDA(cudaStreamSynchronize(g->stream));
  GG_CUDA(cudaMalloc(list, sizeof(uint32_t) * (n ? n : 1)));
  if (n) {
    compact_by_pos<<<grid_for(V, 256, g->num_sms, 16), 256, 0, g->stream>>>(d->deg, V, lo, hi, pos, *list);
    GG_CUDA(cudaGetLastError());
  }
  GG_CUDA(cudaStreamSynchronize(g->stream));
  cudaFree(pos);
  cudaFree(scratch);
  *count = n;
  g->graph_bytes += sizeof(uint32_t) * n;
  return GG_OK;
}

// Chunk table of a vertex list: *prefix (n+1) of ceil(deg/chunk), *owner[c] =
// list index of chunk c.
static int chunk_table(gg_graph *g, const Dir *d, const uint32_t *list, uint32_t n, uint32_t chunk,
                       uint32_t **prefix, uint32_t **owner, uint32_t *nchunks, bool aligned = false) {
  GG_CUDA(cudaMalloc(prefix, sizeof(uint32_t) * ((size_t)n + 1)));
  uint32_t *scratch = nullptr;
  GG_CUDA(cudaMalloc(&scratch, sizeof(uint32_t) * scan_scratch_elems((size_t)n + 1)));
  if (aligned)
    GG_CUDA((exclusive_scan<uint32_t, AlignedChunkCount>(AlignedChunkCount{list, d->off, chunk}, n, *prefix, scratch,
                                                         g->stream, nullptr)));
  else
    GG_CUDA((exclusive_scan<uint32_t, ChunkCount>(ChunkCount{list, d->deg, chunk}, n, *prefix, scratch, g->stream,
                                                  nullptr)));
  uint32_t nc = 0;
  GG_CUDA(cudaMemcpyAsync(&nc, *prefix + n, sizeof(uint32_t), cudaMemcpyDeviceToHost, g->stream));
  GG_CUDA(cudaStreamSynchronize(g->stream));
  cudaFree(scratch);
  *nchunks = nc;
  GG_CUDA(cudaMalloc(owner, sizeof(uint32_t) * (nc ? nc : 1)));
  if (n) {
    fill_chunk_owner<<<grid_for(n, 128, g->num_sms, 8), 128, 0, g->stream>>>(*prefix, n, *owner);
    GG_CUDA(cudaGetLastError());
  }
  GG_CUDA(cudaStreamSynchronize(g->stream));
  g->graph_bytes += sizeof(uint32_t) * ((size_t)n + 1 + nc);
  return GG_OK;
}

// Degree bins of one direction (see Dir).
static int build_bins(gg_graph *g, Dir *d) {
  GG_TRY(bin_list(g, d, d->light, HEAVY_DEG, &d->med, &d->nmed));
  GG_TRY(bin_list(g, d, HEAVY_DEG, 0xffffffffu, &d->heavy, &d->nheavy));
  GG_TRY(chunk_table(g, d, d->heavy, d->nheavy, HEAVY_CHUNK, &d->heavy_chunk, &d->chunk_owner, &d->nchunks));
  GG_TRY(bin_list(g, d, d->light, 0xffffffffu, &d->big, &d->nbig));
  GG_TRY(chunk_table(g, d, d->big, d->nbig, d->chunk, &d->big_chunk, &d->big_owner, &d->nbigchunks, true));
  return GG_OK;
}

static void free_bins(gg_graph *g, Dir *d) {
  g->graph_bytes -= sizeof(uint32_t) * ((size_t)d->nmed + d->nheavy + d->nheavy + 1 + d->nchunks + d->nbig +
                                        d->nbig + 1 + d->nbigchunks);
  uint32_t *lists[] = {d->med, d->heavy, d->heavy_chunk, d->chunk_owner, d->big, d->big_chunk, d->big_owner};
  for (uint32_t *p : lists)
    if (p) cudaFree(p);
  d->med = d->heavy = d->heavy_chunk = d->chunk_owner = d->big = d->big_chunk = d->big_owner = nullptr;
  d->nmed = d->nheavy = d->nchunks = d->nbig = d->nbigchunks = 0;
}

// Rebuilds both directions' degree bins for a light-list bound and a pull
// chunk size (the autotuner's two knobs).
int rebuild_bins(gg_graph *g, uint32_t light, uint32_t chunk, uint32_t vec) {
  if (light < 1 || light > HEAVY_DEG || (chunk != 128 && chunk != 256 && chunk != 512) || vec > 3) {
    set_error("light list bound must be 1..%u, the pull chunk 128, 256 or 512 and the vector flags 0..3",
              HEAVY_DEG);
    return GG_ERR_INVALID;
  }
  g->out.vec = g->in.vec = g->pr.vec = vec;
  GG_CUDA(cudaSetDevice(g->device));
  GG_CUDA(cudaStreamSynchronize(g->stream));
  const bool alias = g->in.nbr == g->out.nbr;
  free_bins(g, &g->out);
  g->out.light = light;
  g->out.chunk = chunk;
  GG_TRY(build_bins(g, &g->out));
  if (alias) {
    g->in = g->out;
  } else {
    free_bins(g, &g->in);
    g->in.light = light;
    g->in.chunk = chunk;
    GG_TRY(build_bins(g, &g->in));
  }
  if (g->pr_ready) {
    free_bins(g, &g->pr);
    g->pr.light = light;
    g->pr.chunk = chunk;
    GG_TRY(build_bins(g, &g->pr));
  }
  if (g->pr_out_ready) {
    free_bins(g, &g->pr_out);
    g->pr_out.light = light;
    g->pr_out.chunk = chunk;
    GG_TRY(build_bins(g, &g->pr_out));
  }
  return GG_OK;
}

// Neighbour / weight storage: device memory, or mapped pinned host memory
// when the graph keeps its adjacency on the host (the kernels dereference
// the same pointer over NVLink-C2C; unified addressing makes the host and
// device addresses of a mapped allocation equal).
int adj_alloc(gg_graph *g, bool host, void **p, size_t bytes) {
  *p = nullptr;
  if (!host) {
    GG_CUDA(cudaMalloc(p, bytes));
    g->graph_bytes += bytes;
    return GG_OK;
  }
  GG_CUDA(cudaHostAlloc(p, bytes, cudaHostAllocMapped));
  void *dp = nullptr;
  cudaError_t e = cudaHostGetDevicePointer(&dp, *p, 0);
  if (e != cudaSuccess || dp != *p) {
    cudaFreeHost(*p);
    *p = nullptr;
    if (e != cudaSuccess) return cuda_status(e, "mapped adjacency");
    set_error("mapped host adjacency needs unified addressing");
    return GG_ERR_CUDA;
  }
  g->host_bytes += bytes;
  return GG_OK;
}

static void adj_release(bool host, void *p) {
  if (!p) return;
  if (host)
    cudaFreeHost(p);
  else
    cudaFree(p);
}

// Degrees (offset differences), the deg > 0 bitmap and the degree bins of a
// direction whose offsets are written.
int finish_dir(gg_graph *g, Dir *d) {
  const uint32_t V = g->V;
  d->nv = V;
  d->ne = g->nadj;
  d->err = g->check_err;
  degrees_from_offsets<<<grid_for(V, 256, g->num_sms, 16), 256, 0, g->stream>>>(d->off, V, d->deg);
  GG_CUDA(cudaGetLastError());
  size_t words = bitmap_words32(V);
  GG_CUDA(cudaMalloc(&d->nz, sizeof(uint32_t) * words));
  g->graph_bytes += sizeof(uint32_t) * words;
  nonzero_bitmap<<<grid_for(words * 32, 256, g->num_sms, 16), 256, 0, g->stream>>>(d->deg, V, d->nz, words);
  GG_CUDA(cudaGetLastError());
  GG_CUDA(cudaStreamSynchronize(g->stream));
  return build_bins(g, d);
}

// Builds one direction from keys already written by make_keys.
static int build_dir(gg_graph *g, uint64_t *keys, uint32_t *vals, uint64_t *k_alt, uint32_t *v_alt, size_t n,
                     int bits, Dir *d, bool weights = true, bool host = false) {
  uint64_t *ks;
  uint32_t *vs;
  GG_TRY(radix_sort(g, keys, vals, k_alt, v_alt, n, 2 * bits, &ks, &vs));
  uint32_t V = g->V;
  GG_CUDA(cudaMalloc(&d->off, sizeof(uint64_t) * ((size_t)V + 1)));
  // padded to a multiple of 64 entries: chunked pulls load whole aligned
  // 16-byte windows that may run past the last list
  const size_t npad = (n + 64) / 64 * 64;
  GG_TRY(adj_alloc(g, host, (void **)&d->nbr, sizeof(uint32_t) * npad));
  GG_CUDA(cudaMemsetAsync(d->nbr + n, 0, sizeof(uint32_t) * (npad - n), g->stream));
  GG_CUDA(cudaMalloc(&d->deg, sizeof(uint32_t) * ((size_t)V + 1)));
  g->graph_bytes += sizeof(uint64_t) * ((size_t)V + 1) + sizeof(uint32_t) * ((size_t)V + 1);
  if (n == 0) {
    GG_CUDA(cudaMemsetAsync(d->off, 0, sizeof(uint64_t) * ((size_t)V + 1), g->stream));
  } else {
    offsets_from_keys<<<grid_for(n, 256, g->num_sms, 16), 256, 0, g->stream>>>(ks, n, bits, V, d->off, d->nbr);
    GG_CUDA(cudaGetLastError());
  }
  if (g->weighted && weights) {
    GG_TRY(adj_alloc(g, host, (void **)&d->w, sizeof(float) * (n ? n : 1)));
    if (n) GG_CUDA(cudaMemcpyAsync(d->w, vs, sizeof(float) * n, cudaMemcpyDefault, g->stream));
  }
  return finish_dir(g, d);
}

static void free_dir(Dir *d, bool adj_host) {
  if (d->off) cudaFree(d->off);
  adj_release(adj_host, d->nbr);
  adj_release(adj_host, d->w);
  if (d->deg) cudaFree(d->deg);
  if (d->nz) cudaFree(d->nz);
  if (d->med) cudaFree(d->med);
  if (d->heavy) cudaFree(d->heavy);
  if (d->heavy_chunk) cudaFree(d->heavy_chunk);
  if (d->chunk_owner) cudaFree(d->chunk_owner);
  if (d->big) cudaFree(d->big);
  if (d->big_chunk) cudaFree(d->big_chunk);
  if (d->big_owner) cudaFree(d->big_owner);
  *d = Dir();
}

// ---------------------------------------------------------------- PageRank layout
// PageRank gathers source state once per edge; a source is gathered as
// often as its out-degree.  Renumbering vertices by descending out-degree
// packs the most gathered values into few cache lines (on R-MAT graphs the
// top 2^20 sources of scale 26 draw ~70% of the gathers), and sorting each
// in-list by the new numbers puts a hub's hottest in-neighbours side by side
// in one warp's loads.  The renumbered incoming adjacency is built once by
// the same radix sort as the load; ranks map back to vertex order on output.
__global__ void degree_rank_keys(const uint32_t *__restrict__ deg, uint32_t V, int bits, uint32_t dmax,
                                 uint64_t *__restrict__ keys) {
  for (size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (size_t)gridDim.x * blockDim.x) {
    const uint32_t dv = deg[v] < dmax ? deg[v] : dmax;
    keys[v] = ((uint64_t)(dmax - dv) << bits) | v;
  }
}

// keys: the V sorted degree keys, vertex id in the low `bits` bits.
__global__ void rank_tables(const uint64_t *__restrict__ keys, uint32_t V, int bits,
                            const uint32_t *__restrict__ out_deg, uint32_t *__restrict__ id_of_rank,
                            uint32_t *__restrict__ rank_of, uint32_t *__restrict__ od) {
  const uint64_t mask = (1ull << bits) - 1;
  for (size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x; r < V; r += (size_t)gridDim.x * blockDim.x) {
    const uint32_t v = (uint32_t)(keys[r] & mask);
    id_of_rank[r] = v;
    rank_of[v] = (uint32_t)r;
    od[r] = out_deg[v];
  }
}

// keys[k] = (rank(v) << bits) | rank(nbr[k]) for every entry k of v's in-list:
// lane per vertex for lists up to d.light, warp per long-list chunk.
__global__ void rank_edge_keys_light(Dir d, uint32_t V, int bits, const uint32_t *__restrict__ rank_of,
                                     uint64_t *__restrict__ keys) {
  for (size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (size_t)gridDim.x * blockDim.x) {
    const uint64_t b = d.off[v], e = d.off[v + 1];
    if (e - b > d.light) continue;
    const uint64_t hi = (uint64_t)rank_of[v] << bits;
    for (uint64_t k = b; k < e; k++) keys[k] = hi | rank_of[nbr_at(d, k, GG_SITE)];
  }
}

__global__ void rank_edge_keys_big(Dir d, int bits, const uint32_t *__restrict__ rank_of,
                                   uint64_t *__restrict__ keys) {
  const size_t nwarps = (size_t)gridDim.x * (blockDim.x / 32);
  for (size_t c = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) / 32; c < d.nbigchunks; c += nwarps) {
    uint32_t v;
    unsigned long long lo, b, e;
    big_range(d, (uint32_t)c, d.chunk, &v, &lo, &b, &e);
    const uint64_t hi = (uint64_t)rank_of[v] << bits;
    for (unsigned long long k = b + lane_id(); k < e; k += 32) keys[k] = hi | rank_of[nbr_at(d, k, GG_SITE)];
  }
}

// Frees a renumbered direction and its device bytes.
static void free_hot_dir(gg_graph *g, Dir *d) {
  const size_t V = g->V;
  free_bins(g, d);
  const size_t npad = (g->nadj + 64) / 64 * 64;
  g->graph_bytes -= sizeof(uint64_t) * (V + 1) + sizeof(uint32_t) * (npad + V + 1) +
                    sizeof(uint32_t) * bitmap_words32(g->V) + (d->w ? sizeof(float) * (g->nadj ? g->nadj : 1) : 0);
  if (d->off) cudaFree(d->off);
  if (d->nbr) cudaFree(d->nbr);
  if (d->w) cudaFree(d->w);
  if (d->deg) cudaFree(d->deg);
  if (d->nz) cudaFree(d->nz);
  *d = Dir();
}

void pr_layout_free(gg_graph *g) {
  if (!g->pr_ready) return;
  cudaStreamSynchronize(g->stream);
  const size_t V = g->V;
  g->graph_bytes -= sizeof(uint32_t) * 3 * V;
  free_hot_dir(g, &g->pr);
  if (g->pr_out_ready) free_hot_dir(g, &g->pr_out);
  g->pr_out_ready = false;
  cudaFree(g->pr_rank_of);
  cudaFree(g->pr_id_of_rank);
  cudaFree(g->pr_od);
  g->pr_rank_of = g->pr_id_of_rank = g->pr_od = nullptr;
  g->pr_ready = false;
}

// src renumbered: list of rank r = the list of vertex id_of_rank[r], its
// entries' neighbour ranks sorted ascending (weights carried along), built by
// the load's radix sort.
static int hot_dir(gg_graph *g, const Dir &src, Dir *dst, bool weights) {
  const uint32_t V = g->V;
  const size_t n = g->nadj;
  const int bits = bits_for(V);
  DevScratch tmp;
  uint64_t *k0 = nullptr, *k1 = nullptr;
  uint32_t *v0 = nullptr, *v1 = nullptr;
  GG_TRY(tmp.get(&k0, n));
  GG_TRY(tmp.get(&k1, n));
  if (weights) {
    GG_TRY(tmp.get(&v0, n));
    GG_TRY(tmp.get(&v1, n));
    if (n) GG_CUDA(cudaMemcpyAsync(v0, src.w, sizeof(float) * n, cudaMemcpyDefault, g->stream));
  }
  rank_edge_keys_light<<<grid_for(V, 256, g->num_sms, 16), 256, 0, g->stream>>>(src, V, bits, g->pr_rank_of, k0);
  if (src.nbigchunks)
    rank_edge_keys_big<<<grid_for((size_t)src.nbigchunks * 32, 256, g->num_sms, 16), 256, 0, g->stream>>>(
        src, bits, g->pr_rank_of, k0);
  GG_CUDA(cudaGetLastError());
  *dst = Dir();
  dst->light = src.light;
  dst->chunk = src.chunk;
  dst->vec = src.vec;
  GG_TRY(build_dir(g, k0, v0, k1, v1, n, bits, dst, weights, false));
  GG_CUDA(cudaStreamSynchronize(g->stream));
  return GG_OK;
}

int hot_out_build(gg_graph *g) {
  if (g->pr_out_ready) return GG_OK;
  GG_TRY(pr_layout_build(g));
  GG_CUDA(cudaSetDevice(g->device));
  const int s = hot_dir(g, g->out, &g->pr_out, g->weighted != 0);
  if (s != GG_OK) {
    free_hot_dir(g, &g->pr_out);
    return s;
  }
  g->pr_out_ready = true;
  return GG_OK;
}

int pr_layout_build(gg_graph *g) {
  if (g->pr_ready) return GG_OK;
  GG_CUDA(cudaSetDevice(g->device));
  const uint32_t V = g->V;
  const size_t n = g->nadj;
  const int bits = bits_for(V);
  int dbits = 1;
  while (dbits < 32 && (1ull << dbits) <= n) dbits++;
  const uint32_t dmax = dbits >= 32 ? 0xFFFFFFFFu : (uint32_t)((1ull << dbits) - 1);
  const size_t nk = V;  // degree keys of the ranking sort
  uint64_t *k0 = nullptr, *k1 = nullptr;
  GG_CUDA(cudaMalloc(&g->pr_rank_of, sizeof(uint32_t) * V));
  GG_CUDA(cudaMalloc(&g->pr_id_of_rank, sizeof(uint32_t) * V));
  GG_CUDA(cudaMalloc(&g->pr_od, sizeof(uint32_t) * V));
  g->graph_bytes += sizeof(uint32_t) * 3 * (size_t)V;
  int status = GG_OK;
  cudaError_t e = cudaMalloc(&k0, sizeof(uint64_t) * (nk ? nk : 1));
  if (e == cudaSuccess) e = cudaMalloc(&k1, sizeof(uint64_t) * (nk ? nk : 1));
  if (e != cudaSuccess) status = cuda_status(e, "PageRank layout keys");
  uint64_t *ks = nullptr;
  uint32_t *vs = nullptr;
  if (status == GG_OK) {
    degree_rank_keys<<<grid_for(V, 256, g->num_sms, 16), 256, 0, g->stream>>>(g->out.deg, V, bits, dmax, k0);
    status = radix_sort(g, k0, nullptr, k1, nullptr, V, bits + dbits, &ks, &vs);
  }
  if (status == GG_OK) {
    rank_tables<<<grid_for(V, 256, g->num_sms, 16), 256, 0, g->stream>>>(ks, V, bits, g->out.deg,
                                                                        g->pr_id_of_rank, g->pr_rank_of, g->pr_od);
    e = cudaGetLastError();
    if (e != cudaSuccess) status = cuda_status(e, "PageRank layout");
  }
  cudaStreamSynchronize(g->stream);
  if (k0) cudaFree(k0);
  if (k1) cudaFree(k1);
  // the incoming adjacency renumbered, with its weights when the graph has
  // them (SSSP's pulls gather them)
  if (status == GG_OK) {
    status = hot_dir(g, g->in, &g->pr, g->weighted != 0);
    if (status != GG_OK) free_hot_dir(g, &g->pr);
  }
  if (status != GG_OK) {
    cudaFree(g->pr_rank_of);
    cudaFree(g->pr_id_of_rank);
    cudaFree(g->pr_od);
    g->graph_bytes -= sizeof(uint32_t) * 3 * (size_t)V;
    g->pr_rank_of = g->pr_id_of_rank = g->pr_od = nullptr;
    return status;
  }
  g->pr_ready = true;
  return GG_OK;
}

void graph_destroy(gg_graph *g) {
  if (!g) return;
  cudaSetDevice(g->device);
  if (g->stream) cudaStreamSynchronize(g->stream);
  pools_destroy(g);
  for (cudaGraphExec_t &x : g->pr_exec) {
    if (x) cudaGraphExecDestroy(x);
    x = nullptr;
  }
  pr_layout_free(g);
  bool alias = g->in.nbr == g->out.nbr;
  free_dir(&g->out, g->adj_host);
  if (!alias) free_dir(&g->in, g->adj_host);
  ws_free_all(g);
  if (g->ev0) cudaEventDestroy(g->ev0);
  if (g->ev1) cudaEventDestroy(g->ev1);
  if (g->fork) cudaEventDestroy(g->fork);
  if (g->join) cudaEventDestroy(g->join);
  if (g->side) {
    cudaStreamSynchronize(g->side);
    cudaStreamDestroy(g->side);
  }
  for (cudaEvent_t e : g->evpool) cudaEventDestroy(e);
  if (g->check_err) cudaFree(g->check_err);
  if (g->stream) cudaStreamDestroy(g->stream);
  delete g;
}

static int graph_create(int device, uint32_t V, int weighted, int symmetric, gg_graph **out) {
  if (V == 0) {
    set_error("vertices must be > 0");
    return GG_ERR_INVALID;
  }
  int ndev = 0;
  GG_CUDA(cudaGetDeviceCount(&ndev));
  if (device < 0 || device >= ndev) {
    set_error("device %d out of range (%d devices)", device, ndev);
    return GG_ERR_INVALID;
  }
  GG_CUDA(cudaSetDevice(device));
  gg_graph *g = new gg_graph();
  g->device = device;
  g->V = V;
  g->weighted = weighted ? 1 : 0;
  g->symmetric = symmetric ? 1 : 0;
  cudaError_t e = cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&g->ev0);
  if (e == cudaSuccess) e = cudaEventCreate(&g->ev1);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&g->side, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&g->fork, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&g->join, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&g->num_sms, cudaDevAttrMultiProcessorCount, device);
  if (e == cudaSuccess) e = cudaMalloc(&g->check_err, 4 * sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMemset(g->check_err, 0, 4 * sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMalloc(&g->ws.ctr, sizeof(Counters));
  if (e == cudaSuccess) e = cudaMallocHost(&g->ws.ctr_host, sizeof(Counters));
  if (e == cudaSuccess) e = cudaHostAlloc(&g->ws.stage, STAGE_BYTES_HOST, cudaHostAllocMapped);
  if (e != cudaSuccess) {
    graph_destroy(g);
    return cuda_status(e, "graph create");
  }
  *out = g;
  return GG_OK;
}

// Builds CSR/CSC from E records in device memory (4-byte aligned).
int build_from_device_records(gg_graph *g, const uint32_t *rec, uint64_t E) {
  int words = g->weighted ? 3 : 2;
  g->E = E;
  size_t n = g->symmetric ? 2 * E : E;
  g->nadj = n;
  if (n >= 0xFFFFFFFFull) {
    set_error("%llu adjacency entries per direction: the device sort supports < 2^32",
              (unsigned long long)n);
    return GG_ERR_TOO_LARGE;
  }
  int bits = bits_for(g->V);
  uint64_t *k0 = nullptr, *k1 = nullptr;
  uint32_t *v0 = nullptr, *v1 = nullptr;
  unsigned *err = nullptr;
  int status = GG_OK;
  cudaError_t e = cudaMalloc(&k0, sizeof(uint64_t) * (n ? n : 1));
  if (e == cudaSuccess) e = cudaMalloc(&k1, sizeof(uint64_t) * (n ? n : 1));
  if (e == cudaSuccess && g->weighted) e = cudaMalloc(&v0, sizeof(uint32_t) * (n ? n : 1));
  if (e == cudaSuccess && g->weighted) e = cudaMalloc(&v1, sizeof(uint32_t) * (n ? n : 1));
  if (e == cudaSuccess) e = cudaMalloc(&err, sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMemsetAsync(err, 0, sizeof(unsigned), g->stream);
  if (e != cudaSuccess) status = cuda_status(e, "build buffers");
  unsigned blocks = grid_for(E, 256, g->num_sms, 16);
  for (int pass = 0; status == GG_OK && pass < (g->symmetric ? 1 : 2); pass++) {
    int mode = g->symmetric ? 2 : pass;
    if (E) {
      make_keys<<<blocks, 256, 0, g->stream>>>(rec, E, words, mode, bits, g->V, k0, v0, err);
      e = cudaGetLastError();
      if (e != cudaSuccess) {
        status = cuda_status(e, "make_keys");
        break;
      }
      unsigned herr = 0;
      e = cudaMemcpyAsync(&herr, err, sizeof(unsigned), cudaMemcpyDeviceToHost, g->stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
      if (e != cudaSuccess) {
        status = cuda_status(e, "make_keys");
        break;
      }
      if (herr) {
        set_error("an edge names a vertex id >= vertices (%u)", g->V);
        status = GG_ERR_RANGE;
        break;
      }
    }
    status = build_dir(g, k0, v0, k1, v1, n, bits, pass == 0 ? &g->out : &g->in, true, g->adj_host != 0);
  }
  cudaStreamSynchronize(g->stream);
  cudaFree(k0);
  cudaFree(k1);
  if (v0) cudaFree(v0);
  if (v1) cudaFree(v1);
  if (err) cudaFree(err);
  if (status == GG_OK && g->symmetric) g->in = g->out;
  return status;
}

static uint64_t unit_of(int weighted) { return weighted ? 12 : 8; }

}  // namespace gg

using namespace gg;

extern "C" {

const char *gg_last_error(void) { return g_err; }

int gg_host_alloc(uint64_t bytes, void **out) {
  if (!out) {
    set_error("null argument");
    return GG_ERR_INVALID;
  }
  GG_CUDA(cudaMallocHost(out, bytes ? bytes : 1));
  return GG_OK;
}

// core/graph.hpp:253-307 with one partition: the file is the array's bytes,
// vertex 0 first.  `array` may be host or device memory.
static bool is_device_ptr(const void *p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

int gg_dump_vertex_array(const void *array, uint64_t elem_size, uint32_t vertices, const char *path) {
  if (!array || !path || elem_size == 0) {
    set_error("null argument");
    return GG_ERR_INVALID;
  }
  const uint64_t bytes = elem_size * vertices;
  std::vector<char> stage;
  const char *src = (const char *)array;
  if (is_device_ptr(array)) {
    stage.resize(bytes);
    GG_CUDA(cudaMemcpy(stage.data(), array, bytes, cudaMemcpyDeviceToHost));
    src = stage.data();
  }
  FILE *f = fopen(path, "wb");
  if (!f) {
    set_error("cannot open %s for writing", path);
    return GG_ERR_IO;
  }
  const size_t n = fwrite(src, 1, bytes, f);
  const int rc = fclose(f);
  if (n != bytes || rc != 0) {
    set_error("short write to %s", path);
    return GG_ERR_IO;
  }
  return GG_OK;
}

int gg_restore_vertex_array(void *array, uint64_t elem_size, uint32_t vertices, const char *path) {
  if (!array || !path || elem_size == 0) {
    set_error("null argument");
    return GG_ERR_INVALID;
  }
  const uint64_t bytes = elem_size * vertices;
  FILE *f = fopen(path, "rb");
  if (!f) {
    set_error("cannot open %s", path);
    return GG_ERR_IO;
  }
  fseek(f, 0, SEEK_END);
  const long len = ftell(f);
  fseek(f, 0, SEEK_SET);
  if (len < 0 || (uint64_t)len != bytes) {
    fclose(f);
    set_error("%s holds %ld bytes, the array %llu", path, len, (unsigned long long)bytes);
    return GG_ERR_INVALID;
  }
  std::vector<char> stage;
  const bool dev = is_device_ptr(array);
  char *dst = (char *)array;
  if (dev) {
    stage.resize(bytes);
    dst = stage.data();
  }
  const size_t n = fread(dst, 1, bytes, f);
  fclose(f);
  if (n != bytes) {
    set_error("short read from %s", path);
    return GG_ERR_IO;
  }
  if (dev) GG_CUDA(cudaMemcpy(array, stage.data(), bytes, cudaMemcpyHostToDevice));
  return GG_OK;
}

int gg_host_free(void *p) {
  if (p) GG_CUDA(cudaFreeHost(p));
  return GG_OK;
}

int gg_graph_from_device_records(const void *d_records, uint64_t bytes, uint32_t vertices, int weighted,
                                 int symmetric, int device, gg_graph **out) {
  if (!out || (!d_records && bytes >= unit_of(weighted))) {
    set_error("null argument");
    return GG_ERR_INVALID;
  }
  if ((uintptr_t)d_records % 4) {
    set_error("device records must be 4-byte aligned");
    return GG_ERR_INVALID;
  }
  gg_graph *g = nullptr;
  GG_TRY(graph_create(device, vertices, weighted, symmetric, &g));
  const uint64_t E = bytes / unit_of(weighted);
  bool part = false;
  uint64_t cap = 0, gcap = 0;
  int s = build_plan(g, E, true, nullptr, &part, &cap, &gcap);
  if (s == GG_OK) s = build_records(g, (const uint32_t *)d_records, E, part, cap, gcap, nullptr);
  if (s != GG_OK) {
    graph_destroy(g);
    return s;
  }
  *out = g;
  return GG_OK;
}

// Device-readable view of host records for the partitioned build: device
// or pinned memory as it is, anything else registered for the call.
struct RecordsView {
  const uint32_t *dev = nullptr;
  void *registered = nullptr;
  void *staged = nullptr;  // pinned copy when the range cannot be registered
  RecordsView() = default;
  RecordsView(const RecordsView &) = delete;
  RecordsView &operator=(const RecordsView &) = delete;
  ~RecordsView() {
    if (registered) cudaHostUnregister(registered);
    if (staged) cudaFreeHost(staged);
  }
};

static int records_view(const void *records, uint64_t bytes, RecordsView *rv) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, records) != cudaSuccess) {
    cudaGetLastError();
    a.type = cudaMemoryTypeUnregistered;
  }
  if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) {
    rv->dev = (const uint32_t *)records;
    return GG_OK;
  }
  if (a.type == cudaMemoryTypeHost && a.devicePointer) {
    rv->dev = (const uint32_t *)a.devicePointer;
    return GG_OK;
  }
  void *p = const_cast<void *>(records);
  cudaError_t e = cudaHostRegister(p, bytes, cudaHostRegisterMapped | cudaHostRegisterReadOnly);
  if (e != cudaSuccess) {
    cudaGetLastError();
    e = cudaHostRegister(p, bytes, cudaHostRegisterMapped);
  }
  void *dp = nullptr;
  if (e == cudaSuccess) {
    rv->registered = p;
    GG_CUDA(cudaHostGetDevicePointer(&dp, p, 0));
  } else {
    // e.g. the range shares pages with memory registered elsewhere
    cudaGetLastError();
    GG_CUDA(cudaHostAlloc(&rv->staged, bytes, cudaHostAllocMapped));
    memcpy(rv->staged, records, bytes);
    GG_CUDA(cudaHostGetDevicePointer(&dp, rv->staged, 0));
  }
  rv->dev = (const uint32_t *)dp;
  return GG_OK;
}

static double wall_ms_since(const std::chrono::steady_clock::time_point &t0) {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

static int graph_create_opts(int device, uint32_t V, int weighted, int symmetric, const gg_build_options *opt,
                             gg_graph **out) {
  GG_TRY(graph_create(device, V, weighted, symmetric, out));
  if (opt && opt->adjacency_host) {
    (*out)->adj_host = 1;
    (*out)->pr_layout = 0;
  }
  if (opt && (opt->force_partitions < 0 || opt->force_partitions > OC_MAX_FORCED)) {
    graph_destroy(*out);
    *out = nullptr;
    set_error("force_partitions must be in [0, %d]", OC_MAX_FORCED);
    return GG_ERR_INVALID;
  }
  return GG_OK;
}

int gg_graph_from_records_ex(const void *records, uint64_t bytes, uint32_t vertices, int weighted, int symmetric,
                             int device, gg_build_options *opt, gg_graph **out) {
  const auto t0 = std::chrono::steady_clock::now();
  uint64_t unit = unit_of(weighted);
  uint64_t E = bytes / unit;
  if (!out || (!records && E)) {
    set_error("null argument");
    return GG_ERR_INVALID;
  }
  if ((uintptr_t)records % 4) {
    set_error("records must be 4-byte aligned");
    return GG_ERR_INVALID;
  }
  gg_graph *g = nullptr;
  GG_TRY(graph_create_opts(device, vertices, weighted, symmetric, opt, &g));
  bool part = false;
  uint64_t cap = 0, gcap = 0;
  int s = build_plan(g, E, false, opt, &part, &cap, &gcap);
  if (s == GG_OK && !part) {
    void *d = nullptr;
    cudaError_t e = cudaMalloc(&d, E * unit ? E * unit : 16);
    if (e == cudaSuccess && E) e = cudaMemcpy(d, records, E * unit, cudaMemcpyDefault);
    s = e == cudaSuccess ? build_records(g, (const uint32_t *)d, E, false, 0, 0, opt) : cuda_status(e, "copy records");
    if (d) cudaFree(d);
  } else if (s == GG_OK) {
    RecordsView rv;
    s = E ? records_view(records, E * unit, &rv) : GG_OK;
    if (s == GG_OK) s = build_records(g, rv.dev, E, true, cap, gcap, opt);
    cudaStreamSynchronize(g->stream);
  }
  if (s != GG_OK) {
    graph_destroy(g);
    return s;
  }
  if (opt) opt->build_ms = wall_ms_since(t0);
  *out = g;
  return GG_OK;
}

int gg_graph_from_records(const void *records, uint64_t bytes, uint32_t vertices, int weighted, int symmetric,
                          int device, gg_graph **out) {
  return gg_graph_from_records_ex(records, bytes, vertices, weighted, symmetric, device, nullptr, out);
}

// Reads [0, bytes) of fd into dst with several threads.
static int read_parallel(int fd, char *dst, uint64_t bytes, const char *path) {
  const int T = 8;
  const uint64_t per = (bytes / T + 4095) / 4096 * 4096;
  std::vector<std::thread> th;
  std::vector<int> bad(T, 0);
  for (int t = 0; t < T; t++) {
    const uint64_t a = per * t, b = std::min<uint64_t>(bytes, per * (t + 1));
    if (a >= b) break;
    th.emplace_back([=, &bad]() {
      uint64_t off = a;
      while (off < b) {
        const size_t want = (size_t)std::min<uint64_t>(b - off, (uint64_t)1 << 30);
        ssize_t r = pread(fd, dst + off, want, (off_t)off);
        if (r <= 0) {
          bad[t] = 1;
          return;
        }
        off += (uint64_t)r;
      }
    });
  }
  for (auto &x : th) x.join();
  for (int t = 0; t < T; t++)
    if (bad[t]) {
      set_error("read error on %s", path);
      return GG_ERR_IO;
    }
  return GG_OK;
}

int gg_graph_load(const char *path, uint32_t vertices, int weighted, int symmetric, int device, gg_graph **out) {
  return gg_graph_load_ex(path, vertices, weighted, symmetric, device, nullptr, out);
}

int gg_graph_load_ex(const char *path, uint32_t vertices, int weighted, int symmetric, int device,
                     gg_build_options *opt, gg_graph **out) {
  const auto t0 = std::chrono::steady_clock::now();
  if (!path || !out) {
    set_error("null argument");
    return GG_ERR_INVALID;
  }
  int fd = open(path, O_RDONLY);
  if (fd < 0) {
    set_error("cannot open %s: %s", path, strerror(errno));
    return GG_ERR_IO;
  }
  struct stat st;
  if (fstat(fd, &st) != 0) {
    set_error("cannot stat %s: %s", path, strerror(errno));
    close(fd);
    return GG_ERR_IO;
  }
  uint64_t unit = unit_of(weighted);
  uint64_t E = (uint64_t)st.st_size / unit;
  uint64_t total = E * unit;
  gg_graph *g = nullptr;
  int s = graph_create_opts(device, vertices, weighted, symmetric, opt, &g);
  if (s != GG_OK) {
    close(fd);
    return s;
  }
  bool part = false;
  uint64_t cap = 0, gcap = 0;
  s = build_plan(g, E, false, opt, &part, &cap, &gcap);
  if (s == GG_OK && part) {
    // records stay in mapped pinned host memory, read by the build kernels
    char *h = nullptr;
    cudaError_t e = cudaHostAlloc((void **)&h, total ? total : 16, cudaHostAllocMapped);
    if (e != cudaSuccess) s = cuda_status(e, "pinned records");
    if (s == GG_OK) s = read_parallel(fd, h, total, path);
    close(fd);
    void *dp = nullptr;
    if (s == GG_OK) {
      e = cudaHostGetDevicePointer(&dp, h, 0);
      if (e != cudaSuccess) s = cuda_status(e, "pinned records");
    }
    if (s == GG_OK) s = build_records(g, (const uint32_t *)dp, E, true, cap, gcap, opt);
    cudaStreamSynchronize(g->stream);
    if (h) cudaFreeHost(h);
    if (s != GG_OK) {
      graph_destroy(g);
      return s;
    }
    if (opt) opt->build_ms = wall_ms_since(t0);
    *out = g;
    return GG_OK;
  }
  if (s != GG_OK) {
    close(fd);
    graph_destroy(g);
    return s;
  }
  // stream the file through two pinned chunks
  const size_t CH = (size_t)64 << 20;
  char *pin[2] = {nullptr, nullptr};
  cudaEvent_t done[2] = {nullptr, nullptr};
  char *d = nullptr;
  cudaError_t e = cudaMalloc((void **)&d, total ? total : 16);
  for (int i = 0; i < 2 && e == cudaSuccess; i++) {
    e = cudaMallocHost((void **)&pin[i], CH);
    if (e == cudaSuccess) e = cudaEventCreate(&done[i]);
  }
  if (e != cudaSuccess) s = cuda_status(e, "load buffers");
  uint64_t off = 0;
  int k = 0;
  while (s == GG_OK && off < total) {
    size_t want = (size_t)((total - off) < CH ? (total - off) : CH);
    e = cudaEventSynchronize(done[k]);
    if (e != cudaSuccess) {
      s = cuda_status(e, "load");
      break;
    }
    size_t got = 0;
    while (got < want) {
      ssize_t r = pread(fd, pin[k] + got, want - got, (off_t)(off + got));
      if (r <= 0) {
        set_error("read error on %s at %llu", path, (unsigned long long)(off + got));
        s = GG_ERR_IO;
        break;
      }
      got += (size_t)r;
    }
    if (s != GG_OK) break;
    e = cudaMemcpyAsync(d + off, pin[k], want, cudaMemcpyHostToDevice, g->stream);
    if (e == cudaSuccess) e = cudaEventRecord(done[k], g->stream);
    if (e != cudaSuccess) {
      s = cuda_status(e, "load copy");
      break;
    }
    off += want;
    k ^= 1;
  }
  close(fd);
  cudaStreamSynchronize(g->stream);
  for (int i = 0; i < 2; i++) {
    if (pin[i]) cudaFreeHost(pin[i]);
    if (done[i]) cudaEventDestroy(done[i]);
  }
  if (s == GG_OK) s = build_records(g, (const uint32_t *)d, E, false, 0, 0, opt);
  if (d) cudaFree(d);
  if (s != GG_OK) {
    graph_destroy(g);
    return s;
  }
  if (opt) opt->build_ms = wall_ms_since(t0);
  *out = g;
  return GG_OK;
}

uint64_t gg_generate_count(int kind, uint32_t p1, uint32_t p2) {
  if (kind == 0) return p1 > 31 ? 0 : ((uint64_t)1 << p1) * p2;
  if (kind == 1) return gg_grid_count(p1);
  return 0;
}

int gg_generate_records(int kind, uint32_t p1, uint32_t p2, uint64_t seed, int weighted, void *records,
                        int threads) {
  uint64_t E = gg_generate_count(kind, p1, p2);
  if ((kind != 0 && kind != 1) || (kind == 0 && (p1 < 1 || p1 > 31)) || (!records && E)) {
    set_error("bad generator arguments");
    return GG_ERR_INVALID;
  }
  if (threads <= 0) threads = (int)std::thread::hardware_concurrency();
  if (threads <= 0) threads = 1;
  uint64_t key = gg_gen_key(seed);
  int words = weighted ? 3 : 2;
  uint32_t *rec = (uint32_t *)records;
  auto work = [&](uint64_t a, uint64_t b) {
    for (uint64_t e = a; e < b; e++) {
      uint32_t s, d;
      if (kind == 0)
        gg_rmat_edge(key, p1, e, &s, &d);
      else
        gg_grid_edge(p1, e, &s, &d);
      rec[e * words] = s;
      rec[e * words + 1] = d;
      if (weighted) {
        float w = gg_gen_weight(key, e);
        memcpy(&rec[e * words + 2], &w, 4);
      }
    }
  };
  std::vector<std::thread> pool;
  uint64_t chunk = (E + threads - 1) / threads;
  for (int t = 0; t < threads; t++) {
    uint64_t a = (uint64_t)t * chunk, b = a + chunk < E ? a + chunk : E;
    if (a >= b) break;
    pool.emplace_back(work, a, b);
  }
  for (auto &th : pool) th.join();
  return GG_OK;
}

int gg_graph_generate(int kind, uint32_t p1, uint32_t p2, uint64_t seed, int weighted, int symmetric, int device,
                      gg_graph **out) {
  return gg_graph_generate_ex(kind, p1, p2, seed, weighted, symmetric, device, nullptr, out);
}

int gg_graph_generate_ex(int kind, uint32_t p1, uint32_t p2, uint64_t seed, int weighted, int symmetric, int device,
                         gg_build_options *opt, gg_graph **out) {
  const auto t0 = std::chrono::steady_clock::now();
  uint64_t E = gg_generate_count(kind, p1, p2);
  uint32_t V;
  if (kind == 0 && p1 >= 1 && p1 <= 31) {
    V = 1u << p1;
  } else if (kind == 1 && p1 >= 1 && (uint64_t)p1 * p1 < 0xFFFFFFFFull) {
    V = p1 * p1;
  } else {
    set_error("bad generator arguments");
    return GG_ERR_INVALID;
  }
  if (!out) {
    set_error("null argument");
    return GG_ERR_INVALID;
  }
  gg_graph *g = nullptr;
  GG_TRY(graph_create_opts(device, V, weighted, symmetric, opt, &g));
  uint32_t *d = nullptr;
  int words = weighted ? 3 : 2;
  cudaError_t e = cudaMalloc(&d, E ? E * words * 4 : 16);
  uint64_t key = gg_gen_key(seed);
  if (e == cudaSuccess && E) {
    unsigned blocks = grid_for(E, 256, g->num_sms, 32);
    if (kind == 0)
      gen_rmat_kernel<<<blocks, 256, 0, g->stream>>>(d, E, p1, key, weighted);
    else
      gen_grid_kernel<<<blocks, 256, 0, g->stream>>>(d, E, p1, key, weighted);
    e = cudaGetLastError();
  }
  bool part = false;
  uint64_t cap = 0, gcap = 0;
  int s = e == cudaSuccess ? build_plan(g, E, true, opt, &part, &cap, &gcap) : cuda_status(e, "generate");
  if (s == GG_OK) s = build_records(g, d, E, part, cap, gcap, opt);
  if (d) cudaFree(d);
  if (s != GG_OK) {
    graph_destroy(g);
    return s;
  }
  if (opt) opt->build_ms = wall_ms_since(t0);
  *out = g;
  return GG_OK;
}

int gg_graph_free(gg_graph *g) {
  graph_destroy(g);
  return GG_OK;
}

int gg_graph_info_get(const gg_graph *g, gg_graph_info *info) {
  if (!g || !info) {
    set_error("null argument");
    return GG_ERR_INVALID;
  }
  info->vertices = g->V;
  info->edges = g->E;
  info->adj_entries = g->nadj;
  info->weighted = g->weighted;
  info->symmetric = g->symmetric;
  info->transposed = g->transposed;
  info->device = g->device;
  uint64_t ws_bytes = 0;
  for (int i = 0; i < WS_NSLOTS; i++) ws_bytes += g->ws.bytes[i];
  info->device_bytes = g->graph_bytes + ws_bytes;
  info->host_bytes = g->host_bytes;
  return GG_OK;
}

int gg_graph_transpose(gg_graph *g) {
  if (!g) {
    set_error("null argument");
    return GG_ERR_INVALID;
  }
  pr_layout_free(g);
  Dir t = g->out;
  g->out = g->in;
  g->in = t;
  g->transposed ^= 1;
  return GG_OK;
}

int gg_graph_device_view(const gg_graph *g, int incoming, gg_device_adj *out) {
  if (!g || !out) {
    set_error("null argument");
    return GG_ERR_INVALID;
  }
  const Dir &d = incoming ? g->in : g->out;
  out->offsets = d.off;
  out->neighbours = d.nbr;
  out->weights = d.w;
  out->degree = d.deg;
  out->vertices = g->V;
  out->entries = g->nadj;
  out->edges = g->E;
  out->device = g->device;
  return GG_OK;
}

int gg_graph_adjacency(const gg_graph *g, int incoming, uint64_t *offsets, uint32_t *neighbours, float *weights,
                       uint32_t *degree) {
  if (!g) {
    set_error("null argument");
    return GG_ERR_INVALID;
  }
  GG_CUDA(cudaSetDevice(g->device));
  const Dir &d = incoming ? g->in : g->out;
  if (offsets) GG_CUDA(cudaMemcpy(offsets, d.off, sizeof(uint64_t) * ((size_t)g->V + 1), cudaMemcpyDeviceToHost));
  if (neighbours && g->nadj)
    GG_CUDA(cudaMemcpy(neighbours, d.nbr, sizeof(uint32_t) * g->nadj, cudaMemcpyDefault));
  if (weights && g->weighted && g->nadj)
    GG_CUDA(cudaMemcpy(weights, d.w, sizeof(float) * g->nadj, cudaMemcpyDefault));
  if (degree) GG_CUDA(cudaMemcpy(degree, d.deg, sizeof(uint32_t) * g->V, cudaMemcpyDeviceToHost));
  return GG_OK;
}

int gg_is_sparse(uint64_t active_edges, uint64_t edges) { return active_edges < edges / 20 ? 1 : 0; }

const void *gg_result_device_ptr(const gg_graph *g, int which) {
  if (!g || which < 0 || which > 1) return nullptr;
  return g->result[which];
}

}  // extern "C"
