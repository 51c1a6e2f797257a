// Shared device-side definitions of the GB300 edge-processing engine.
//
// Memory layout in HBM (one graph, one GPU):
//   out.off  uint64[V+1]  CSR offsets (grouped by source, "outgoing")
//   out.nbr  uint32[A]    CSR neighbour ids, sorted ascending in each list
//   out.w    float[A]     CSR edge weights (weighted graphs only), parallel array
//   out.deg  uint32[V]    out_degree (core/graph.hpp:110)
//   in.*                  the same for the CSC (grouped by destination)
// A = adjacency entries per direction = E (directed) or 2E (symmetric, where
// in.* aliases out.*, as core/graph.hpp:733-738 does).
// Vertex subsets are bitmaps in the reference's layout (core/bitmap.hpp:
// bit v%64 of 64-bit word v/64, V/64+1 words).  On a little-endian device the
// same bytes read as uint32 words give bit v%32 of word v/32, so kernels use
// 32-bit words and one warp owns the word of its 32 consecutive vertices.
#ifndef GG_COMMON_CUH
#define GG_COMMON_CUH

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include <stdint.h>
#include <stdio.h>

#include <string>
#include <type_traits>
#include <vector>

#include "../../include/gemini_gb300.h"

#define GG_WARP 32
#define GG_FULL 0xffffffffu

namespace gg {

// ---------------------------------------------------------------- errors
void set_error(const char *fmt, ...);
int cuda_status(cudaError_t e, const char *what);

#define GG_CUDA(call)                                 \
  do {                                                \
    cudaError_t _e = (call);                          \
    if (_e != cudaSuccess) return ::gg::cuda_status(_e, #call); \
  } while (0)

#define GG_TRY(call)            \
  do {                          \
    int _s = (call);            \
    if (_s != GG_OK) return _s; \
  } while (0)

// ---------------------------------------------------------------- graph
// Degree bins of one direction, built once at load time (the GB300 form of
// Graph::tune_chunks, core/graph.hpp:1341-1404): pull kernels give a light
// list (deg <= LIGHT_DEG) one lane, a medium list one warp, and split every
// heavy list (deg > HEAVY_DEG) into HEAVY_CHUNK-edge chunks, one block each.
constexpr uint32_t LIGHT_DEG = 32;     // default light-list bound (Dir.light; autotuned)
constexpr uint32_t HEAVY_DEG = 2048;
constexpr uint32_t HEAVY_CHUNK = 2048;
constexpr uint32_t PULL_CHUNK = 256;   // default reduction-pull chunk (Dir.chunk; autotuned)

struct Dir {
  uint32_t light = LIGHT_DEG;       // lists up to this long are "light" (one lane)
  uint32_t chunk = PULL_CHUNK;      // edges per warp work item of the reduction pulls
  uint32_t vec = 1;                 // chunked pulls: 1 = 16-byte window per lane, 0 = lane-strided entries
  uint64_t *off = nullptr;
  uint32_t *nbr = nullptr;
  float *w = nullptr;
  uint32_t *deg = nullptr;
  uint32_t *nz = nullptr;           // bitmap: deg > 0
  uint32_t *med = nullptr;          // LIGHT_DEG < deg <= HEAVY_DEG, ascending
  uint32_t nmed = 0;
  uint32_t *heavy = nullptr;        // deg > HEAVY_DEG, ascending
  uint32_t nheavy = 0;
  uint32_t *heavy_chunk = nullptr;  // nheavy+1: prefix of per-vertex chunk counts
  uint32_t *chunk_owner = nullptr;  // nchunks: index into heavy of each chunk
  uint32_t nchunks = 0;
  uint32_t *big = nullptr;          // deg > LIGHT_DEG, ascending (reduction pulls)
  uint32_t nbig = 0;
  uint32_t *big_chunk = nullptr;    // nbig+1: prefix of per-vertex chunk counts (aligned blocks, see big_range)
  uint32_t *big_owner = nullptr;    // nbigchunks: index into big of each chunk
  uint32_t nbigchunks = 0;
  // bounds of the ids and entries, and the graph's error word (GG_CHECK builds)
  uint32_t nv = 0;
  uint64_t ne = 0;
  unsigned *err = nullptr;
};

// Per-call counters written by the activation epilogue of every edge kernel.
struct Counters {
  unsigned long long edges;     // sum of out_degree over newly activated vertices
  unsigned long long in_edges;  // sum of in_degree over newly activated vertices
  unsigned int activated;       // vertices whose active_out bit this call set
  unsigned int qlen;            // entries appended to the output queue
  double delta;                 // PageRank delta accumulator
  unsigned int err;             // device-side error flag (bounds checks)
  unsigned int maxdeg;          // largest out_degree among newly activated vertices
};

enum WsSlot {
  WS_BM0, WS_BM1, WS_BM2, WS_BM3,       // bitmaps
  WS_Q0, WS_Q1, WS_QLEV,                // queues / level order
  WS_PREFIX,                            // uint64 prefix of queue degrees
  WS_MSG,                               // per-queue-entry message snapshot (4 or 8 B)
  WS_S0, WS_S1, WS_S2, WS_S3,           // vertex state arrays
  WS_SCAN,                              // scan scratch
  WS_HUBSUM,                            // per-iteration counters (PageRank)
  WS_PARTIAL,                           // per-chunk partial results of heavy lists
  WS_PIPE,                              // second result buffer of the pipelined calls
  WS_QPOS,                              // per-word queue positions (queue_from_bitmap)
  WS_STAMP,                             // per-vertex activation stamps (small sparse runs)
  WS_SMALL,                             // SmallRun state and its trace rows
  WS_MS_VISIT, WS_MS_FRONT, WS_MS_NEXT, // batched traversals: lane masks
  WS_MS_LVL, WS_MS_PAR, WS_MS_DIST,     // batched traversals: per-lane state (vertex-major)
  WS_MS_MISC, WS_MS_ROOTS,              // batched traversals: counters, roots
  WS_MS_OUT0, WS_MS_OUT1,               // batched traversals: lane-major results
  WS_SCAN32,                            // scan scratch for 32-bit scans
  WS_NSLOTS
};

struct Workspace {
  void *ptr[WS_NSLOTS] = {};
  size_t bytes[WS_NSLOTS] = {};
  Counters *ctr = nullptr;       // device
  Counters *ctr_host = nullptr;  // pinned mirror
  void *stage = nullptr;         // page-locked, device-mapped staging for read_small
};
constexpr size_t STAGE_BYTES_HOST = 64 * 1024;

class LanePool;
void pools_destroy(gg_graph *g);
int pr_layout_build(gg_graph *g);
int hot_out_build(gg_graph *g);
void pr_layout_free(gg_graph *g);

}  // namespace gg

// Everything the launches of a captured PageRank run depend on: the kernels'
// arguments and grids, the buffers and events.  A run whose key equals the
// cached one replays the cached CUDA graph.
struct PrGraphKey {
  gg::Dir din;
  const void *od, *buf0, *buf1, *out, *per_iter, *partial;
  uint32_t V;
  int32_t iterations, tsize, ranked, timing;
  uint32_t hot;
  uint32_t split;
  cudaStream_t side;
};

struct gg_graph {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // second stream of the reduction pulls: the light-list kernel runs beside
  // the chunk kernel (fork / join events)
  cudaStream_t side = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
  uint32_t V = 0;
  uint64_t E = 0;
  uint64_t nadj = 0;
  int weighted = 0, symmetric = 0, transposed = 0;
  gg::Dir out, in;
  gg::Workspace ws;
  uint64_t graph_bytes = 0;
  // neighbour and weight arrays in mapped pinned host memory (kernels read
  // them over NVLink-C2C); offsets, degrees and bins stay in device memory
  int adj_host = 0;
  uint64_t host_bytes = 0;
  int num_sms = 0;
  const void *result[2] = {nullptr, nullptr};
  std::vector<cudaEvent_t> evpool;  // events for per-call kernel timing
  gg::LanePool *pool_bfs = nullptr;  // lane pools of the batched calls
  gg::LanePool *pool_sssp = nullptr;
  // PageRank's hot-source layout of the incoming adjacency (built on the
  // first PageRank call, dropped by transpose): vertices renumbered by
  // descending out-degree, so the ranks gathered most often sit together.
  gg::Dir pr;
  uint32_t *pr_rank_of = nullptr;     // V: new number of vertex v
  uint32_t *pr_id_of_rank = nullptr;  // V: vertex with new number r
  uint32_t *pr_od = nullptr;          // V: out-degree in the new numbering
  bool pr_ready = false;
  // the outgoing adjacency in the same numbering (directed graphs; built on
  // demand by SSSP, whose push steps walk out-lists)
  gg::Dir pr_out;
  bool pr_out_ready = false;
  int pr_layout = 1;                  // 0: PageRank pulls the plain incoming adjacency
  // batched SSSP bucket width (0: plain Bellman-Ford rounds) and the least
  // edge weight (bucketing needs none negative), found on first use
  float sssp_delta = 0.0f;
  // batched BFS steps pull (dense) when the union frontier's out-edges reach
  // edges / batched_switch_div, else push
  uint32_t batched_switch_div = 20;
  // batched SSSP steps with at most this many lanes in flight relax edges
  // one thread per edge (msp_push_thread) instead of one warp per edge
  uint32_t batched_thread_lanes = 16;
  // batched BFS / SSSP (without buckets) run their steps device-driven: a
  // CUDA graph whose loop node repeats one step, no host wait between steps
  // (off by default: measured slower than one host wait per step)
  int batched_graph = 0;
  // gg_bfs_batched without parents keeps the lanes' levels as level lists
  // (one 16-byte entry per vertex and step that reached it) rather than
  // 256-byte rows per vertex
  int batched_lists = 1;
  // reduction pulls whose light and chunk kernels run side by side: blocks
  // per SM of the light kernel (the chunk kernel gets the other 8 - n), so
  // the two share every SM from the start; 0: each launched over all SMs
  uint32_t pull_light_blocks = 0;
  // gg_bfs calls run the pull kernels when active out-edges >= E / this
  // (20: the reference's switch; the trace always records the reference's mode)
  uint32_t bfs_pull_div = 20;
  int wmin_known = 0;
  float wmin = 0.0f;
  // reduction pulls on the hot-source layout: gathered state of the first
  // l1_hot_bytes worth of sources is cached in L1, the rest read past it
  uint32_t l1_hot_bytes = 0xffffffffu;
  // device error word of the bounds checks of a GG_CHECK build: first
  // failing site, its value (low, high), number of failures
  unsigned *check_err = nullptr;
  // CC and SSSP: a dense call (by the reference's switch) whose active
  // out-edges are below nadj / dense_push_div runs the push kernels over the
  // frontier instead of pulling every in-list (0: always pull; 4 measured
  // best for SSSP on R-MAT 25, neutral for CC on R-MAT 26)
  uint32_t dense_push_div = 4;
  // PageRank's iterations captured as one CUDA graph, replayed while the key
  // (arguments, buffers, events) is unchanged
  cudaGraphExec_t pr_exec[2] = {nullptr, nullptr};  // float, double
  PrGraphKey pr_key[2];
};

namespace gg {

// ---------------------------------------------------------------- host helpers
int ws_get(gg_graph *g, WsSlot slot, size_t bytes, void **out);
template <typename T>
inline int ws(gg_graph *g, WsSlot slot, size_t count, T **out) {
  return ws_get(g, slot, count * sizeof(T), (void **)out);
}
int ws_free_all(gg_graph *g);
int counters_reset(gg_graph *g);
int counters_read(gg_graph *g, Counters *out);
// Small device-to-host reads on the graph's stream, copied by the SMs into
// page-locked device-mapped memory: they do not wait behind a large
// copy-engine transfer running on another stream (pipelined result copies).
// Waits for the stream.
int read_small(gg_graph *g, void *dst, const void *src, size_t bytes);

inline size_t bitmap_words32(uint32_t V) { return 2 * ((size_t)V / 64 + 1); }
inline unsigned grid_for(size_t work, int threads, int num_sms, int per_sm = 8) {
  size_t blocks = (work + threads - 1) / threads;
  size_t cap = (size_t)num_sms * per_sm;
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  return (unsigned)blocks;
}

// Exclusive scan of `in(i)` for i < n into out[0..n] (out[n] = total).
// Three-phase (tile reduce, recursive scan of tile sums, tile scan): no
// inter-block waiting.  scratch must hold scan_scratch_elems(n) elements.
size_t scan_scratch_elems(size_t n);

// Stats/trace helper for toolkits: one row per process_edges call, and, when
// the caller passed call_ms, CUDA events around each call's edge kernel.
// Per-call record of a toolkit run (the process_edges trace), and the NVTX
// ranges a profiler cuts the run by: one range named after the run (when a
// name is given), and
// inside it one range per process_edges call ("process_edges sparse" or
// "process_edges dense", payload = the call's active_edges), which holds the
// call's kernel launches.  Calls that a cooperative small-run launch
// executes on the device are recorded after it and get empty ranges.
struct Trace {
  gg_run_stats *st;
  gg_graph *g;
  std::vector<int> ev_call;
  std::vector<cudaEvent_t> ev;
  int nvtx_depth = 0;
  // replay of a captured run: kbegin / kend name the events the graph
  // records instead of recording them
  bool replay = false;
  bool capturing = false;  // the graph's stream is being captured
  int record(cudaEvent_t e);
  Trace(gg_run_stats *s, gg_graph *gr, const char *run = nullptr) : st(s), g(gr) {
    if (run) {
      nvtxRangePushA(run);
      nvtx_depth = 1;
    }
    if (st) {
      st->calls = 0;
      st->active_edges_total = 0;
      st->device_ms = 0;
      st->kernel_launches = 0;
    }
  }
  ~Trace() {
    for (; nvtx_depth > 0; nvtx_depth--) nvtxRangePop();
  }
  Trace(const Trace &) = delete;
  Trace &operator=(const Trace &) = delete;
  void call_range(int mode, uint64_t active_edges) {
    if (nvtx_depth == 0) return;
    if (nvtx_depth == 2) {
      nvtxRangePop();
      nvtx_depth = 1;
    }
    nvtxEventAttributes_t a = {};
    a.version = NVTX_VERSION;
    a.size = NVTX_EVENT_ATTRIB_STRUCT_SIZE;
    a.messageType = NVTX_MESSAGE_TYPE_ASCII;
    a.message.ascii = mode ? "process_edges dense" : "process_edges sparse";
    a.payloadType = NVTX_PAYLOAD_TYPE_UNSIGNED_INT64;
    a.payload.ullValue = active_edges;
    if (nvtx_depth == 1) {
      nvtxRangePushEx(&a);
      nvtx_depth = 2;
    }
  }
  void add(int mode, uint64_t active_edges, uint64_t activated) {
    call_range(mode, active_edges);
    if (!st) return;
    int i = st->calls;
    if (i < st->trace_capacity) {
      if (st->mode) st->mode[i] = mode;
      if (st->active_edges) st->active_edges[i] = active_edges;
      if (st->activated) st->activated[i] = activated;
      if (st->call_ms) st->call_ms[i] = 0.0;
    }
    st->calls = i + 1;
    st->active_edges_total += active_edges;
  }
  void set_activated(uint64_t activated) {
    if (!st) return;
    int i = st->calls - 1;
    if (i >= 0 && i < st->trace_capacity && st->activated) st->activated[i] = activated;
  }
  bool timing() const { return st && st->call_ms && st->calls >= 1 && st->calls - 1 < st->trace_capacity; }
  int timing_requested() const { return st && st->call_ms ? 1 + st->trace_capacity : 0; }
  int kbegin();
  int kend();
  int reserve_events(size_t n);  // before a capture: no event is created inside it
  int collect();  // after the stream has been synchronised
};

int check_status(gg_graph *g);
int timed_begin(gg_graph *g);
int timed_end(gg_graph *g, gg_run_stats *st, int launches);

// ---------------------------------------------------------------- device helpers
__device__ __forceinline__ bool bm_test(const uint32_t *bm, uint32_t v) {
  return (bm[v >> 5] >> (v & 31)) & 1u;
}
__device__ __forceinline__ bool bm_test_ldg(const uint32_t *__restrict__ bm, uint32_t v) {
  return (__ldg(bm + (v >> 5)) >> (v & 31)) & 1u;
}
// Sets bit v; returns true if it was clear before (this thread activated v).
__device__ __forceinline__ bool bm_set_atomic(uint32_t *bm, uint32_t v) {
  uint32_t bit = 1u << (v & 31);
  if (bm[v >> 5] & bit) return false;
  return !(atomicOr(bm + (v >> 5), bit) & bit);
}

__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }

// Chunk c of the long-list table: owner vertex v, aligned block start lo
// (a multiple of chunk in the adjacency array) and the list's part [b, e)
// inside [lo, lo + chunk).
__device__ __forceinline__ void big_range(const Dir &d, uint32_t c, uint32_t chunk, uint32_t *v,
                                          unsigned long long *lo, unsigned long long *b,
                                          unsigned long long *e) {
  const uint32_t o = d.big_owner[c];
  *v = d.big[o];
  const unsigned long long b0 = d.off[*v], e0 = d.off[*v + 1];
  *lo = (b0 / chunk + (c - d.big_chunk[o])) * (unsigned long long)chunk;
  *b = b0 > *lo ? b0 : *lo;
  *e = e0 < *lo + chunk ? e0 : *lo + chunk;
}

// ---------------------------------------------------------------- bounds checks
// A GG_CHECK build (libgemini_gb300_check.so) checks every adjacency entry
// index against the direction's entries and every neighbour id read from the
// adjacency against the vertex count before it is used.  A failing check
// records its site (16-bit hash of the source file name, line) and value in
// the graph's error word, substitutes 0 so that no access leaves its array,
// and the run returns GG_ERR_CHECK.  Other builds compile the plain loads.
constexpr uint32_t site_file_hash(const char *f) {
  const char *b = f;
  for (const char *p = f; *p; p++)
    if (*p == '/') b = p + 1;
  uint32_t h = 2166136261u;
  for (const char *p = b; *p; p++) h = (h ^ (uint32_t)(unsigned char)*p) * 16777619u;
  return (h ^ (h >> 16)) & 0xffffu;
}
#define GG_SITE \
  (std::integral_constant<uint32_t, (gg::site_file_hash(__FILE__) << 16) | ((uint32_t)__LINE__ & 0xffffu)>::value)

__device__ __forceinline__ void check_fail(unsigned *err, uint32_t site, unsigned long long value) {
  if (!err) return;
  if (atomicCAS(err, 0u, site) == 0u) {
    err[1] = (unsigned)value;
    err[2] = (unsigned)(value >> 32);
  }
  atomicAdd(err + 3, 1u);
}
// The neighbour id of entry k of direction d.
__device__ __forceinline__ uint32_t nbr_at(const Dir &d, unsigned long long k, uint32_t site) {
#if defined(GG_CHECK)
  if (k >= d.ne) {
    check_fail(d.err, site, k);
    return 0u;
  }
  const uint32_t u = d.nbr[k];
  if (u >= d.nv) {
    check_fail(d.err, site, u);
    return 0u;
  }
  return u;
#else
  (void)site;
  return d.nbr[k];
#endif
}
// A vertex id loaded some other way (vector loads, queues).
__device__ __forceinline__ uint32_t vertex_ok(const Dir &d, uint32_t u, uint32_t site) {
#if defined(GG_CHECK)
  if (u >= d.nv) {
    check_fail(d.err, site, u);
    return 0u;
  }
#else
  (void)d;
  (void)site;
#endif
  return u;
}

// Adjacency entries that a warp reads once (coalesced) are not kept in L1,
// which then holds the gathered vertex state.
__device__ __forceinline__ uint32_t ld_once(const uint32_t *p) {
  uint32_t v;
  asm("ld.global.nc.L1::no_allocate.u32 %0, [%1];" : "=r"(v) : "l"(p));
  return v;
}
__device__ __forceinline__ uint4 ld_once_v4(const uint32_t *p) {
  uint4 v;
  asm("ld.global.nc.L1::no_allocate.v4.u32 {%0, %1, %2, %3}, [%4];"
      : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
      : "l"(p));
  return v;
}
__device__ __forceinline__ float ld_once(const float *p) {
  float v;
  asm("ld.global.nc.L1::no_allocate.f32 %0, [%1];" : "=f"(v) : "l"(p));
  return v;
}
__device__ __forceinline__ double ld_once(const double *p) {
  double v;
  asm("ld.global.nc.L1::no_allocate.f64 %0, [%1];" : "=d"(v) : "l"(p));
  return v;
}

// A gathered value of vertex state: the first `hot` entries (on the
// hot-source layout, the most gathered sources) are cached in L1; the rest
// are read past L1, so that they do not evict the hot entries.  The state
// was written by an earlier kernel, so the read-only path is safe.
template <typename T>
__device__ __forceinline__ T ld_gather(const T *a, uint32_t u, uint32_t hot) {
  return u < hot ? a[u] : ld_once(a + u);
}
// nbr_at for entries a warp reads once (past L1).
__device__ __forceinline__ uint32_t nbr_once(const Dir &d, unsigned long long k, uint32_t site) {
#if defined(GG_CHECK)
  if (k >= d.ne) {
    check_fail(d.err, site, k);
    return 0u;
  }
  return vertex_ok(d, ld_once(d.nbr + k), site);
#else
  (void)site;
  return ld_once(d.nbr + k);
#endif
}
__device__ __forceinline__ unsigned lanemask_lt() { return (1u << lane_id()) - 1u; }

template <typename T>
__device__ __forceinline__ T warp_sum(T x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(GG_FULL, x, o);
  return x;
}
template <typename T>
__device__ __forceinline__ T warp_min(T x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    T y = __shfl_xor_sync(GG_FULL, x, o);
    x = y < x ? y : x;
  }
  return x;
}

// Warp-aggregated append: every lane of the warp must call it.
__device__ __forceinline__ void queue_push(bool pred, uint32_t v, uint32_t *q, unsigned *qlen) {
  unsigned m = __ballot_sync(GG_FULL, pred);
  if (!m) return;
  unsigned lane = lane_id();
  unsigned leader = __ffs(m) - 1;
  unsigned base = 0;
  if (lane == leader) base = atomicAdd(qlen, (unsigned)__popc(m));
  base = __shfl_sync(GG_FULL, base, leader);
  if (pred) q[base + __popc(m & lanemask_lt())] = v;
}

// Per-thread activation totals, flushed once per block.
struct Tally {
  unsigned long long edges = 0, in_edges = 0;
  unsigned int activated = 0;
  unsigned int maxdeg = 0;
  double delta = 0.0;
  // all threads of the block must call flush
  __device__ __forceinline__ void flush(Counters *ctr) {
    __shared__ unsigned long long s_e[32], s_i[32];
    __shared__ unsigned int s_a[32], s_m[32];
    __shared__ double s_d[32];
    unsigned long long e = warp_sum(edges), ie = warp_sum(in_edges);
    unsigned int a = warp_sum(activated);
    unsigned int m = __reduce_max_sync(GG_FULL, maxdeg);
    double dl = warp_sum(delta);
    unsigned w = threadIdx.x >> 5, lane = lane_id();
    if (lane == 0) {
      s_e[w] = e;
      s_i[w] = ie;
      s_a[w] = a;
      s_m[w] = m;
      s_d[w] = dl;
    }
    __syncthreads();
    if (w == 0) {
      unsigned nw = (blockDim.x + 31) >> 5;
      e = lane < nw ? s_e[lane] : 0ull;
      ie = lane < nw ? s_i[lane] : 0ull;
      a = lane < nw ? s_a[lane] : 0u;
      m = lane < nw ? s_m[lane] : 0u;
      dl = lane < nw ? s_d[lane] : 0.0;
      e = warp_sum(e);
      ie = warp_sum(ie);
      a = warp_sum(a);
      m = __reduce_max_sync(GG_FULL, m);
      dl = warp_sum(dl);
      if (lane == 0) {
        if (m) atomicMax(&ctr->maxdeg, m);
        if (e) atomicAdd(&ctr->edges, e);
        if (ie) atomicAdd(&ctr->in_edges, ie);
        if (a) atomicAdd(&ctr->activated, a);
        if (dl != 0.0) atomicAdd(&ctr->delta, dl);
      }
    }
  }
};

}  // namespace gg

#endif
