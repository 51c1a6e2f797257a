// The reference's generic engine API on the GPU: process_vertices and
// process_edges (core/graph.hpp:1406-1469, 1493-1869) over device bitmaps
// and device vertex arrays, with the user's signal/slot code as device
// lambdas (nvcc --extended-lambda) instantiated into this translation unit's
// kernels.  The graph itself is loaded, sorted and owned by
// libgemini_gb300.so (Graph<EdgeData> in gemini/graph.hpp); this header
// reaches its adjacency through gg_graph_device_view.
//
// GPU forms of the reference's callbacks.  The reference hands a slot or a
// dense signal the whole adjacency list of a vertex, which one CPU thread
// walks.  Here the engine walks the lists itself, spreading long lists over
// lanes, warps and chunks, and calls the user's code once per edge:
//
//   sparse mode (active_edges < edges / 20, core/graph.hpp:1509):
//     sparse_signal(v) -> Msg<M>             per active v; emit(x) or no_msg<M>()
//                                            (the reference's emit(v, x))
//     sparse_slot(src, msg, dst, edge) -> R   per out-edge of an emitting src
//   dense mode:
//     dense_want(dst) -> bool                 skip dst altogether (the early
//                                             return in the reference's signal)
//     dense_signal(dst, src, edge) -> Msg<M>  contribution of one in-edge
//     dense_combine(Msg<M>& acc, Msg<M> x)    folds x into acc; returns true
//       -> bool                               when no later in-edge can change
//                                             acc (the reference's `break`)
//     dense_slot(dst, msg) -> R               per dst whose fold holds a message
//
// dense_combine must be associative: a list longer than 32 entries is folded
// in CSC order by a tree over lanes and chunks, so "first active
// in-neighbour" (BFS), sums (PageRank, BC) and minima (CC, SSSP) all work.
// Every signal of a call runs before any of its slots, in both modes (the
// reference's order within a call: its slots consume the messages its
// signals produced), so signals read the state as it was when the call
// began.  R is the sum of the slots' returns (integer or floating point).
// One partition: dense_selective is accepted and ignored, as the reference
// does for partitions == 1 (core/graph.hpp:1662).
//
// List form, for callbacks written the reference's way (a slot or a dense
// signal that walks a VertexAdjList with a loop of its own):
//   process_edges<R, M>(sparse_signal(v), sparse_slot(src, msg, VertexAdjList),
//                       dense_signal(dst, VertexAdjList), dense_slot(dst, msg),
//                       active)
// with the reference's argument lists (core/graph.hpp:1493-1494).  Callbacks
// are __device__ lambdas capturing by value (device lambdas cannot capture
// by reference); signals call graph->emit(v, msg) on the DeviceGraph of
// Engine::device_graph(), and the device forms of cas / write_min /
// write_add below are at hand.  Each callback call gets a piece of at most
// LIST_PIECE consecutive entries of one list, so a long list is handed over
// in several calls -- as the reference itself does when a vertex's edges are
// split over sockets or partitions (core/graph.hpp:1614-1658, 1755-1789),
// where a dense signal may emit one partial message per part and the dense
// slot combines them.  Minima, first-hit CAS and write_add slots (the five
// toolkits) give the single-call results; sums differ in order only.
#ifndef GEMINI_GB300_ENGINE_CUH
#define GEMINI_GB300_ENGINE_CUH

#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <string>
#include <type_traits>
#include <vector>

#include "gemini/graph.hpp"

// Device forms of the reference's atomics (core/atomic.hpp:24-51), for the
// list form's callbacks: compare-and-swap on 4- or 8-byte values, and the
// min / add loops built on it.
template <class T>
__device__ inline bool cas(T *ptr, T old_val, T new_val) {
  static_assert(sizeof(T) == 4 || sizeof(T) == 8, "cas works on 4- or 8-byte values");
  if constexpr (sizeof(T) == 4) {
    unsigned o, n;
    memcpy(&o, &old_val, 4);
    memcpy(&n, &new_val, 4);
    return atomicCAS(reinterpret_cast<unsigned *>(ptr), o, n) == o;
  } else {
    unsigned long long o, n;
    memcpy(&o, &old_val, 8);
    memcpy(&n, &new_val, 8);
    return atomicCAS(reinterpret_cast<unsigned long long *>(ptr), o, n) == o;
  }
}
template <class T>
__device__ inline bool write_min(T *ptr, T val) {
  T cur = *reinterpret_cast<volatile T *>(ptr);
  while (cur > val) {
    if (cas(ptr, cur, val)) return true;
    cur = *reinterpret_cast<volatile T *>(ptr);
  }
  return false;
}
template <class T>
__device__ inline void write_add(T *ptr, T val) {
  T cur = *reinterpret_cast<volatile T *>(ptr);
  while (!cas(ptr, cur, (T)(cur + val))) cur = *reinterpret_cast<volatile T *>(ptr);
}

namespace gemini {

inline void cuda_check(cudaError_t e, const char *what) {
  if (e != cudaSuccess) throw Error(GG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

template <typename M>
struct Msg {
  M value;
  int emit;
};
template <typename M>
__host__ __device__ inline Msg<M> emit(const M &v) {
  Msg<M> m;
  m.value = v;
  m.emit = 1;
  return m;
}
template <typename M>
__host__ __device__ inline Msg<M> no_msg() {
  Msg<M> m;
  memset(&m, 0, sizeof(m));
  return m;
}

template <class SS, class SL>
struct SparseOps {
  SS signal;
  SL slot;
};
template <class DW, class DS, class DC, class DL>
struct DenseOps {
  DW want;
  DS signal;
  DC combine;
  DL slot;
};
template <class SS, class SL>
SparseOps<SS, SL> sparse(SS signal, SL slot) {
  return SparseOps<SS, SL>{signal, slot};
}
template <class DW, class DS, class DC, class DL>
DenseOps<DW, DS, DC, DL> dense(DW want, DS signal, DC combine, DL slot) {
  return DenseOps<DW, DS, DC, DL>{want, signal, combine, slot};
}

namespace detail {

constexpr unsigned FULL = 0xffffffffu;
constexpr int THREADS = 256;
constexpr uint32_t LIGHT = 32;        // in-lists up to this long: one lane
constexpr uint32_t HEAVY = 8192;      // longer in-lists: chunks of CHUNK edges
constexpr uint32_t CHUNK = 2048;
constexpr int SCAN_TILE = 2048;

template <typename E>
__device__ inline E edge_at(const float *, uint64_t);
template <>
__device__ inline Empty edge_at<Empty>(const float *, uint64_t) {
  return Empty{};
}
template <>
__device__ inline float edge_at<float>(const float *w, uint64_t k) {
  return w[k];
}

// Shuffles of any trivially copyable value, 32 bits at a time.
template <typename T>
__device__ inline T shfl_down_any(const T &x, int off) {
  constexpr int W = (sizeof(T) + 3) / 4;
  uint32_t w[W] = {};
  memcpy(w, &x, sizeof(T));
#pragma unroll
  for (int i = 0; i < W; i++) w[i] = __shfl_down_sync(FULL, w[i], off);
  T y;
  memcpy(&y, w, sizeof(T));
  return y;
}
template <typename T>
__device__ inline T shfl_any(const T &x, int src) {
  constexpr int W = (sizeof(T) + 3) / 4;
  uint32_t w[W] = {};
  memcpy(w, &x, sizeof(T));
#pragma unroll
  for (int i = 0; i < W; i++) w[i] = __shfl_sync(FULL, w[i], src);
  T y;
  memcpy(&y, w, sizeof(T));
  return y;
}

template <typename R>
__device__ inline R warp_sum(R x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += shfl_down_any(x, o);
  return x;
}
__device__ inline void atomic_add_r(unsigned *p, unsigned v) { atomicAdd(p, v); }
__device__ inline void atomic_add_r(int *p, int v) { atomicAdd(p, v); }
__device__ inline void atomic_add_r(unsigned long long *p, unsigned long long v) { atomicAdd(p, v); }
__device__ inline void atomic_add_r(unsigned long *p, unsigned long v) {
  atomicAdd(reinterpret_cast<unsigned long long *>(p), (unsigned long long)v);
}
__device__ inline void atomic_add_r(long long *p, long long v) {
  atomicAdd(reinterpret_cast<unsigned long long *>(p), (unsigned long long)v);
}
__device__ inline void atomic_add_r(long *p, long v) {
  atomicAdd(reinterpret_cast<unsigned long long *>(p), (unsigned long long)v);
}
__device__ inline void atomic_add_r(float *p, float v) { atomicAdd(p, v); }
__device__ inline void atomic_add_r(double *p, double v) { atomicAdd(p, v); }

// Sum of r over the block into *out (one atomic per block); all threads call.
template <typename R>
__device__ inline void block_reduce_add(R r, R *out) {
  __shared__ __align__(16) unsigned char smem[sizeof(R) * (THREADS / 32)];
  R *s = reinterpret_cast<R *>(smem);
  r = warp_sum(r);
  const unsigned lane = threadIdx.x & 31u, w = threadIdx.x >> 5;
  if (lane == 0) s[w] = r;
  __syncthreads();
  if (w == 0) {
    R t = lane < (blockDim.x >> 5) ? s[lane] : R(0);
    t = warp_sum(t);
    if (lane == 0 && t != R(0)) atomic_add_r(out, t);
  }
}

inline unsigned grid_for(size_t work, int sms, int per_sm = 8) {
  size_t b = (work + THREADS - 1) / THREADS;
  const size_t cap = (size_t)sms * per_sm;
  if (b > cap) b = cap;
  return (unsigned)(b < 1 ? 1 : b);
}

static __global__ void fill_bits(unsigned long long *data, size_t size, size_t words) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < words; i += (size_t)gridDim.x * blockDim.x) {
    const size_t lo = i * 64;
    data[i] = lo + 64 <= size ? ~0ull : (lo >= size ? 0ull : ((1ull << (size - lo)) - 1));
  }
}
static __global__ void set_one_bit(unsigned long long *data, uint32_t v) { atomicOr(data + (v >> 6), 1ull << (v & 63)); }
template <typename T>
__global__ void fill_array(T *a, size_t n, T value) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    a[i] = value;
}

// process_vertices: one thread per 64-bit word of the active bitmap.
template <typename R, class F>
__global__ void __launch_bounds__(THREADS)
    vertices_kernel(const unsigned long long *__restrict__ bm, size_t words, uint32_t V, F f, R *out) {
  R r = R(0);
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < words; i += (size_t)gridDim.x * blockDim.x) {
    unsigned long long w = bm[i];
    while (w) {
      const int b = __ffsll((long long)w) - 1;
      w &= w - 1;
      const size_t v = i * 64 + b;
      if (v < V) r += f((uint32_t)v);
    }
  }
  block_reduce_add(r, out);
}

// Sparse signal: every active vertex's message, appended to (qv, qm).
template <typename M, class SS>
__global__ void __launch_bounds__(THREADS)
    sparse_signal_kernel(const unsigned long long *__restrict__ bm, size_t words, uint32_t V, SS ss,
                         uint32_t *__restrict__ qv, M *__restrict__ qm, unsigned *__restrict__ qlen) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < words; i += (size_t)gridDim.x * blockDim.x) {
    unsigned long long w = bm[i];
    while (w) {
      const int b = __ffsll((long long)w) - 1;
      w &= w - 1;
      const size_t v = i * 64 + b;
      if (v >= V) continue;
      const Msg<M> m = ss((uint32_t)v);
      if (m.emit) {
        const unsigned am = __activemask();
        const int leader = __ffs(am) - 1;
        const unsigned lane = threadIdx.x & 31u;
        const unsigned rank = __popc(am & ((1u << lane) - 1u));
        unsigned base = 0;
        if ((int)lane == leader) base = atomicAdd(qlen, (unsigned)__popc(am));
        base = __shfl_sync(am, base, leader);
        qv[base + rank] = (uint32_t)v;
        qm[base + rank] = m.value;
      }
    }
  }
}

// Exclusive scan of deg[qv[i]] (i < n) into pre[0..n], three passes.
static __global__ void scan_tile_sums(const uint32_t *__restrict__ qv, const uint32_t *__restrict__ deg, size_t n,
                               unsigned long long *__restrict__ tiles) {
  const size_t t = blockIdx.x;
  unsigned long long s = 0;
  for (size_t i = t * SCAN_TILE + threadIdx.x; i < n && i < (t + 1) * SCAN_TILE; i += blockDim.x) s += deg[qv[i]];
  block_reduce_add(s, tiles + t);
}
static __global__ void scan_tiles_serial(unsigned long long *tiles, size_t ntiles) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    unsigned long long run = 0;
    for (size_t t = 0; t < ntiles; t++) {
      const unsigned long long x = tiles[t];
      tiles[t] = run;
      run += x;
    }
    tiles[ntiles] = run;
  }
}
static __global__ void __launch_bounds__(THREADS)
    scan_tile_apply(const uint32_t *__restrict__ qv, const uint32_t *__restrict__ deg, size_t n,
                    const unsigned long long *__restrict__ tiles, size_t ntiles, unsigned long long *__restrict__ pre) {
  __shared__ unsigned long long s_warp[THREADS / 32];
  __shared__ unsigned long long s_run;
  const size_t t = blockIdx.x;
  const unsigned lane = threadIdx.x & 31u, w = threadIdx.x >> 5;
  if (threadIdx.x == 0) s_run = tiles[t];
  __syncthreads();
  for (size_t base = t * SCAN_TILE; base < (t + 1) * SCAN_TILE && base < n; base += THREADS) {
    const size_t i = base + threadIdx.x;
    const unsigned long long x = i < n ? (unsigned long long)deg[qv[i]] : 0ull;
    unsigned long long incl = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long y = __shfl_up_sync(FULL, incl, o);
      if (lane >= (unsigned)o) incl += y;
    }
    if (lane == 31) s_warp[w] = incl;
    __syncthreads();
    unsigned long long before = s_run;
    for (unsigned k = 0; k < w; k++) before += s_warp[k];
    if (i < n) pre[i] = before + incl - x;
    __syncthreads();
    if (threadIdx.x == THREADS - 1) s_run = before + incl;
    __syncthreads();
  }
  if (t == ntiles - 1 && threadIdx.x == 0) pre[n] = tiles[ntiles];
}

// Sparse slot: the out-edges of the queued vertices, edge-balanced (edge e
// of the concatenation belongs to queue entry upper_bound(pre, e) - 1).
template <typename R, typename M, typename E, class SL>
__global__ void __launch_bounds__(THREADS)
    sparse_slot_kernel(const uint64_t *__restrict__ off, const uint32_t *__restrict__ nbr,
                       const float *__restrict__ w, const uint32_t *__restrict__ qv, const M *__restrict__ qm,
                       const unsigned long long *__restrict__ pre, size_t n, SL sl, R *out) {
  const unsigned long long total = pre[n];
  R r = R(0);
  for (unsigned long long e = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (unsigned long long)gridDim.x * blockDim.x) {
    size_t lo = 0, hi = n;  // first index with pre > e, in (0, n]
    while (lo < hi) {
      const size_t mid = (lo + hi) >> 1;
      if (pre[mid] <= e)
        lo = mid + 1;
      else
        hi = mid;
    }
    const size_t i = lo - 1;
    const uint32_t src = qv[i];
    const uint64_t k = off[src] + (e - pre[i]);
    r += sl(src, qm[i], nbr[k], edge_at<E>(w, k));
  }
  block_reduce_add(r, out);
}

// Dense signal, lists of 1..LIGHT entries: one lane each, folded in order
// into dmsg[v] (every vertex with a nonempty in-list gets an entry).
template <typename M, typename E, class DW, class DS, class DC>
__global__ void __launch_bounds__(THREADS)
    dense_light_kernel(const uint64_t *__restrict__ off, const uint32_t *__restrict__ nbr,
                       const float *__restrict__ w, uint32_t V, DW dw, DS ds, DC dc, Msg<M> *__restrict__ dmsg) {
  for (size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (size_t)gridDim.x * blockDim.x) {
    const uint64_t b = off[v], e = off[v + 1];
    if (e == b || e - b > LIGHT) continue;
    Msg<M> acc = no_msg<M>();
    if (dw((uint32_t)v))
      for (uint64_t k = b; k < e; k++)
        if (dc(acc, ds((uint32_t)v, nbr[k], edge_at<E>(w, k)))) break;
    dmsg[v] = acc;
  }
}

// In-order fold of [b, e) by one warp, 32 entries per step, stopping when
// the combine says so; the result is valid in lane 0.
template <typename M, typename E, class DS, class DC>
__device__ inline Msg<M> warp_fold(uint32_t v, uint64_t b, uint64_t e, const uint32_t *__restrict__ nbr,
                                   const float *__restrict__ w, DS &ds, DC &dc) {
  const unsigned lane = threadIdx.x & 31u;
  Msg<M> acc = no_msg<M>();
  for (uint64_t base = b; base < e; base += 32) {
    const uint64_t k = base + lane;
    Msg<M> x = k < e ? ds(v, nbr[k], edge_at<E>(w, k)) : no_msg<M>();
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const Msg<M> y = shfl_down_any(x, o);
      if ((lane & (2 * o - 1)) == 0 && lane + o < 32) dc(x, y);
    }
    int stop = 0;
    if (lane == 0) stop = dc(acc, x) ? 1 : 0;
    if (__shfl_sync(FULL, stop, 0)) break;
  }
  return acc;
}

// Dense signal, lists of LIGHT+1..HEAVY entries: one warp per vertex.
template <typename M, typename E, class DW, class DS, class DC>
__global__ void __launch_bounds__(THREADS)
    dense_medium_kernel(const uint64_t *__restrict__ off, const uint32_t *__restrict__ nbr,
                        const float *__restrict__ w, const uint32_t *__restrict__ list, uint32_t n, DW dw, DS ds,
                        DC dc, Msg<M> *__restrict__ dmsg) {
  const size_t nwarps = (size_t)gridDim.x * (blockDim.x >> 5);
  for (size_t i = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += nwarps) {
    const uint32_t v = list[i];
    Msg<M> acc = no_msg<M>();
    if (dw(v)) acc = warp_fold<M, E>(v, off[v], off[v + 1], nbr, w, ds, dc);
    if ((threadIdx.x & 31u) == 0) dmsg[v] = acc;
  }
}

// Dense, lists longer than HEAVY: one warp per CHUNK-entry chunk
// (partials[c]), then one lane per vertex folding its chunks in order.
template <typename M, typename E, class DW, class DS, class DC>
__global__ void __launch_bounds__(THREADS)
    dense_chunk_kernel(const uint64_t *__restrict__ off, const uint32_t *__restrict__ nbr,
                       const float *__restrict__ w, const uint32_t *__restrict__ heavy,
                       const uint32_t *__restrict__ chunk_owner, const uint32_t *__restrict__ chunk_first,
                       uint32_t nchunks, DW dw, DS ds, DC dc, Msg<M> *__restrict__ partials) {
  const size_t nwarps = (size_t)gridDim.x * (blockDim.x >> 5);
  for (size_t c = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < nchunks; c += nwarps) {
    const uint32_t h = chunk_owner[c];
    const uint32_t v = heavy[h];
    Msg<M> acc = no_msg<M>();
    if (dw(v)) {
      const uint64_t b = off[v] + (uint64_t)(c - chunk_first[h]) * CHUNK;
      const uint64_t e = b + CHUNK < off[v + 1] ? b + CHUNK : off[v + 1];
      acc = warp_fold<M, E>(v, b, e, nbr, w, ds, dc);
    }
    if ((threadIdx.x & 31u) == 0) partials[c] = acc;
  }
}
template <typename M, class DW, class DC>
__global__ void __launch_bounds__(THREADS)
    dense_chunk_finish(const uint32_t *__restrict__ heavy, const uint32_t *__restrict__ chunk_first, uint32_t nheavy,
                       const Msg<M> *__restrict__ partials, DW dw, DC dc, Msg<M> *__restrict__ dmsg) {
  for (size_t h = (size_t)blockIdx.x * blockDim.x + threadIdx.x; h < nheavy; h += (size_t)gridDim.x * blockDim.x) {
    const uint32_t v = heavy[h];
    Msg<M> acc = no_msg<M>();
    if (dw(v))
      for (uint32_t c = chunk_first[h]; c < chunk_first[h + 1]; c++)
        if (dc(acc, partials[c])) break;
    dmsg[v] = acc;
  }
}

// Dense slot: after every signal of the call, each vertex whose fold holds
// a message.
template <typename R, typename M, class DL>
__global__ void __launch_bounds__(THREADS)
    dense_slot_kernel(const uint64_t *__restrict__ off, uint32_t V, const Msg<M> *__restrict__ dmsg, DL dl, R *out) {
  R r = R(0);
  for (size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (size_t)gridDim.x * blockDim.x) {
    if (off[v + 1] == off[v]) continue;
    const Msg<M> m = dmsg[v];
    if (m.emit) r += dl((uint32_t)v, m.value);
  }
  block_reduce_add(r, out);
}

// ---- list form (process_edges with VertexAdjList callbacks)
constexpr uint64_t LIST_PIECE = 64;  // entries per callback call at most

template <typename E>
__global__ void interleave_adjacency(const uint32_t *__restrict__ nbr, const float *__restrict__ w, uint64_t n,
                                     AdjUnit<E> *__restrict__ out) {
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
    AdjUnit<E> a;
    a.neighbour = nbr[k];
    a.edge_data = w[k];
    out[k] = a;
  }
}

// Sparse signals: every active vertex (they emit through the DeviceGraph).
template <class SS>
__global__ void __launch_bounds__(THREADS)
    list_sparse_signal(const unsigned long long *__restrict__ bm, size_t words, uint32_t V, SS ss) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < words; i += (size_t)gridDim.x * blockDim.x) {
    unsigned long long w = bm[i];
    while (w) {
      const int b = __ffsll((long long)w) - 1;
      w &= w - 1;
      const size_t v = i * 64 + b;
      if (v < V) ss((uint32_t)v);
    }
  }
}

// Sparse slots: the out-edges of the emitted messages, cut into pieces of
// LIST_PIECE entries of the messages' concatenated lists (pre = prefix of
// their out-degrees); a piece calls the slot once per message it covers.
template <typename R, typename M, typename E, class SL>
__global__ void __launch_bounds__(THREADS)
    list_sparse_slot(AdjUnit<E> *adj, const uint64_t *__restrict__ off, const uint32_t *__restrict__ qv,
                     const M *__restrict__ qm, const unsigned long long *__restrict__ pre, size_t n, SL sl, R *out) {
  const unsigned long long total = pre[n];
  const unsigned long long pieces = (total + LIST_PIECE - 1) / LIST_PIECE;
  R r = R(0);
  for (unsigned long long p = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; p < pieces;
       p += (unsigned long long)gridDim.x * blockDim.x) {
    const unsigned long long e0 = p * LIST_PIECE, e1 = e0 + LIST_PIECE < total ? e0 + LIST_PIECE : total;
    size_t lo = 0, hi = n;  // first message index with pre > e0, in (0, n]
    while (lo < hi) {
      const size_t mid = (lo + hi) >> 1;
      if (pre[mid] <= e0)
        lo = mid + 1;
      else
        hi = mid;
    }
    for (size_t i = lo - 1; i < n && pre[i] < e1; i++) {
      const unsigned long long a = pre[i] > e0 ? pre[i] : e0, b = pre[i + 1] < e1 ? pre[i + 1] : e1;
      if (a >= b) continue;
      const uint32_t src = qv[i];
      AdjUnit<E> *base = adj + (off[src] - pre[i]);
      r += sl(src, qm[i], VertexAdjList<E>(base + a, base + b));
    }
  }
  block_reduce_add(r, out);
}

// Dense signals: the in-lists cut into pieces of LIST_PIECE consecutive
// entries of the CSC; a piece calls the signal once per vertex it covers.
template <typename E, class DS>
__global__ void __launch_bounds__(THREADS)
    list_dense_signal(AdjUnit<E> *adj, const uint64_t *__restrict__ off, uint32_t V, uint64_t entries, DS ds) {
  const unsigned long long pieces = (entries + LIST_PIECE - 1) / LIST_PIECE;
  for (unsigned long long p = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; p < pieces;
       p += (unsigned long long)gridDim.x * blockDim.x) {
    const uint64_t e0 = p * LIST_PIECE, e1 = e0 + LIST_PIECE < entries ? e0 + LIST_PIECE : entries;
    uint32_t lo = 0, hi = V;  // first vertex with off > e0, in (0, V]
    while (lo < hi) {
      const uint32_t mid = lo + ((hi - lo) >> 1);
      if (off[mid] <= e0)
        lo = mid + 1;
      else
        hi = mid;
    }
    for (uint32_t v = lo - 1; v < V && off[v] < e1; v++) {
      const uint64_t a = off[v] > e0 ? off[v] : e0, b = off[v + 1] < e1 ? off[v + 1] : e1;
      if (a < b) ds(v, VertexAdjList<E>(adj + a, adj + b));
    }
  }
}

// Dense slots: every message the signals emitted.
template <typename R, typename M, class DL>
__global__ void __launch_bounds__(THREADS)
    list_dense_slot(const uint32_t *__restrict__ mv, const M *__restrict__ mm, unsigned n, DL dl, R *out) {
  R r = R(0);
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    r += dl(mv[i], mm[i]);
  block_reduce_add(r, out);
}

struct OutDegree {
  const uint32_t *deg;
  __device__ unsigned long long operator()(uint32_t v) const { return deg[v]; }
};
struct One {
  __device__ unsigned long long operator()(uint32_t) const { return 1ull; }
};

}  // namespace detail

// A vertex subset in device memory, in the reference's bitmap layout
// (core/bitmap.hpp: bit v % 64 of 64-bit word v / 64, size / 64 + 1 words).
class DeviceSubset {
 public:
  size_t size;
  size_t words;
  unsigned long long *data = nullptr;
  DeviceSubset(size_t n, cudaStream_t s, int sms) : size(n), words(n / 64 + 1), s_(s), sms_(sms) {
    cuda_check(cudaMalloc(&data, words * sizeof(unsigned long long)), "subset");
    clear();
  }
  ~DeviceSubset() {
    if (data) cudaFree(data);
  }
  DeviceSubset(const DeviceSubset &) = delete;
  DeviceSubset &operator=(const DeviceSubset &) = delete;
  void clear() { cuda_check(cudaMemsetAsync(data, 0, words * sizeof(unsigned long long), s_), "subset clear"); }
  void fill() {
    detail::fill_bits<<<detail::grid_for(words, sms_), detail::THREADS, 0, s_>>>(data, size, words);
    cuda_check(cudaGetLastError(), "subset fill");
  }
  // On the host: sets one bit with a kernel on the engine's stream.  In
  // device code (callbacks of the list form): an atomic OR, as the
  // reference's set_bit (core/bitmap.hpp:54-56).
  __host__ __device__ void set_bit(uint32_t v) {
#if defined(__CUDA_ARCH__)
    atomicOr(data + (v >> 6), 1ull << (v & 63));
#else
    if (v >= size) throw Error(GG_ERR_INVALID, "set_bit: vertex out of range");
    detail::set_one_bit<<<1, 1, 0, s_>>>(data, v);
    cuda_check(cudaGetLastError(), "subset set_bit");
#endif
  }
  __device__ bool get_bit(uint32_t v) const { return (data[v >> 6] >> (v & 63)) & 1ull; }
  // Subsets live in managed memory, so that a callback may dereference the
  // pointer the reference's code holds (active_out->set_bit(dst)); delete
  // frees them as the reference's toolkits do.
  static void *operator new(size_t n) {
    void *p = nullptr;
    cuda_check(cudaMallocManaged(&p, n), "subset");
    return p;
  }
  static void operator delete(void *p) { cudaFree(p); }

 private:
  cudaStream_t s_;
  int sms_;
};

// Device handle of a DeviceSubset for lambdas (captured by value).
struct SubsetRef {
  unsigned long long *data;
  __device__ bool get_bit(uint32_t v) const { return (data[v >> 6] >> (v & 63)) & 1ull; }
  __device__ bool set_bit(uint32_t v) const {  // true when this call set it
    const unsigned long long bit = 1ull << (v & 63);
    return !(atomicOr(data + (v >> 6), bit) & bit);
  }
};
inline SubsetRef ref(DeviceSubset *s) { return SubsetRef{s->data}; }

// The graph as the list form's callbacks see it (Engine::device_graph(), in
// managed memory): the reference's public fields and emit (core/graph.hpp:
// 94-111, 1480-1490), which appends (vertex, message) to the current call's
// message buffer.
template <typename EdgeData>
struct DeviceGraph {
  VertexId vertices;
  EdgeId edges;
  int partition_id;
  int partitions;
  uint32_t *msg_v;
  void *msg_m;
  unsigned *msg_len;
  unsigned msg_cap;
  template <typename M>
  __device__ void emit(VertexId v, M msg) const {
    const unsigned i = atomicAdd(msg_len, 1u);
    if (i < msg_cap) {
      msg_v[i] = v;
      static_cast<M *>(msg_m)[i] = msg;
    }
  }
};

template <typename EdgeData = Empty>
class Engine {
 public:
  uint32_t vertices = 0;
  uint64_t edges = 0;
  const uint32_t *out_degree = nullptr;  // device
  const uint32_t *in_degree = nullptr;   // device
  int last_mode = -1;                    // 0 sparse, 1 dense: the last process_edges call

  explicit Engine(Graph<EdgeData> &graph) : graph_(graph) {
    refresh();
    cuda_check(cudaStreamCreateWithFlags(&s_, cudaStreamNonBlocking), "engine stream");
    cuda_check(cudaMalloc(&red_, 16), "engine reduction");
    cuda_check(cudaMalloc(&qlen_, sizeof(unsigned)), "engine queue length");
    cuda_check(cudaMalloc(&qv_, sizeof(uint32_t) * ((size_t)vertices + 1)), "engine queue");
    cuda_check(cudaMalloc(&pre_, sizeof(unsigned long long) * ((size_t)vertices + 1)), "engine prefix");
    ntiles_max_ = ((size_t)vertices + detail::SCAN_TILE - 1) / detail::SCAN_TILE + 1;
    cuda_check(cudaMalloc(&tiles_, sizeof(unsigned long long) * (ntiles_max_ + 1)), "engine scan");
    build_bins();
  }
  ~Engine() {
    if (s_) cudaStreamSynchronize(s_);
    void *ps[] = {red_, qlen_, qv_, qm_, pre_, tiles_, med_, heavy_, chunk_owner_, chunk_first_, partials_, dmsg_,
                  lmv_, lmm_, dgraph_};
    for (void *p : ps)
      if (p) cudaFree(p);
    free_list_adjacency();
    if (s_) cudaStreamDestroy(s_);
  }
  Engine(const Engine &) = delete;
  Engine &operator=(const Engine &) = delete;

  cudaStream_t stream() const { return s_; }
  void sync() { cuda_check(cudaStreamSynchronize(s_), "engine sync"); }

  // core/graph.hpp:327
  DeviceSubset *alloc_vertex_subset() { return new DeviceSubset(vertices, s_, sms_); }
  // core/graph.hpp:229-251, in device memory
  template <typename T>
  T *alloc_vertex_array() {
    T *p = nullptr;
    cuda_check(cudaMalloc(&p, sizeof(T) * vertices), "alloc_vertex_array");
    return p;
  }
  template <typename T>
  void dealloc_vertex_array(T *p) {
    sync();
    cudaFree(p);
  }
  template <typename T>
  void fill_vertex_array(T *p, T value) {
    detail::fill_array<T><<<detail::grid_for(vertices, sms_), detail::THREADS, 0, s_>>>(p, vertices, value);
    cuda_check(cudaGetLastError(), "fill_vertex_array");
  }
  template <typename T>
  void copy_to_host(T *host, const T *dev) {
    cuda_check(cudaMemcpyAsync(host, dev, sizeof(T) * vertices, cudaMemcpyDeviceToHost, s_), "copy_to_host");
    sync();
  }

  // core/graph.hpp:760: the library swaps the directions; the views and the
  // dense bins follow.
  void transpose() {
    sync();
    graph_.transpose();
    refresh();
    build_bins();
    free_list_adjacency();
  }

  // The graph handle for the list form's callbacks (allocated once, in
  // managed memory).
  DeviceGraph<EdgeData> *device_graph() {
    if (!dgraph_) {
      cuda_check(cudaMallocManaged(&dgraph_, sizeof(DeviceGraph<EdgeData>)), "device graph");
      memset(dgraph_, 0, sizeof(DeviceGraph<EdgeData>));
    }
    auto *dg = static_cast<DeviceGraph<EdgeData> *>(dgraph_);
    dg->vertices = vertices;
    dg->edges = edges;
    dg->partition_id = 0;
    dg->partitions = 1;
    return dg;
  }

  // core/graph.hpp:1493-1869, list form (see the top of this file): the
  // callbacks take whole (pieces of) adjacency lists, as in the reference.
  template <typename R, typename M, class SS, class SL, class DS, class DL>
  R process_edges(SS sparse_signal, SL sparse_slot, DS dense_signal, DL dense_slot, DeviceSubset *active,
                  DeviceSubset *dense_selective = nullptr) {
    (void)dense_selective;
    static_assert(std::is_arithmetic<R>::value, "process_edges reduces an arithmetic type");
    static_assert(std::is_trivially_copyable<M>::value, "messages are stored in device buffers");
    DeviceGraph<EdgeData> *dg = device_graph();
    const unsigned long long active_edges = process_vertices<unsigned long long>(detail::OutDegree{out_degree}, active);
    R *out = reinterpret_cast<R *>(red_);
    cuda_check(cudaMemsetAsync(red_, 0, 16, s_), "process_edges");
    cuda_check(cudaMemsetAsync(qlen_, 0, sizeof(unsigned), s_), "process_edges");
    if (active_edges < edges / 20) {
      last_mode = 0;
      ensure_messages(sizeof(M));
      AdjUnit<EdgeData> *adj = list_adjacency(false);
      sync();
      dg->msg_v = qv_;
      dg->msg_m = qm_;
      dg->msg_len = qlen_;
      dg->msg_cap = vertices + 1;
      detail::list_sparse_signal<SS><<<detail::grid_for(active->words, sms_), detail::THREADS, 0, s_>>>(
          active->data, active->words, vertices, sparse_signal);
      cuda_check(cudaGetLastError(), "sparse signal");
      const unsigned n = messages_emitted(vertices + 1);
      if (n) {
        const size_t ntiles = ((size_t)n + detail::SCAN_TILE - 1) / detail::SCAN_TILE;
        cuda_check(cudaMemsetAsync(tiles_, 0, sizeof(unsigned long long) * (ntiles + 1), s_), "scan");
        detail::scan_tile_sums<<<(unsigned)ntiles, detail::THREADS, 0, s_>>>(qv_, out_degree, n, tiles_);
        detail::scan_tiles_serial<<<1, 32, 0, s_>>>(tiles_, ntiles);
        detail::scan_tile_apply<<<(unsigned)ntiles, detail::THREADS, 0, s_>>>(qv_, out_degree, n, tiles_, ntiles,
                                                                             pre_);
        unsigned long long total = 0;
        cuda_check(cudaMemcpyAsync(&total, pre_ + n, sizeof(total), cudaMemcpyDeviceToHost, s_), "scan");
        sync();
        const unsigned long long pieces = (total + detail::LIST_PIECE - 1) / detail::LIST_PIECE;
        if (pieces)
          detail::list_sparse_slot<R, M, EdgeData, SL><<<detail::grid_for(pieces, sms_, 16), detail::THREADS, 0, s_>>>(
              adj, out_.offsets, qv_, reinterpret_cast<const M *>(qm_), pre_, n, sparse_slot, out);
        cuda_check(cudaGetLastError(), "sparse slot");
      }
    } else {
      last_mode = 1;
      const unsigned long long pieces = (in_.entries + detail::LIST_PIECE - 1) / detail::LIST_PIECE;
      const size_t cap = (size_t)vertices + pieces + 1;
      ensure_list_messages(cap, sizeof(M));
      AdjUnit<EdgeData> *adj = list_adjacency(true);
      sync();
      dg->msg_v = lmv_;
      dg->msg_m = lmm_;
      dg->msg_len = qlen_;
      dg->msg_cap = (unsigned)cap;
      if (pieces)
        detail::list_dense_signal<EdgeData, DS><<<detail::grid_for(pieces, sms_, 16), detail::THREADS, 0, s_>>>(
            adj, in_.offsets, vertices, in_.entries, dense_signal);
      cuda_check(cudaGetLastError(), "dense signal");
      const unsigned n = messages_emitted((unsigned)cap);
      if (n)
        detail::list_dense_slot<R, M, DL><<<detail::grid_for(n, sms_), detail::THREADS, 0, s_>>>(
            lmv_, reinterpret_cast<const M *>(lmm_), n, dense_slot, out);
      cuda_check(cudaGetLastError(), "dense slot");
    }
    R r;
    cuda_check(cudaMemcpyAsync(&r, out, sizeof(R), cudaMemcpyDeviceToHost, s_), "process_edges");
    sync();
    return r;
  }

  // core/graph.hpp:1406-1469
  template <typename R, class F>
  R process_vertices(F f, DeviceSubset *active) {
    static_assert(std::is_arithmetic<R>::value, "process_vertices reduces an arithmetic type");
    R *out = reinterpret_cast<R *>(red_);
    cuda_check(cudaMemsetAsync(red_, 0, 16, s_), "process_vertices");
    detail::vertices_kernel<R, F><<<detail::grid_for(active->words, sms_), detail::THREADS, 0, s_>>>(
        active->data, active->words, vertices, f, out);
    cuda_check(cudaGetLastError(), "process_vertices");
    R r;
    cuda_check(cudaMemcpyAsync(&r, out, sizeof(R), cudaMemcpyDeviceToHost, s_), "process_vertices");
    sync();
    return r;
  }

  // core/graph.hpp:1493-1869
  template <typename R, typename M, class SS, class SL, class DW, class DS, class DC, class DL>
  R process_edges(SparseOps<SS, SL> sp, DenseOps<DW, DS, DC, DL> dn, DeviceSubset *active,
                  DeviceSubset *dense_selective = nullptr) {
    (void)dense_selective;
    static_assert(std::is_arithmetic<R>::value, "process_edges reduces an arithmetic type");
    static_assert(std::is_trivially_copyable<M>::value, "messages are copied between lanes");
    const unsigned long long active_edges = process_vertices<unsigned long long>(detail::OutDegree{out_degree}, active);
    R *out = reinterpret_cast<R *>(red_);
    cuda_check(cudaMemsetAsync(red_, 0, 16, s_), "process_edges");
    if (active_edges < edges / 20) {
      last_mode = 0;
      ensure_messages(sizeof(M));
      M *qm = reinterpret_cast<M *>(qm_);
      cuda_check(cudaMemsetAsync(qlen_, 0, sizeof(unsigned), s_), "sparse signal");
      detail::sparse_signal_kernel<M, SS><<<detail::grid_for(active->words, sms_), detail::THREADS, 0, s_>>>(
          active->data, active->words, vertices, sp.signal, qv_, qm, qlen_);
      cuda_check(cudaGetLastError(), "sparse signal");
      unsigned n = 0;
      cuda_check(cudaMemcpyAsync(&n, qlen_, sizeof(n), cudaMemcpyDeviceToHost, s_), "sparse signal");
      sync();
      if (n) {
        const size_t ntiles = ((size_t)n + detail::SCAN_TILE - 1) / detail::SCAN_TILE;
        cuda_check(cudaMemsetAsync(tiles_, 0, sizeof(unsigned long long) * (ntiles + 1), s_), "scan");
        detail::scan_tile_sums<<<(unsigned)ntiles, detail::THREADS, 0, s_>>>(qv_, out_degree, n, tiles_);
        detail::scan_tiles_serial<<<1, 32, 0, s_>>>(tiles_, ntiles);
        detail::scan_tile_apply<<<(unsigned)ntiles, detail::THREADS, 0, s_>>>(qv_, out_degree, n, tiles_, ntiles,
                                                                             pre_);
        unsigned long long total = 0;
        cuda_check(cudaMemcpyAsync(&total, pre_ + n, sizeof(total), cudaMemcpyDeviceToHost, s_), "scan");
        sync();
        if (total)
          detail::sparse_slot_kernel<R, M, EdgeData, SL><<<detail::grid_for(total, sms_, 16), detail::THREADS, 0, s_>>>(
              out_.offsets, out_.neighbours, out_.weights, qv_, qm, pre_, n, sp.slot, out);
        cuda_check(cudaGetLastError(), "sparse slot");
      }
    } else {
      last_mode = 1;
      ensure_dense_messages(sizeof(Msg<M>));
      Msg<M> *dmsg = reinterpret_cast<Msg<M> *>(dmsg_);
      detail::dense_light_kernel<M, EdgeData><<<detail::grid_for(vertices, sms_), detail::THREADS, 0, s_>>>(
          in_.offsets, in_.neighbours, in_.weights, vertices, dn.want, dn.signal, dn.combine, dmsg);
      if (nmed_)
        detail::dense_medium_kernel<M, EdgeData><<<detail::grid_for((size_t)nmed_ * 32, sms_), detail::THREADS, 0,
                                                   s_>>>(in_.offsets, in_.neighbours, in_.weights, med_, nmed_,
                                                         dn.want, dn.signal, dn.combine, dmsg);
      if (nheavy_) {
        ensure_partials(sizeof(Msg<M>) * nchunks_);
        Msg<M> *part = reinterpret_cast<Msg<M> *>(partials_);
        detail::dense_chunk_kernel<M, EdgeData><<<detail::grid_for((size_t)nchunks_ * 32, sms_), detail::THREADS, 0,
                                                  s_>>>(in_.offsets, in_.neighbours, in_.weights, heavy_,
                                                        chunk_owner_, chunk_first_, nchunks_, dn.want, dn.signal,
                                                        dn.combine, part);
        detail::dense_chunk_finish<M><<<detail::grid_for(nheavy_, sms_), detail::THREADS, 0, s_>>>(
            heavy_, chunk_first_, nheavy_, part, dn.want, dn.combine, dmsg);
      }
      detail::dense_slot_kernel<R, M><<<detail::grid_for(vertices, sms_), detail::THREADS, 0, s_>>>(
          in_.offsets, vertices, dmsg, dn.slot, out);
      cuda_check(cudaGetLastError(), "dense");
    }
    R r;
    cuda_check(cudaMemcpyAsync(&r, out, sizeof(R), cudaMemcpyDeviceToHost, s_), "process_edges");
    sync();
    return r;
  }

  // Vertices whose bit is set (process_vertices of 1).
  uint64_t count(DeviceSubset *s) { return process_vertices<unsigned long long>(detail::One{}, s); }

 private:
  void refresh() {
    check(gg_graph_device_view(graph_.handle(), 0, &out_), "device view");
    check(gg_graph_device_view(graph_.handle(), 1, &in_), "device view");
    vertices = out_.vertices;
    edges = out_.edges;
    out_degree = out_.degree;
    in_degree = in_.degree;
    cuda_check(cudaSetDevice(out_.device), "device");
    int sms = 0;
    cuda_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, out_.device), "device");
    sms_ = sms;
  }
  // Medium and heavy in-lists and the heavy chunk table, on the host from
  // the in-degrees (once per direction).
  void build_bins() {
    std::vector<uint32_t> deg(vertices);
    cuda_check(cudaMemcpy(deg.data(), in_.degree, sizeof(uint32_t) * vertices, cudaMemcpyDeviceToHost), "bins");
    std::vector<uint32_t> med, heavy, owner, first(1, 0);
    for (uint32_t v = 0; v < vertices; v++) {
      if (deg[v] > detail::HEAVY) {
        const uint32_t nc = (deg[v] + detail::CHUNK - 1) / detail::CHUNK;
        for (uint32_t c = 0; c < nc; c++) owner.push_back((uint32_t)heavy.size());
        heavy.push_back(v);
        first.push_back(first.back() + nc);
      } else if (deg[v] > detail::LIGHT) {
        med.push_back(v);
      }
    }
    void *old[] = {med_, heavy_, chunk_owner_, chunk_first_};
    for (void *p : old)
      if (p) cudaFree(p);
    nmed_ = (uint32_t)med.size();
    nheavy_ = (uint32_t)heavy.size();
    nchunks_ = (uint32_t)owner.size();
    upload(&med_, med);
    upload(&heavy_, heavy);
    upload(&chunk_owner_, owner);
    upload(&chunk_first_, first);
  }
  static void upload(uint32_t **dst, const std::vector<uint32_t> &h) {
    cuda_check(cudaMalloc(dst, sizeof(uint32_t) * (h.size() ? h.size() : 1)), "bins");
    if (!h.empty()) cuda_check(cudaMemcpy(*dst, h.data(), sizeof(uint32_t) * h.size(), cudaMemcpyHostToDevice), "bins");
  }
  void ensure_messages(size_t msg_bytes) {
    const size_t need = msg_bytes * ((size_t)vertices + 1);
    if (need <= qm_bytes_) return;
    sync();
    if (qm_) cudaFree(qm_);
    cuda_check(cudaMalloc(&qm_, need), "message queue");
    qm_bytes_ = need;
  }
  void ensure_dense_messages(size_t msg_bytes) {
    const size_t need = msg_bytes * ((size_t)vertices + 1);
    if (need <= dmsg_bytes_) return;
    sync();
    if (dmsg_) cudaFree(dmsg_);
    cuda_check(cudaMalloc(&dmsg_, need), "dense messages");
    dmsg_bytes_ = need;
  }
  // Messages the signals emitted; more than the buffer holds is an error
  // (a signal emitted more than once per call).
  unsigned messages_emitted(unsigned cap) {
    unsigned n = 0;
    cuda_check(cudaMemcpyAsync(&n, qlen_, sizeof(n), cudaMemcpyDeviceToHost, s_), "emit count");
    sync();
    if (n > cap) throw Error(GG_ERR_LIMIT, "process_edges: signals emitted more messages than one per call");
    return n;
  }
  void ensure_list_messages(size_t cap, size_t msg_bytes) {
    if (cap * msg_bytes <= lmm_bytes_ && cap * sizeof(uint32_t) <= lmv_bytes_) return;
    sync();
    if (lmv_) cudaFree(lmv_);
    if (lmm_) cudaFree(lmm_);
    cuda_check(cudaMalloc(&lmv_, cap * sizeof(uint32_t)), "dense messages");
    cuda_check(cudaMalloc(&lmm_, cap * msg_bytes), "dense messages");
    lmv_bytes_ = cap * sizeof(uint32_t);
    lmm_bytes_ = cap * msg_bytes;
  }
  // The adjacency as AdjUnit entries: an unweighted entry is the neighbour id
  // itself (the library's array, read in place); weighted entries are an
  // interleaved copy made on first use.
  AdjUnit<EdgeData> *list_adjacency(bool incoming) {
    const gg_device_adj &d = incoming ? in_ : out_;
    if constexpr (std::is_same<EdgeData, Empty>::value) {
      static_assert(sizeof(AdjUnit<Empty>) == sizeof(uint32_t), "an unweighted entry is its neighbour id");
      return reinterpret_cast<AdjUnit<Empty> *>(const_cast<uint32_t *>(d.neighbours));
    } else {
      AdjUnit<EdgeData> *&a = incoming ? adj_in_ : adj_out_;
      AdjUnit<EdgeData> *other = incoming ? adj_out_ : adj_in_;
      if (!a && other && in_.neighbours == out_.neighbours) a = other;  // symmetric: one copy
      if (!a) {
        if (!d.weights) throw Error(GG_ERR_UNWEIGHTED, "the list form needs the graph's edge data");
        cuda_check(cudaMalloc(&a, sizeof(AdjUnit<EdgeData>) * (d.entries ? d.entries : 1)), "adjacency units");
        detail::interleave_adjacency<EdgeData><<<detail::grid_for(d.entries, sms_), detail::THREADS, 0, s_>>>(
            d.neighbours, d.weights, d.entries, a);
        cuda_check(cudaGetLastError(), "adjacency units");
      }
      return a;
    }
  }
  void free_list_adjacency() {
    if (adj_out_) cudaFree(adj_out_);
    if (adj_in_ && adj_in_ != adj_out_) cudaFree(adj_in_);
    adj_out_ = adj_in_ = nullptr;
  }
  void ensure_partials(size_t bytes) {
    if (bytes <= partial_bytes_) return;
    sync();
    if (partials_) cudaFree(partials_);
    cuda_check(cudaMalloc(&partials_, bytes ? bytes : 16), "chunk partials");
    partial_bytes_ = bytes;
  }

  Graph<EdgeData> &graph_;
  gg_device_adj out_{}, in_{};
  cudaStream_t s_ = nullptr;
  int sms_ = 1;
  void *red_ = nullptr;
  unsigned *qlen_ = nullptr;
  uint32_t *qv_ = nullptr;
  void *qm_ = nullptr;
  size_t qm_bytes_ = 0;
  unsigned long long *pre_ = nullptr, *tiles_ = nullptr;
  size_t ntiles_max_ = 0;
  uint32_t *med_ = nullptr, *heavy_ = nullptr, *chunk_owner_ = nullptr, *chunk_first_ = nullptr;
  uint32_t nmed_ = 0, nheavy_ = 0, nchunks_ = 0;
  void *partials_ = nullptr;
  size_t partial_bytes_ = 0;
  void *dmsg_ = nullptr;
  size_t dmsg_bytes_ = 0;
  // list form: dense messages, interleaved adjacency units, the device graph
  uint32_t *lmv_ = nullptr;
  void *lmm_ = nullptr;
  size_t lmv_bytes_ = 0, lmm_bytes_ = 0;
  AdjUnit<EdgeData> *adj_out_ = nullptr, *adj_in_ = nullptr;
  void *dgraph_ = nullptr;
};

}  // namespace gemini

#endif
