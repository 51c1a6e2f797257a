// Edge-processing engine: the GB300 form of Graph::process_edges
// (core/graph.hpp:1492-1867) and Graph::process_vertices (:1406-1469).
//
// Reference semantics kept exactly:
//  * switch: sparse iff active_edges < edges / 20 (:1509), active_edges =
//    sum of out_degree over the active set (:1503-1508);
//  * every signal of a call is computed before any slot of the call applies
//    (messages are buffered, :1541-1556 and :1755-1793).  Push kernels read
//    their message from a snapshot taken before the kernel (or from state no
//    slot of the call can write); pull kernels that read a state array the
//    same call writes use two buffers (read one, write the other).
// Fused on the device:
//  * signal + slot: the push kernel computes the slot for each edge of each
//    queued vertex; the pull kernel gathers the in-list (signal) and applies
//    the slot to its own vertex with a plain store (one writer per vertex);
//  * the activation epilogue of every edge kernel sets the active_out bit,
//    appends the vertex to the next queue and adds its out_degree to the
//    next call's active_edges, so the switch of the next call and the
//    process_vertices(active_out) count need no extra pass.
#ifndef GG_ENGINE_CUH
#define GG_ENGINE_CUH

#include <string.h>

#include <cooperative_groups.h>
#include <type_traits>

#include "gg_common.cuh"
#include "gg_scan.cuh"

namespace gg {

constexpr uint32_t NONE32 = 0xffffffffu;

// Ops whose gather adds an edge weight (SSSP) may take the weight from the
// kernel (gather_w): the chunk kernel reads weights coalesced and past L1,
// as it reads neighbour ids, so that L1 keeps the gathered state.
template <class Op, class = void>
struct has_gather_w : std::false_type {};
template <class Op>
struct has_gather_w<Op, std::void_t<decltype(&Op::gather_w)>> : std::true_type {};
constexpr int PUSH_THREADS = 256;
constexpr int PUSH_TILE = 1024;              // edges per block iteration of push_lb
constexpr int PUSH_STAGE = PUSH_TILE + 1;    // queue entries a tile spans when each has >= 1 edge
constexpr int PULL_THREADS = 256;

// Where an edge kernel records activations.  Only push (sparse) calls append
// to a queue; after a pull (dense) call the next queue, if the next call is
// sparse, is compacted from the bitmap in vertex order (queue_from_bitmap),
// which avoids one same-address atomic per warp of activated vertices.
struct ActOut {
  uint32_t *active_out = nullptr;  // bitmap; null: the call activates nothing
  uint32_t *visited = nullptr;     // also set here when non-null
  uint32_t *q_out = nullptr;       // next queue (push calls); null: none
  unsigned *qlen = nullptr;
  const uint32_t *out_deg = nullptr;
  const uint32_t *in_deg = nullptr;  // optional: also sum in_degree
  bool queue_nonzero_only = false;   // append only vertices with out_degree > 0
};

// Push activation: pred may be true for several lanes naming the same
// vertex; the bitmap decides who appends.  All lanes must call.
__device__ __forceinline__ void push_activate(bool pred, uint32_t v, const ActOut &a, Tally &t) {
  bool fresh = false;
  if (pred) {
    fresh = bm_set_atomic(a.active_out, v);
    if (fresh && a.visited) atomicOr(a.visited + (v >> 5), 1u << (v & 31));
  }
  uint32_t od = fresh ? a.out_deg[v] : 0u;
  if (a.q_out) queue_push(fresh && (!a.queue_nonzero_only || od > 0), v, a.q_out, a.qlen);
  if (fresh) {
    t.activated += 1;
    t.edges += od;
    t.maxdeg = od > t.maxdeg ? od : t.maxdeg;
    if (a.in_deg) t.in_edges += a.in_deg[v];
  }
}

// Pull activation: the warp owns bitmap word g (vertices 32g..32g+31), so the
// word is written with plain stores.  All lanes must call.
__device__ __forceinline__ void pull_activate(bool act, uint32_t v, size_t g, const ActOut &a, Tally &t) {
  unsigned bits = __ballot_sync(GG_FULL, act);
  if (lane_id() == 0 && bits) {
    a.active_out[g] = bits;
    if (a.visited) a.visited[g] |= bits;
  }
  if (act) {
    const uint32_t od = a.out_deg[v];
    t.activated += 1;
    t.edges += od;
    t.maxdeg = od > t.maxdeg ? od : t.maxdeg;
    if (a.in_deg) t.in_edges += a.in_deg[v];
  }
}

template <typename T>
__device__ __forceinline__ uint32_t upper_bound_idx(const T *P, uint32_t lo, uint32_t hi, T x) {
  // first index in [lo, hi) with P[i] > x (hi if none)
  while (lo < hi) {
    uint32_t mid = lo + ((hi - lo) >> 1);
    if (P[mid] <= x)
      lo = mid + 1;
    else
      hi = mid;
  }
  return lo;
}

// ---------------------------------------------------------------- push
// Sparse mode (core/graph.hpp:1510-1663): for every queued vertex q[i] and
// every out-edge, op.push(src, i, dst, w) applies the slot and returns
// whether it may activate dst.  Work is split by EDGES: P is the exclusive
// prefix of the queued vertices' degrees (P[n] = total); each block
// iteration takes PUSH_TILE consecutive edges, stages the tile's slice of P
// with the sources and their list offsets in shared memory, and each thread
// finds its edge's source by binary search there.  A hub's list is spread
// over as many blocks as it needs and neighbour loads are coalesced.  A tile
// spanning more than PUSH_STAGE entries (queues holding degree-0 vertices)
// searches P in global memory instead.
template <class Op>
__global__ void __launch_bounds__(PUSH_THREADS)
    push_lb(const uint32_t *__restrict__ q, const unsigned long long *__restrict__ P, uint32_t n,
            unsigned long long total, Dir d, Op op, ActOut act, Counters *ctr) {
  __shared__ unsigned long long s_P[PUSH_STAGE + 1];
  __shared__ unsigned long long s_base[PUSH_STAGE];
  __shared__ uint32_t s_src[PUSH_STAGE];
  __shared__ uint32_t s_lo, s_hi;
  Tally t;
  unsigned long long ntiles = (total + PUSH_TILE - 1) / PUSH_TILE;
  for (unsigned long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    unsigned long long e0 = tile * PUSH_TILE;
    unsigned long long e1 = e0 + PUSH_TILE < total ? e0 + PUSH_TILE : total;
    if (threadIdx.x == 0) {
      uint32_t lo = upper_bound_idx<unsigned long long>(P, 0, n + 1, e0) - 1;
      s_lo = lo;
      s_hi = upper_bound_idx<unsigned long long>(P, lo, n + 1, e1 - 1);  // one past the entry holding e1-1
    }
    __syncthreads();
    const uint32_t lo = s_lo, hi = s_hi, cnt = hi - lo;
    const bool staged = cnt <= (uint32_t)PUSH_STAGE;
    if (staged) {
      for (uint32_t i = threadIdx.x; i < cnt; i += PUSH_THREADS) {
        unsigned long long pi = P[lo + i];
        uint32_t src = q[lo + i];
        s_P[i] = pi;
        s_src[i] = src;
        s_base[i] = d.off[src] - pi;
      }
    }
    __syncthreads();
    for (unsigned long long base = e0; base < e1; base += PUSH_THREADS) {
      unsigned long long e = base + threadIdx.x;
      bool pred = false;
      uint32_t dst = 0;
      if (e < e1) {
        uint32_t qi, src;
        unsigned long long k;
        if (staged) {
          uint32_t i = upper_bound_idx<unsigned long long>(s_P, 0, cnt, e) - 1;
          src = s_src[i];
          k = s_base[i] + e;
          qi = lo + i;
        } else {
          qi = upper_bound_idx<unsigned long long>(P, lo, hi, e) - 1;
          src = q[qi];
          k = d.off[src] + (e - P[qi]);
        }
        dst = nbr_at(d, k, GG_SITE);
        float w = d.w ? d.w[k] : 0.0f;
        pred = op.push(src, qi, dst, w);
      }
      if (act.active_out) push_activate(pred, dst, act, t);
    }
    __syncthreads();
  }
  t.flush(ctr);
}

// ---------------------------------------------------------------- pull
// Dense mode (core/graph.hpp:1664-1855), reduction form.  For each vertex v
// with op.want(v): acc = op.identity(v) combined (op.combine) with
// op.gather(d, k, u) (u = the k-th entry) over its in-list, then
// op.finish(v, acc, deg, tally) applies the slot and returns whether v is
// activated.  Op::Acc is the message type; op.identity_coop() is the
// neutral element of combine.  Work is split by the direction's degree bins:
//   pull_light   one warp per 32 consecutive vertices, each lane serially
//                over a list of <= d.light entries (and every deg-0 vertex);
//                the warp owns the bitmap word of its 32 vertices
//   pull_chunks / pull_big_finish(_warps)
//                every longer list cut into d.chunk-edge chunks, one warp
//                per chunk, then a lane (or, without activations, a warp)
//                per vertex combining its chunks
// The chunk kernel runs beside pull_light (second stream); the finish runs
// after both and sets its bitmap bits atomically.
// WIN: each lane reads its list by aligned 32-byte windows (two 16-byte
// loads through L1: eight entries per two load instructions instead of
// eight), the window's entries of [b, e) gathered together and combined in
// list order, so the sums equal the scalar form's bit for bit.  The neighbour
// arrays are padded to a multiple of 64 entries, so a window never leaves
// the array.  Picked per graph by the autotuner (Dir.vec bit 1).
constexpr unsigned LIGHT_WIN = 8;
template <class Op, bool WIN>
__global__ void __launch_bounds__(PULL_THREADS) pull_light(Dir d, uint32_t V, Op op, ActOut act, Counters *ctr) {
  using Acc = typename Op::Acc;
  Tally t;
  size_t nwarps = (size_t)gridDim.x * (PULL_THREADS / 32);
  size_t groups = ((size_t)V + 31) / 32;
  unsigned lane = lane_id();
  for (size_t g = (size_t)blockIdx.x * (PULL_THREADS / 32) + (threadIdx.x >> 5); g < groups; g += nwarps) {
    uint32_t v = (uint32_t)(g * 32 + lane);
    bool todo = v < V && op.want(v);
    unsigned long long b = 0, e = 0;
    if (todo) {
      b = d.off[v];
      e = d.off[v + 1];
    }
    uint32_t deg = (uint32_t)(e - b);
    bool a = false;
    if (todo && deg <= d.light) {
      Acc acc = op.identity(v);
      if constexpr (WIN) {
        for (unsigned long long k = b & ~(unsigned long long)(LIGHT_WIN - 1); k < e; k += LIGHT_WIN) {
          const uint4 w0 = *reinterpret_cast<const uint4 *>(d.nbr + k);
          const uint4 w1 = *reinterpret_cast<const uint4 *>(d.nbr + k + 4);
          const uint32_t u[LIGHT_WIN] = {w0.x, w0.y, w0.z, w0.w, w1.x, w1.y, w1.z, w1.w};
          Acc gv[LIGHT_WIN];
#pragma unroll
          for (unsigned j = 0; j < LIGHT_WIN; j++)
            gv[j] = k + j >= b && k + j < e ? op.gather(d, k + j, vertex_ok(d, u[j], GG_SITE)) : op.identity_coop();
#pragma unroll
          for (unsigned j = 0; j < LIGHT_WIN; j++)
            if (k + j >= b && k + j < e) acc = op.combine(acc, gv[j]);
        }
      } else {
        // four independent gathers in flight, combined in list order
        unsigned long long k = b;
        for (; k + 4 <= e; k += 4) {
          const uint32_t u0 = nbr_at(d, k, GG_SITE), u1 = nbr_at(d, k + 1, GG_SITE), u2 = nbr_at(d, k + 2, GG_SITE), u3 = nbr_at(d, k + 3, GG_SITE);
          Acc g0 = op.gather(d, k, u0), g1 = op.gather(d, k + 1, u1), g2 = op.gather(d, k + 2, u2),
              g3 = op.gather(d, k + 3, u3);
          acc = op.combine(op.combine(op.combine(op.combine(acc, g0), g1), g2), g3);
        }
        for (; k < e; k++) acc = op.combine(acc, op.gather(d, k, nbr_at(d, k, GG_SITE)));
      }
      a = op.finish(v, acc, deg, t);
    }
    if (act.active_out) pull_activate(a, v, g, act, t);
  }
  t.flush(ctr);
}

// Lists longer than d.light: one warp per d.chunk-edge aligned block of the
// adjacency (d.chunk = 32 * PER_LANE, 128 / 256 / 512), PER_LANE gathers in
// flight per lane; partials[c] = the chunk's combine (lane order, then the
// warp tree).  Two load shapes (d.vec, picked per graph by the autotuner):
//   VEC    lane l loads the block's 16-byte windows l, l + 32, ... with one
//          vector load each (fewer load instructions), read past L1;
//   !VEC   lane l takes entries l, l + 32, ... (a warp's gathers touch
//          consecutive entries, which share cache sectors where an in-list
//          holds runs of consecutive source numbers), read past L1.
template <class Op, int PER_LANE, bool VEC>
__global__ void __launch_bounds__(PULL_THREADS)
    pull_chunks(Dir d, Op op, typename Op::Acc *__restrict__ partials) {
  using Acc = typename Op::Acc;
  constexpr int WIN = PER_LANE / 4;
  const size_t nwarps = (size_t)gridDim.x * (PULL_THREADS / 32);
  const unsigned lane = lane_id();
  for (size_t c = (size_t)blockIdx.x * (PULL_THREADS / 32) + (threadIdx.x >> 5); c < d.nbigchunks; c += nwarps) {
    uint32_t v;
    unsigned long long lo, b, e;
    big_range(d, (uint32_t)c, 32 * PER_LANE, &v, &lo, &b, &e);
    Acc part = op.identity_coop();
    if (op.want(v)) {
      Acc vals[PER_LANE];
      constexpr bool WT = has_gather_w<Op>::value;
      if constexpr (VEC) {
        uint4 w[WIN], wt[WT ? WIN : 1];
#pragma unroll
        for (int i = 0; i < WIN; i++) {
          const unsigned long long p = lo + 4 * (lane + 32 * i);
          const bool in = p < e && p + 4 > b;
          w[i] = in ? ld_once_v4(d.nbr + p) : make_uint4(0, 0, 0, 0);
          if constexpr (WT)
            wt[i] = in ? ld_once_v4(reinterpret_cast<const uint32_t *>(d.w) + p) : make_uint4(0, 0, 0, 0);
        }
#pragma unroll
        for (int i = 0; i < WIN; i++) {
          const unsigned long long p = lo + 4 * (lane + 32 * i);
          const uint32_t u[4] = {vertex_ok(d, w[i].x, GG_SITE), vertex_ok(d, w[i].y, GG_SITE),
                                 vertex_ok(d, w[i].z, GG_SITE), vertex_ok(d, w[i].w, GG_SITE)};
#pragma unroll
          for (int j = 0; j < 4; j++) {
            const bool in = p + j >= b && p + j < e;
            if constexpr (WT) {
              const uint32_t wb[4] = {wt[i].x, wt[i].y, wt[i].z, wt[i].w};
              vals[4 * i + j] = in ? op.gather_w(u[j], __uint_as_float(wb[j])) : op.identity_coop();
            } else {
              vals[4 * i + j] = in ? op.gather(d, p + j, u[j]) : op.identity_coop();
            }
          }
        }
      } else {
        uint32_t u[PER_LANE];
        float wt[WT ? PER_LANE : 1];
#pragma unroll
        for (int j = 0; j < PER_LANE; j++) {
          const unsigned long long k = b + lane + 32 * j;
          u[j] = k < e ? nbr_once(d, k, GG_SITE) : 0u;
          if constexpr (WT) wt[j] = k < e ? ld_once(d.w + k) : 0.0f;
        }
#pragma unroll
        for (int j = 0; j < PER_LANE; j++) {
          const unsigned long long k = b + lane + 32 * j;
          if constexpr (WT)
            vals[j] = k < e ? op.gather_w(u[j], wt[j]) : op.identity_coop();
          else
            vals[j] = k < e ? op.gather(d, k, u[j]) : op.identity_coop();
        }
      }
#pragma unroll
      for (int j = 0; j < PER_LANE; j++) part = op.combine(part, vals[j]);
    }
    part = op.warp_combine(part);
    if (lane == 0) partials[c] = part;
  }
}

// Long-list vertices of a call that activates nothing (PageRank, BC's
// backward sweep): one warp per vertex; the lanes read its chunk partials
// (coalesced, lane-strided), the warp tree combines them, lane 0 applies the
// slot.  Measured against the lane-per-vertex finish below: PageRank R-MAT 20
// 286 -> 326 GTEPS (there the lanes, adding up to 32 partials each in series,
// are latency-bound); calls with activations keep the lane form, which
// records a warp's 32 activations together (SSSP R-MAT 25: 145 against 138).
template <class Op>
__global__ void __launch_bounds__(PULL_THREADS)
    pull_big_finish_warps(Dir d, Op op, const typename Op::Acc *__restrict__ partials, Counters *ctr) {
  using Acc = typename Op::Acc;
  Tally t;
  const size_t nwarps = (size_t)gridDim.x * (PULL_THREADS / 32);
  const unsigned lane = lane_id();
  for (size_t i = (size_t)blockIdx.x * (PULL_THREADS / 32) + (threadIdx.x >> 5); i < d.nbig; i += nwarps) {
    const uint32_t v = d.big[i];
    if (!op.want(v)) continue;
    const uint32_t c0 = d.big_chunk[i], c1 = d.big_chunk[i + 1];
    Acc part = op.identity_coop();
    for (uint32_t c = c0 + lane; c < c1; c += 32) part = op.combine(part, partials[c]);
    part = op.warp_combine(part);
    if (lane == 0) op.finish(v, op.combine(op.identity(v), part), d.deg[v], t);
  }
  t.flush(ctr);
}

// One lane per long-list vertex combines its chunk partials in order (a warp
// does it for vertices with more than 32 chunks), then applies the slot.
template <class Op>
__global__ void __launch_bounds__(PULL_THREADS)
    pull_big_finish(Dir d, Op op, const typename Op::Acc *__restrict__ partials, ActOut act, Counters *ctr) {
  using Acc = typename Op::Acc;
  Tally t;
  const size_t stride = (size_t)gridDim.x * PULL_THREADS;
  const size_t n = ((size_t)d.nbig + 31) / 32 * 32;
  const unsigned lane = lane_id();
  for (size_t i = (size_t)blockIdx.x * PULL_THREADS + threadIdx.x; i < n; i += stride) {
    const bool valid = i < d.nbig;
    const uint32_t v = valid ? d.big[i] : 0u;
    const bool todo = valid && op.want(v);
    uint32_t c0 = 0, c1 = 0;
    if (todo) {
      c0 = d.big_chunk[i];
      c1 = d.big_chunk[i + 1];
    }
    Acc acc = op.identity(v);
    if (todo && c1 - c0 <= 32)
      for (uint32_t c = c0; c < c1; c++) acc = op.combine(acc, partials[c]);
    unsigned coop = __ballot_sync(GG_FULL, todo && c1 - c0 > 32);
    while (coop) {
      const unsigned leader = __ffs(coop) - 1;
      coop &= coop - 1;
      const uint32_t lc0 = __shfl_sync(GG_FULL, c0, leader), lc1 = __shfl_sync(GG_FULL, c1, leader);
      Acc part = op.identity_coop();
      for (uint32_t c = lc0 + lane; c < lc1; c += 32) part = op.combine(part, partials[c]);
      part = op.warp_combine(part);
      if (lane == leader) acc = op.combine(acc, part);
    }
    const bool a = todo && op.finish(v, acc, d.deg[v], t);
    if (act.active_out) push_activate(a, v, act, t);
  }
  t.flush(ctr);
}

// ---------------------------------------------------------------- BFS pull
// toolkits/bfs.cpp:60-76: an unvisited vertex takes the FIRST in-neighbour
// (in CSC order) that is in the active set as its parent.  Every bin keeps
// that order: lanes scan their own list in order; a warp takes the lowest
// lane of the first 32-wide chunk with a hit; heavy chunks record the index
// of their first hit and the finish takes the lowest.
static __global__ void __launch_bounds__(PULL_THREADS, 8)
    bfs_pull_light(Dir d, uint32_t V, const uint32_t *__restrict__ active_in, uint32_t *parent, ActOut act,
                   Counters *ctr) {
  Tally t;
  const size_t nwarps = (size_t)gridDim.x * (PULL_THREADS / 32);
  const size_t groups = ((size_t)V + 31) / 32;
  const unsigned lane = lane_id();
  // Software-pipelined over the warp's groups: the visited word, offsets and
  // out-degree of group g + nwarps are loaded before group g is scanned.
  size_t g = (size_t)blockIdx.x * (PULL_THREADS / 32) + (threadIdx.x >> 5);
  uint32_t vis = 0, od = 0;
  unsigned long long b = 0, e = 0;
  bool todo = false;
  if (g < groups) {
    uint32_t v = (uint32_t)(g * 32 + lane);
    vis = act.visited[g];
    todo = v < V && !((vis >> lane) & 1u);
    if (todo) {
      b = d.off[v];
      e = d.off[v + 1];
      od = act.out_deg[v];
    }
  }
  while (g < groups) {
    const size_t gn = g + nwarps;
    uint32_t visn = 0, odn = 0;
    unsigned long long bn = 0, en = 0;
    bool todon = false;
    if (gn < groups) {
      uint32_t vn = (uint32_t)(gn * 32 + lane);
      visn = act.visited[gn];
      todon = vn < V && !((visn >> lane) & 1u);
      if (todon) {
        bn = d.off[vn];
        en = d.off[vn + 1];
        odn = act.out_deg[vn];
      }
    }
    // the first LIGHT_DEG entries of every list, four independent loads at a
    // time; longer lists without a hit there go on in the medium / heavy kernels
    const uint32_t v = (uint32_t)(g * 32 + lane);
    uint32_t found = NONE32;
    if (todo) {
      unsigned long long lim = e - b <= d.light ? e : b + d.light;
      for (unsigned long long k = b; k < lim && found == NONE32; k += 4) {
        uint32_t s0 = nbr_at(d, k, GG_SITE);
        uint32_t s1 = k + 1 < lim ? nbr_at(d, k + 1, GG_SITE) : s0;
        uint32_t s2 = k + 2 < lim ? nbr_at(d, k + 2, GG_SITE) : s0;
        uint32_t s3 = k + 3 < lim ? nbr_at(d, k + 3, GG_SITE) : s0;
        bool h0 = bm_test_ldg(active_in, s0), h1 = bm_test_ldg(active_in, s1);
        bool h2 = bm_test_ldg(active_in, s2), h3 = bm_test_ldg(active_in, s3);
        found = h0 ? s0 : h1 ? s1 : h2 ? s2 : h3 ? s3 : NONE32;
      }
    }
    const bool a = found != NONE32;
    if (a) parent[v] = found;
    const unsigned bits = __ballot_sync(GG_FULL, a);
    if (lane == 0 && bits) {
      act.active_out[g] = bits;
      act.visited[g] = vis | bits;
    }
    if (a) {
      t.activated += 1;
      t.edges += od;
      t.maxdeg = od > t.maxdeg ? od : t.maxdeg;
    }
    g = gn;
    vis = visn;
    todo = todon;
    b = bn;
    e = en;
    od = odn;
  }
  t.flush(ctr);
}

static __global__ void __launch_bounds__(PULL_THREADS)
    bfs_pull_medium(Dir d, const uint32_t *__restrict__ active_in, uint32_t *parent, ActOut act, Counters *ctr) {
  Tally t;
  size_t nwarps = (size_t)gridDim.x * (PULL_THREADS / 32);
  unsigned lane = lane_id();
  for (size_t i = (size_t)blockIdx.x * (PULL_THREADS / 32) + (threadIdx.x >> 5); i < d.nmed; i += nwarps) {
    uint32_t v = d.med[i];
    uint32_t found = NONE32;
    if (!bm_test(act.visited, v)) {
      unsigned long long b = d.off[v] + d.light, e = d.off[v + 1];
      for (unsigned long long base = b; base < e; base += 32) {
        unsigned long long k = base + lane;
        uint32_t s = 0;
        bool hit = false;
        if (k < e) {
          s = nbr_at(d, k, GG_SITE);
          hit = bm_test_ldg(active_in, s);
        }
        unsigned m = __ballot_sync(GG_FULL, hit);
        if (m) {
          found = __shfl_sync(GG_FULL, s, __ffs(m) - 1);
          break;
        }
      }
    }
    bool a = lane == 0 && found != NONE32;
    if (a) parent[v] = found;
    push_activate(a, v, act, t);
  }
  t.flush(ctr);
}

// partials[c] = edge index of the chunk's first active in-neighbour, or ~0.
static __global__ void __launch_bounds__(PULL_THREADS)
    bfs_heavy_first(Dir d, const uint32_t *__restrict__ active_in, const uint32_t *__restrict__ visited,
                    unsigned long long *first) {
  // one warp per HEAVY_CHUNK-entry chunk of a list longer than HEAVY_DEG;
  // first[h] = the lowest hit index of heavy vertex h, so a chunk starting
  // past it (or a vertex already visited) is skipped and a scan stops at it
  const size_t nwarps = (size_t)gridDim.x * (PULL_THREADS / 32);
  const unsigned lane = lane_id();
  for (size_t c = (size_t)blockIdx.x * (PULL_THREADS / 32) + (threadIdx.x >> 5); c < d.nchunks; c += nwarps) {
    const uint32_t h = d.chunk_owner[c];
    const uint32_t v = d.heavy[h];
    if (bm_test(visited, v)) continue;
    const unsigned long long b = d.off[v] + (unsigned long long)(c - d.heavy_chunk[h]) * HEAVY_CHUNK;
    const unsigned long long end = d.off[v + 1];
    const unsigned long long e = b + HEAVY_CHUNK < end ? b + HEAVY_CHUNK : end;
    for (unsigned long long base = b; base < e; base += 32) {
      unsigned long long best = 0;
      if (lane == 0) best = *(volatile unsigned long long *)(first + h);
      if (__shfl_sync(GG_FULL, best, 0) < base) break;
      const unsigned long long k = base + lane;
      const bool hit = k < e && bm_test_ldg(active_in, nbr_at(d, k, GG_SITE));
      const unsigned bal = __ballot_sync(GG_FULL, hit);
      if (bal) {
        if (lane == 0) atomicMin(first + h, base + (unsigned long long)(__ffs(bal) - 1));
        break;
      }
    }
  }
}

static __global__ void __launch_bounds__(PULL_THREADS)
    bfs_heavy_finish(Dir d, const unsigned long long *__restrict__ first, uint32_t *parent, ActOut act,
                     Counters *ctr) {
  Tally t;
  const size_t n = ((size_t)d.nheavy + 31) / 32 * 32;
  for (size_t h = (size_t)blockIdx.x * blockDim.x + threadIdx.x; h < n; h += (size_t)gridDim.x * blockDim.x) {
    bool a = false;
    uint32_t v = 0;
    if (h < d.nheavy) {
      v = d.heavy[h];
      const unsigned long long f = first[h];
      if (f != ~0ull && !bm_test(act.visited, v)) {
        parent[v] = nbr_at(d, f, GG_SITE);
        a = true;
      }
    }
    push_activate(a, v, act, t);
  }
  t.flush(ctr);
}

// ---------------------------------------------------------------- small sparse runs
// A run of consecutive sparse calls whose frontiers are small (high-diameter
// graphs such as grids, and the tails of power-law BFS) is driven from the
// device: each call is one push_small launch (plus a snapshot gather for CC
// and SSSP) that reads its queue length and active_edges from SmallRun; the
// last block to finish (a ticket counter, no waiting) writes the call's trace
// row, moves the accumulated counters to the next call, and decides whether
// the next call may also run here -- the same switch (sparse iff active_edges
// < edges/20) plus size limits.  The host enqueues a batch of launches without
// synchronising; launches after the run stops return at once.
constexpr int SMALL_THREADS = 256;
constexpr uint32_t SMALL_BATCH = 512;        // calls enqueued per host round trip
constexpr uint32_t SMALL_MAX_QUEUE = 65536;  // largest queue a small call takes
constexpr unsigned long long SMALL_MAX_AE = 1ull << 20;
constexpr uint32_t SMALL_MAX_DEG = 1024;     // largest out-degree in a small call's queue
constexpr int COOP_BLOCKS = 32;              // blocks of a cooperative small run (all resident)

struct SmallRun {
  unsigned long long ae;         // active_edges of the call about to run
  unsigned long long edges_lim;  // edges / 20
  unsigned long long total_ae;   // sum of active_edges over the run's calls
  unsigned int n;                // its queue length
  unsigned int go;               // the next launch runs a call
  unsigned int calls;            // trace rows written in this batch
  unsigned int level;            // activation stamp of the current call (> 0)
  unsigned int ticket;           // blocks finished in the current call
  unsigned int last_activated;   // activated count of the last call
  unsigned int maxdeg;           // largest out-degree in the queue of the call about to run
  Counters next;                 // accumulators of the current call
};

// Queue append from divergent lanes: one atomic per group of lanes that
// reach this point together.
__device__ __forceinline__ void queue_append_any(uint32_t v, uint32_t *q, unsigned *qlen) {
  const unsigned am = __activemask();
  const int leader = __ffs(am) - 1;
  const unsigned lane = lane_id();
  unsigned base = 0;
  if ((int)lane == leader) base = atomicAdd(qlen, (unsigned)__popc(am));
  base = __shfl_sync(am, base, leader);
  q[base + __popc(am & ((1u << lane) - 1u))] = v;
}

// Activation inside a small push call: stamp-deduplicated unless the op's
// slot already lets one thread win (BFS's CAS).  Lanes may be divergent.
template <bool kUnique>
__device__ __forceinline__ void small_activate(uint32_t v, SmallRun *st, uint32_t *stamp, unsigned level,
                                               uint32_t *visited, uint32_t *q_out, const uint32_t *out_deg,
                                               const uint32_t *in_deg, Tally &t) {
  if (!kUnique) {
    if (stamp[v] == level || atomicExch(stamp + v, level) == level) return;
  }
  if (visited) atomicOr(visited + (v >> 5), 1u << (v & 31));
  uint32_t od = out_deg[v];
  t.activated += 1;
  t.edges += od;
  t.maxdeg = od > t.maxdeg ? od : t.maxdeg;
  if (in_deg) t.in_edges += in_deg[v];
  if (od > 0) queue_append_any(v, q_out, &st->next.qlen);
}

// One small push call over q_in (n entries): slots, activation, and the
// call's tally flushed into st->next.  Every thread of the block calls it.
template <class Op, bool kUnique>
__device__ __forceinline__ void small_call(SmallRun *st, const uint32_t *__restrict__ q_in, uint32_t *__restrict__ q_out,
                                           const Dir &d, const Op &op, uint32_t *stamp, uint32_t *visited,
                                           const uint32_t *__restrict__ out_deg, const uint32_t *__restrict__ in_deg,
                                           uint32_t n, unsigned level) {
  const unsigned lane = lane_id();
  Tally t;
  const size_t nround = ((size_t)n + 31) / 32 * 32;
  for (size_t i = (size_t)blockIdx.x * SMALL_THREADS + threadIdx.x; i < nround; i += (size_t)gridDim.x * SMALL_THREADS) {
    const bool valid = i < n;
    uint32_t src = 0;
    unsigned long long b = 0, e = 0;
    if (valid) {
      src = q_in[i];
      b = d.off[src];
      e = d.off[src + 1];
    }
    if (valid && e - b <= LIGHT_DEG) {
      for (unsigned long long k = b; k < e; k++) {
        uint32_t dst = nbr_at(d, k, GG_SITE);
        if (op.push(src, (uint32_t)i, dst, d.w ? d.w[k] : 0.0f))
          small_activate<kUnique>(dst, st, stamp, level, visited, q_out, out_deg, in_deg, t);
      }
    }
    unsigned coop = __ballot_sync(GG_FULL, valid && e - b > LIGHT_DEG);
    while (coop) {
      const unsigned leader = __ffs(coop) - 1;
      coop &= coop - 1;
      const unsigned long long lb = __shfl_sync(GG_FULL, b, leader), le = __shfl_sync(GG_FULL, e, leader);
      const uint32_t lsrc = __shfl_sync(GG_FULL, src, leader);
      const uint32_t li = (uint32_t)__shfl_sync(GG_FULL, (unsigned long long)i, leader);
      for (unsigned long long k = lb + lane; k < le; k += 32) {
        uint32_t dst = nbr_at(d, k, GG_SITE);
        if (op.push(lsrc, li, dst, d.w ? d.w[k] : 0.0f))
          small_activate<kUnique>(dst, st, stamp, level, visited, q_out, out_deg, in_deg, t);
      }
    }
  }
  t.flush(&st->next);
}

// small_call with the tally and the queue counter in `tally` (the
// cooperative path keeps three of them).
template <bool kUnique>
__device__ __forceinline__ void small_activate_t(uint32_t v, Counters *tally, uint32_t *stamp, unsigned level,
                                                 uint32_t *visited, uint32_t *q_out, const uint32_t *out_deg,
                                                 const uint32_t *in_deg, Tally &t) {
  if (!kUnique) {
    if (stamp[v] == level || atomicExch(stamp + v, level) == level) return;
  }
  if (visited) atomicOr(visited + (v >> 5), 1u << (v & 31));
  uint32_t od = out_deg[v];
  t.activated += 1;
  t.edges += od;
  t.maxdeg = od > t.maxdeg ? od : t.maxdeg;
  if (in_deg) t.in_edges += in_deg[v];
  if (od > 0) queue_append_any(v, q_out, &tally->qlen);
}
template <class Op, bool kUnique>
__device__ __forceinline__ void small_call_t(Counters *tally, const uint32_t *__restrict__ q_in,
                                             uint32_t *__restrict__ q_out, const Dir &d, const Op &op,
                                             uint32_t *stamp, uint32_t *visited,
                                             const uint32_t *__restrict__ out_deg,
                                             const uint32_t *__restrict__ in_deg, uint32_t n, unsigned level) {
  const unsigned lane = lane_id();
  Tally t;
  const size_t nround = ((size_t)n + 31) / 32 * 32;
  for (size_t i = (size_t)blockIdx.x * SMALL_THREADS + threadIdx.x; i < nround; i += (size_t)gridDim.x * SMALL_THREADS) {
    const bool valid = i < n;
    uint32_t src = 0;
    unsigned long long b = 0, e = 0;
    if (valid) {
      src = q_in[i];
      b = d.off[src];
      e = d.off[src + 1];
    }
    if (valid && e - b <= LIGHT_DEG) {
      for (unsigned long long k = b; k < e; k++) {
        uint32_t dst = nbr_at(d, k, GG_SITE);
        if (op.push(src, (uint32_t)i, dst, d.w ? d.w[k] : 0.0f))
          small_activate_t<kUnique>(dst, tally, stamp, level, visited, q_out, out_deg, in_deg, t);
      }
    }
    unsigned coop = __ballot_sync(GG_FULL, valid && e - b > LIGHT_DEG);
    while (coop) {
      const unsigned leader = __ffs(coop) - 1;
      coop &= coop - 1;
      const unsigned long long lb = __shfl_sync(GG_FULL, b, leader), le = __shfl_sync(GG_FULL, e, leader);
      const uint32_t lsrc = __shfl_sync(GG_FULL, src, leader);
      const uint32_t li = (uint32_t)__shfl_sync(GG_FULL, (unsigned long long)i, leader);
      for (unsigned long long k = lb + lane; k < le; k += 32) {
        uint32_t dst = nbr_at(d, k, GG_SITE);
        if (op.push(lsrc, li, dst, d.w ? d.w[k] : 0.0f))
          small_activate_t<kUnique>(dst, tally, stamp, level, visited, q_out, out_deg, in_deg, t);
      }
    }
  }
  t.flush(tally);
}

// Closes a small call (one thread, after every block's tally is in): the
// trace row, the next call's queue and switch value, and whether it runs.
__device__ __forceinline__ void small_close(SmallRun *st, unsigned long long *tr_ae, unsigned int *tr_act,
                                            unsigned level) {
  const unsigned long long ne = atomicAdd(&st->next.edges, 0ull);
  const unsigned int na = atomicAdd(&st->next.activated, 0u);
  const unsigned int nq = atomicAdd(&st->next.qlen, 0u);
  const unsigned int nm = atomicAdd(&st->next.maxdeg, 0u);
  const unsigned int r = st->calls;
  tr_ae[r] = st->ae;
  tr_act[r] = na;
  st->calls = r + 1;
  st->total_ae += st->ae;
  st->level = level + 1;
  st->ae = ne;
  st->n = nq;
  st->last_activated = na;
  st->next.edges = 0;
  st->next.in_edges = 0;
  st->next.activated = 0;
  st->next.qlen = 0;
  st->next.maxdeg = 0;
  st->ticket = 0;
  st->maxdeg = nm;
  st->go = (na > 0 && ne < st->edges_lim && nq <= SMALL_MAX_QUEUE && ne <= SMALL_MAX_AE && nm <= SMALL_MAX_DEG)
               ? 1u
               : 0u;
  __threadfence();
}

template <class Op, bool kUnique>
__global__ void __launch_bounds__(SMALL_THREADS)
    push_small(SmallRun *st, const uint32_t *__restrict__ q_in, uint32_t *__restrict__ q_out, Dir d, Op op,
               uint32_t *stamp, uint32_t *visited, const uint32_t *__restrict__ out_deg,
               const uint32_t *__restrict__ in_deg, unsigned long long *tr_ae, unsigned int *tr_act) {
  __shared__ unsigned s_go, s_n, s_level, s_last;
  if (threadIdx.x == 0) {
    s_go = st->go;
    s_n = st->n;
    s_level = st->level;
  }
  __syncthreads();
  if (!s_go) return;
  small_call<Op, kUnique>(st, q_in, q_out, d, op, stamp, visited, out_deg, in_deg, s_n, s_level);
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    s_last = atomicAdd(&st->ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (s_last && threadIdx.x == 0) {
    __threadfence();
    small_close(st, tr_ae, tr_act, s_level);
  }
}

// The same calls in one cooperative launch: up to max_calls of them, the
// queues alternating (qa -> qb, then qb -> qa, ...), one grid-wide barrier
// per call.  Call c's tally goes to tally[c % 3]; after the barrier every
// block reads it and derives the next call's queue length, switch value and
// whether it runs (identical in all blocks, so all leave the loop together);
// block 0 writes the trace row and clears tally[(c + 1) % 3], which no block
// reads any more (the last reads were before the previous barrier).
template <class Op, bool kUnique>
__global__ void __launch_bounds__(SMALL_THREADS)
    push_small_coop(SmallRun *st, Counters *tally, uint32_t *qa, uint32_t *qb, Dir d, Op op, uint32_t *stamp,
                    uint32_t *visited, const uint32_t *__restrict__ out_deg, const uint32_t *__restrict__ in_deg,
                    unsigned long long *tr_ae, unsigned int *tr_act, unsigned max_calls) {
  cooperative_groups::grid_group grid = cooperative_groups::this_grid();
  unsigned n = st->n, level = st->level, go = st->go, maxdeg = st->maxdeg, na = 0;
  unsigned long long ae = st->ae, total = st->total_ae;
  const unsigned long long lim = st->edges_lim;
  unsigned c = 0;
  for (; c < max_calls && go; c++) {
    Counters *cur = tally + (c % 3);
    if (blockIdx.x == 0 && threadIdx.x == 0) memset(tally + ((c + 1) % 3), 0, sizeof(Counters));
    small_call_t<Op, kUnique>(cur, (c & 1) ? qb : qa, (c & 1) ? qa : qb, d, op, stamp, visited, out_deg, in_deg, n,
                              level);
    grid.sync();
    const unsigned long long ne = *(volatile unsigned long long *)&cur->edges;
    na = *(volatile unsigned *)&cur->activated;
    const unsigned nq = *(volatile unsigned *)&cur->qlen;
    const unsigned nm = *(volatile unsigned *)&cur->maxdeg;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      tr_ae[c] = ae;
      tr_act[c] = na;
    }
    total += ae;
    level += 1;
    ae = ne;
    n = nq;
    maxdeg = nm;
    go = (na > 0 && ne < lim && nq <= SMALL_MAX_QUEUE && ne <= SMALL_MAX_AE && nm <= SMALL_MAX_DEG) ? 1u : 0u;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    st->calls = c;
    st->total_ae = total;
    st->level = level;
    st->ae = ae;
    st->n = n;
    st->last_activated = na;
    st->maxdeg = maxdeg;
    st->go = go;
    __threadfence();
  }
}

// Snapshot gather of a small call (CC, SSSP): msg[i] = src[q[i]].
template <typename T>
__global__ void small_gather(const SmallRun *st, const uint32_t *__restrict__ q, const T *__restrict__ src,
                             T *__restrict__ msg) {
  if (!st->go) return;
  const uint32_t n = st->n;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    msg[i] = src[q[i]];
}

// ---------------------------------------------------------------- queue from bitmap
// popcount of (bm & mask) per 32-bit word: the scan input of queue_from_bitmap.
struct MaskedPopc {
  const uint32_t *bm;
  const uint32_t *mask;
  __device__ __forceinline__ uint32_t operator()(size_t i) const {
    uint32_t w = bm[i];
    if (mask) w &= mask[i];
    return (uint32_t)__popc(w);
  }
};

// q[pos[i] ...] = the vertices of word i of (bm & mask), ascending.
static __global__ void queue_scatter(const uint32_t *__restrict__ bm, const uint32_t *__restrict__ mask,
                                     size_t words, const uint32_t *__restrict__ pos, uint32_t *__restrict__ q) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < words; i += (size_t)gridDim.x * blockDim.x) {
    uint32_t w = bm[i];
    if (mask) w &= mask[i];
    uint32_t p = pos[i];
    while (w) {
      uint32_t b = __ffs(w) - 1;
      w &= w - 1;
      q[p++] = (uint32_t)(i * 32 + b);
    }
  }
}

// ---------------------------------------------------------------- small kernels
// out[i] = src[q[i]]: the message snapshot of a push call's queued vertices.
template <typename T>
static __global__ void gather_by_queue(const uint32_t *__restrict__ q, uint32_t n, const T *__restrict__ src,
                                       T *__restrict__ out) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    out[i] = src[q[i]];
}

template <typename T>
static __global__ void fill_kernel(T *__restrict__ a, size_t n, T v) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    a[i] = v;
}

static __global__ void iota_u32(uint32_t *__restrict__ a, uint32_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    a[i] = (uint32_t)i;
}

// dst |= src, word by word.
static __global__ void bitmap_or(uint32_t *__restrict__ dst, const uint32_t *__restrict__ src, size_t words) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < words; i += (size_t)gridDim.x * blockDim.x)
    dst[i] |= src[i];
}

// Sets the bits of the n queued vertices.
static __global__ void bitmap_from_queue(const uint32_t *__restrict__ q, uint32_t n, uint32_t *__restrict__ bm) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    uint32_t v = q[i];
    atomicOr(bm + (v >> 5), 1u << (v & 31));
  }
}

// Bitmap::fill (core/bitmap.hpp:42-52): bits [0, V) set, the rest clear.
static __global__ void bitmap_fill(uint32_t *__restrict__ bm, size_t words, uint32_t V) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < words; i += (size_t)gridDim.x * blockDim.x) {
    size_t lo = i * 32;
    uint32_t w;
    if (lo + 32 <= V)
      w = 0xffffffffu;
    else if (lo >= V)
      w = 0u;
    else
      w = (1u << (V - lo)) - 1u;
    bm[i] = w;
  }
}

// Launch helpers shared by the toolkits.
struct Launch {
  gg_graph *g;
  int launches = 0;
  explicit Launch(gg_graph *gr) : g(gr) {}
  unsigned pull_grid() const { return grid_for(((size_t)g->V + 31) / 32 * 32, PULL_THREADS, g->num_sms, 8); }
  unsigned push_grid(unsigned long long total) const {
    unsigned long long tiles = (total + PUSH_TILE - 1) / PUSH_TILE;
    unsigned long long cap = (unsigned long long)g->num_sms * 8;
    return (unsigned)(tiles < 1 ? 1 : (tiles > cap ? cap : tiles));
  }
  unsigned med_grid(const Dir &d) const {
    return grid_for((size_t)d.nmed * 32, PULL_THREADS, g->num_sms, 8);
  }
  unsigned heavy_grid(const Dir &d) const {
    return grid_for((size_t)d.nchunks * 32, PULL_THREADS, g->num_sms, 8);
  }
  // Kernels one reduction pull launches.
  static int pull_launches(const Dir &d) { return d.nbig ? 3 : 1; }
  // All bins of one dense call, in order: light, medium, heavy chunks, heavy finish.
  template <class Op>
  int pull(const Dir &d, const Op &op, const ActOut &act, Counters *ctr) {
    cudaStream_t s = g->stream;
    // light lists on the side stream, beside the chunk kernel (disjoint
    // vertices); the finish, which sets bitmap bits atomically in words the
    // light kernel stores whole, runs after the join
    const bool fork = d.nbig && g->side;
    if (fork) {
      GG_CUDA(cudaEventRecord(g->fork, s));
      GG_CUDA(cudaStreamWaitEvent(g->side, g->fork, 0));
    }
    // split: both kernels resident on every SM at once (8 blocks of 256
    // threads fill an SM), rather than the chunk kernel waiting for the
    // light kernel's blocks to retire
    const uint32_t split = fork && g->pull_light_blocks > 0 && g->pull_light_blocks < 8 ? g->pull_light_blocks : 0;
    unsigned lg = pull_grid();
    if (split) lg = grid_for(((size_t)g->V + 31) / 32 * 32, PULL_THREADS, g->num_sms, (int)split);
    if (d.vec & 2)
      pull_light<Op, true><<<lg, PULL_THREADS, 0, fork ? g->side : s>>>(d, g->V, op, act, ctr);
    else
      pull_light<Op, false><<<lg, PULL_THREADS, 0, fork ? g->side : s>>>(d, g->V, op, act, ctr);
    launches += 1;
    if (fork) GG_CUDA(cudaEventRecord(g->join, g->side));
    if (d.nbig) {
      typename Op::Acc *part = nullptr;
      GG_TRY(ws(g, WS_PARTIAL, d.nbigchunks, &part));
      const unsigned cg = grid_for((size_t)d.nbigchunks * 32, PULL_THREADS, g->num_sms, split ? 8 - (int)split : 8);
      if (d.vec & 1) {
        if (d.chunk == 128)
          pull_chunks<Op, 4, true><<<cg, PULL_THREADS, 0, s>>>(d, op, part);
        else if (d.chunk == 512)
          pull_chunks<Op, 16, true><<<cg, PULL_THREADS, 0, s>>>(d, op, part);
        else
          pull_chunks<Op, 8, true><<<cg, PULL_THREADS, 0, s>>>(d, op, part);
      } else {
        if (d.chunk == 128)
          pull_chunks<Op, 4, false><<<cg, PULL_THREADS, 0, s>>>(d, op, part);
        else if (d.chunk == 512)
          pull_chunks<Op, 16, false><<<cg, PULL_THREADS, 0, s>>>(d, op, part);
        else
          pull_chunks<Op, 8, false><<<cg, PULL_THREADS, 0, s>>>(d, op, part);
      }
      if (fork) GG_CUDA(cudaStreamWaitEvent(s, g->join, 0));
      if (act.active_out)
        pull_big_finish<Op><<<grid_for(d.nbig, PULL_THREADS, g->num_sms, 8), PULL_THREADS, 0, s>>>(d, op, part, act,
                                                                                                    ctr);
      else
        pull_big_finish_warps<Op><<<grid_for((size_t)d.nbig * 32, PULL_THREADS, g->num_sms, 8), PULL_THREADS, 0, s>>>(
            d, op, part, ctr);
      launches += 2;
    }
    GG_CUDA(cudaGetLastError());
    return GG_OK;
  }
  int bfs_pull(const Dir &d, const uint32_t *active_in, uint32_t *parent, const ActOut &act, Counters *ctr) {
    cudaStream_t s = g->stream;
    bfs_pull_light<<<pull_grid(), PULL_THREADS, 0, s>>>(d, g->V, active_in, parent, act, ctr);
    launches += 1;
    if (d.nmed) {
      bfs_pull_medium<<<med_grid(d), PULL_THREADS, 0, s>>>(d, active_in, parent, act, ctr);
      launches += 1;
    }
    if (d.nheavy) {
      unsigned long long *first = nullptr;
      GG_TRY(ws(g, WS_PARTIAL, d.nheavy, &first));
      GG_CUDA(cudaMemsetAsync(first, 0xff, sizeof(unsigned long long) * d.nheavy, s));
      bfs_heavy_first<<<heavy_grid(d), PULL_THREADS, 0, s>>>(d, active_in, act.visited, first);
      bfs_heavy_finish<<<grid_for(d.nheavy, PULL_THREADS, g->num_sms, 8), PULL_THREADS, 0, s>>>(d, first, parent,
                                                                                                act, ctr);
      launches += 2;
    }
    GG_CUDA(cudaGetLastError());
    return GG_OK;
  }
  // Ordered queue of the set bits of bm (restricted to mask when non-null);
  // *n receives its length.
  int queue_from_bitmap(const uint32_t *bm, const uint32_t *mask, uint32_t *q, uint32_t *n) {
    size_t words = bitmap_words32(g->V);
    uint32_t *pos = nullptr, *scratch = nullptr;
    GG_TRY(ws(g, WS_QPOS, words + 1, &pos));
    GG_TRY(ws(g, WS_SCAN32, scan_scratch_elems(words), &scratch));
    GG_CUDA((exclusive_scan<uint32_t, MaskedPopc>(MaskedPopc{bm, mask}, words, pos, scratch, g->stream,
                                                  &launches)));
    queue_scatter<<<grid_for(words, 256, g->num_sms, 8), 256, 0, g->stream>>>(bm, mask, words, pos, q);
    launches += 1;
    GG_CUDA(cudaGetLastError());
    return read_small(g, n, pos + words, sizeof(uint32_t));
  }
  // Runs consecutive small sparse calls on the device (see SmallRun).  On
  // entry q[*cur] holds the active vertices with out-degree > 0 (nq of them)
  // and ae is the call's active_edges.  On return *cur, *nq, *ae describe the
  // first call that did not run here and *n_act is the previous call's
  // activated count; the trace has one row per call that ran.
  template <class Op, bool kUnique, typename T>
  int small_run(const Dir &d, const Op &op, uint32_t *q[2], int *cur, uint32_t *nq, unsigned long long *ae,
                uint32_t *maxdeg, uint32_t *n_act, uint32_t *visited, const uint32_t *in_deg, const T *snap_src, T *snap_msg,
                Trace &tr, uint32_t *stamp) {
    SmallRun *st;
    unsigned long long *tr_ae;
    unsigned *tr_act;
    char *blob;
    const size_t st_bytes = 256, ae_bytes = sizeof(unsigned long long) * SMALL_BATCH;
    const size_t act_bytes = sizeof(unsigned) * SMALL_BATCH;
    GG_TRY(ws(g, WS_SMALL, st_bytes + ae_bytes + act_bytes + 3 * sizeof(Counters) + 64, &blob));
    Counters *coop_tally = (Counters *)(blob + ((st_bytes + ae_bytes + act_bytes + 63) / 64 * 64));
    st = (SmallRun *)blob;
    tr_ae = (unsigned long long *)(blob + st_bytes);
    tr_act = (unsigned *)(blob + st_bytes + ae_bytes);
    static thread_local std::vector<unsigned long long> h_ae;
    static thread_local std::vector<unsigned> h_act;
    h_ae.resize(SMALL_BATCH);
    h_act.resize(SMALL_BATCH);
    SmallRun h;
    memset(&h, 0, sizeof(h));
    h.ae = *ae;
    h.edges_lim = g->E / 20;
    h.n = *nq;
    h.go = 1;
    h.maxdeg = *maxdeg;
    h.level = next_level();
    cudaStream_t s = g->stream;
    const unsigned grid = grid_for(SMALL_MAX_QUEUE, SMALL_THREADS, g->num_sms, 1);
    // batches of 2, 4, 8, ... launches: a short run wastes few no-op launches;
    // full batches of a long run replay one captured CUDA graph
    auto enqueue = [&](uint32_t n) {
      for (uint32_t i = 0; i < n; i++) {
        const int c = *cur ^ (int)(i & 1);
        if (snap_msg) small_gather<T><<<grid, SMALL_THREADS, 0, s>>>(st, q[c], snap_src, snap_msg);
        push_small<Op, kUnique><<<grid, SMALL_THREADS, 0, s>>>(st, q[c], q[c ^ 1], d, op, stamp, visited,
                                                                d.deg, in_deg, tr_ae, tr_act);
      }
    };
    cudaGraphExec_t exec = nullptr;
    int exec_parity = -1;
    int status = GG_OK;
    // Without message snapshots the calls need no host step between them: one
    // cooperative launch runs a whole batch (grid = one block per SM, all
    // resident by the cooperative launch's guarantee) and stops early.
    const bool coop = !snap_msg && coop_ok();
    uint32_t batch = coop ? SMALL_BATCH : 2;
    for (;;) {
      cudaError_t e = cudaMemcpyAsync(st, &h, sizeof(h), cudaMemcpyHostToDevice, s);
      if (e == cudaSuccess && coop) {
        uint32_t *qa = q[*cur], *qb = q[*cur ^ 1];
        Dir dd = d;
        Op oo = op;
        const uint32_t *deg = d.deg;
        unsigned mc = batch;
        Counters *tally = coop_tally;
        e = cudaMemsetAsync(tally, 0, sizeof(Counters), s);
        void *args[] = {&st, &tally, &qa, &qb, &dd, &oo, &stamp, &visited, (void *)&deg, (void *)&in_deg,
                        &tr_ae, &tr_act, &mc};
        if (e == cudaSuccess)
          e = cudaLaunchCooperativeKernel((const void *)push_small_coop<Op, kUnique>, dim3(COOP_BLOCKS),
                                          dim3(SMALL_THREADS), args, 0, s);
        launches += 1;
      } else if (e == cudaSuccess && batch == SMALL_BATCH) {
        if (!exec || exec_parity != *cur) {
          if (exec) cudaGraphExecDestroy(exec);
          exec = nullptr;
          cudaGraph_t graph = nullptr;
          e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
          if (e == cudaSuccess) {
            enqueue(batch);
            e = cudaStreamEndCapture(s, &graph);
          }
          if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
          if (graph) cudaGraphDestroy(graph);
          exec_parity = *cur;
        }
        if (e == cudaSuccess) e = cudaGraphLaunch(exec, s);
      } else if (e == cudaSuccess) {
        enqueue(batch);
      }
      if (e == cudaSuccess) e = cudaGetLastError();
      if (e != cudaSuccess) {
        status = cuda_status(e, "small run");
        break;
      }
      if (!coop) launches += batch * (snap_msg ? 2 : 1);
      status = read_small(g, &h, st, sizeof(h));
      if (status == GG_OK) status = read_small(g, h_ae.data(), tr_ae, sizeof(unsigned long long) * batch);
      if (status == GG_OK) status = read_small(g, h_act.data(), tr_act, sizeof(unsigned) * batch);
      if (status != GG_OK) break;
      for (uint32_t r = 0; r < h.calls; r++) {
        tr.add(0, h_ae[r], h_act[r]);
        *n_act = h_act[r];
      }
      *cur ^= (int)(h.calls & 1);
      level_ = h.level;
      if (h.go) {  // the batch ended with the run still going
        h.calls = 0;
        batch = batch * 2 < SMALL_BATCH ? batch * 2 : SMALL_BATCH;
        continue;
      }
      break;
    }
    if (exec) cudaGraphExecDestroy(exec);
    if (status != GG_OK) return status;
    *nq = h.n;
    *ae = h.ae;
    *maxdeg = h.maxdeg;
    return GG_OK;
  }
  // Cooperative launches available (queried once per device).
  bool coop_ok() const {
    int v = 0;
    return cudaDeviceGetAttribute(&v, cudaDevAttrCooperativeLaunch, g->device) == cudaSuccess && v;
  }
  static bool small_ok(uint32_t nq, unsigned long long ae, uint32_t maxdeg) {
    return ae > 0 && nq <= SMALL_MAX_QUEUE && ae <= SMALL_MAX_AE && maxdeg <= SMALL_MAX_DEG;
  }
  // Activation stamps grow across small runs of one graph; 0 marks "never".
  unsigned level_ = 0;
  unsigned next_level() { return level_ + 1; }
  int scan_queue_degrees(const uint32_t *q, uint32_t n, const uint32_t *deg, unsigned long long **P) {
    unsigned long long *p = nullptr, *scratch = nullptr;
    GG_TRY(ws(g, WS_PREFIX, (size_t)g->V + 2, &p));
    GG_TRY(ws(g, WS_SCAN, scan_scratch_elems((size_t)g->V + 1), &scratch));
    GG_CUDA((exclusive_scan<unsigned long long, QueueDegreeIn>(QueueDegreeIn{q, deg}, n, p, scratch, g->stream,
                                                               &launches)));
    *P = p;
    return GG_OK;
  }
};

}  // namespace gg

#endif
