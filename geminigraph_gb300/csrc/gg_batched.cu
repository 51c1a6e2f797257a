// Batched multi-source BFS and SSSP: up to 64 roots per traversal, one bit
// (BFS) or one float slot (SSSP) per root ("lane") for every vertex.  The
// reference has no batching; each lane's result equals the single-root
// toolkit's on the same root (BFS levels identical and parents a valid BFS
// tree, as for gg_bfs; SSSP distances bit-identical -- the least fixpoint of
// fl(d[u] + w) does not depend on the relaxation order).
//
// Layout (vertex-major, so one vertex's lanes share cache lines):
//   visit, front, next   uint64[V]   lane bit masks
//   lvl, par             uint32[V*64] discovery iteration / parent per lane
//   dist                 float[V*64]  SSSP distances per lane
// One iteration advances every live lane by one level.  It is a pull (each
// vertex gathers the lanes that reach it from its in-neighbours' frontier
// masks) when the union frontier's out-edges are >= edges/20, else a push
// over the union frontier's out-edges -- the reference's switch rule applied
// to the union.  Lanes are independent, so a lane that finishes leaves its bit
// clear and the others go on.
#include <math.h>
#include <string.h>

#include <vector>

#include "gg_engine.cuh"
#include "gg_gen.h"

#include "gg_lanes.cuh"

namespace gg {

typedef unsigned long long u64;
constexpr int LANES = 64;

typedef LaneCounters MsCounters;

// write_min on a float (core/atomic.hpp:35-42): true if this call lowered *p.
__device__ __forceinline__ bool atomic_min_float_b(float *p, float v) {
  if (!(v < 0.0f)) {
    int old = atomicMin((int *)p, __float_as_int(v));
    return __int_as_float(old) > v;
  }
  unsigned old = atomicMax((unsigned *)p, __float_as_uint(v));
  return __uint_as_float(old) > v;
}

__device__ __forceinline__ u64 warp_or64(u64 x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x |= __shfl_xor_sync(GG_FULL, x, o);
  return x;
}

// Block-level flush of the per-thread iteration tallies.
__device__ __forceinline__ void ms_flush(MsCounters *mc, u64 alive, u64 edges, unsigned touched) {
  __shared__ u64 s_a[32], s_e[32];
  __shared__ unsigned s_t[32];
  alive = warp_or64(alive);
  edges = warp_sum(edges);
  touched = warp_sum(touched);
  unsigned w = threadIdx.x >> 5, lane = lane_id();
  if (lane == 0) {
    s_a[w] = alive;
    s_e[w] = edges;
    s_t[w] = touched;
  }
  __syncthreads();
  if (w == 0) {
    unsigned nw = (blockDim.x + 31) >> 5;
    alive = lane < nw ? s_a[lane] : 0ull;
    edges = lane < nw ? s_e[lane] : 0ull;
    touched = lane < nw ? s_t[lane] : 0u;
    alive = warp_or64(alive);
    edges = warp_sum(edges);
    touched = warp_sum(touched);
    if (lane == 0) {
      if (alive) atomicOr(&mc->alive, alive);
      if (edges) atomicAdd(&mc->edges, edges);
      if (touched) atomicAdd(&mc->touched, touched);
    }
  }
}

__device__ __forceinline__ void ms_record(uint32_t v, u64 bits, uint32_t u, uint32_t iter, uint32_t *lvl,
                                          uint32_t *par) {
  while (bits) {
    const int l = __ffsll((long long)bits) - 1;
    bits &= bits - 1;
    lvl[(size_t)v * LANES + l] = iter;
    if (par) par[(size_t)v * LANES + l] = u;
  }
}

// Levels of newly reached lanes, written a 256-byte row at a time (lvl null:
// the sums only, the levels going to a level list): each lane
// of the warp holds a vertex v with its new lanes m and out-degree dg; for
// every vertex with lanes, thread t writes lvl[v][t] and lvl[v][t + 32] where
// set and adds them to its per-lane sums (reached, out-degree).
struct LaneSums {
  u64 c0 = 0, c1 = 0, e0 = 0, e1 = 0;
  // all threads of the block call it (shared-memory reduction, then one
  // atomic per lane and block)
  __device__ __forceinline__ void flush(u64 *lane_sum) {
    __shared__ u64 s_sum[2 * LANES];
    for (int i = threadIdx.x; i < 2 * LANES; i += blockDim.x) s_sum[i] = 0;
    __syncthreads();
    const unsigned lane = lane_id();
    if (c0) {
      atomicAdd(&s_sum[lane], c0);
      atomicAdd(&s_sum[LANES + lane], e0);
    }
    if (c1) {
      atomicAdd(&s_sum[lane + 32], c1);
      atomicAdd(&s_sum[LANES + lane + 32], e1);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 2 * LANES; i += blockDim.x)
      if (s_sum[i]) atomicAdd(lane_sum + i, s_sum[i]);
  }
};
__device__ __forceinline__ void mark_rows_warp(uint32_t v, u64 m, uint32_t dg, uint32_t *lvl, uint32_t iter,
                                               LaneSums &ls) {
  const unsigned lane = lane_id();
  unsigned bal = __ballot_sync(GG_FULL, m != 0);
  while (bal) {
    const int j = __ffs(bal) - 1;
    bal &= bal - 1;
    const uint32_t vj = __shfl_sync(GG_FULL, v, j);
    const unsigned lo = __shfl_sync(GG_FULL, (unsigned)m, j), hi = __shfl_sync(GG_FULL, (unsigned)(m >> 32), j);
    const uint32_t dj = __shfl_sync(GG_FULL, dg, j);
    uint32_t *row = lvl + (size_t)vj * LANES;
    if ((lo >> lane) & 1u) {
      if (lvl) row[lane] = iter;
      ls.c0 += 1;
      ls.e0 += dj;
    }
    if ((hi >> lane) & 1u) {
      if (lvl) row[lane + 32] = iter;
      ls.c1 += 1;
      ls.e1 += dj;
    }
  }
}

// Level-list slots a warp takes from the step's counter at a time (one
// atomic per LIST_CHUNK entries rather than per warp and vertex group); the
// slots a warp leaves unused hold empty entries (mask 0).
constexpr unsigned LIST_CHUNK = 256;
struct ListCursor {
  unsigned next = 0, end = 0;  // the warp's slots [next, end), the same in all lanes
  // Appends (v, iter, m) for the lanes whose m is nonzero.  All lanes call.
  __device__ __forceinline__ void push(u64 m, uint32_t v, uint32_t iter, LevelEntry *list, unsigned *n) {
    const unsigned b = __ballot_sync(GG_FULL, m != 0);
    if (!b) return;
    const unsigned cnt = __popc(b);
    if (end - next < cnt) {
      close(list);
      unsigned base = 0;
      if (lane_id() == 0) base = atomicAdd(n, LIST_CHUNK);
      next = __shfl_sync(GG_FULL, base, 0);
      end = next + LIST_CHUNK;
    }
    if (m) list[next + __popc(b & lanemask_lt())] = make_uint4(v, iter, (unsigned)m, (unsigned)(m >> 32));
    next += cnt;
  }
  // The unused slots as empty entries.  All lanes call.
  __device__ __forceinline__ void close(LevelEntry *list) {
    for (unsigned i = next + lane_id(); i < end; i += 32) list[i] = make_uint4(0, 0, 0, 0);
    next = end;
  }
};

// ---------------------------------------------------------------- BFS pull
// Light lists (<= LIGHT_DEG): the lane's own vertex, in CSC order, so each
// lane bit takes the first in-neighbour that has it (as bfs.cpp:63-66 does for
// one root).  next[v] is written for every v (0 for long lists, which the
// chunk kernel then ORs into).
// G: a step of the device-driven loop; the step's lanes, masks and
// iteration come from the pool state st (written by the previous kernel)
// instead of the arguments.  The same holds for every kernel below with G.
// L: the levels of newly reached lanes go to the level list (list, slots
// from mc->lpos) instead of the level rows.
template <bool G, bool L>
__global__ void __launch_bounds__(256)
    ms_pull_light(Dir d, uint32_t V, u64 alive, const u64 *__restrict__ front, u64 *visit, u64 *next, uint32_t *lvl,
                  uint32_t *par, uint32_t iter, const uint32_t *__restrict__ out_deg, MsCounters *mc,
                  u64 *lane_sum, const MsState *st, LevelEntry *list) {
  if (G) {
    alive = st->active;
    front = st->front;
    next = st->next;
    iter = st->iter;
  }
  u64 t_alive = 0, t_edges = 0;
  unsigned t_touched = 0;
  LaneSums ls;
  ListCursor lc;
  for (size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x; v < ((size_t)V + 255) / 256 * 256;
       v += (size_t)gridDim.x * blockDim.x) {
    u64 acc = 0;
    if (v < V) {
      const u64 vis = visit[v];
      u64 need = ~vis & alive;
      const unsigned long long b = d.off[v], e = d.off[v + 1];
      if (need && e - b <= d.light) {
        // four independent neighbour / frontier loads per step; within a
        // step any in-neighbour on a lane's frontier is a valid parent
        for (unsigned long long k = b; k < e && need; k += 4) {
          uint32_t u[4];
          u64 f[4];
#pragma unroll
          for (int i = 0; i < 4; i++) u[i] = k + i < e ? nbr_at(d, k + i, GG_SITE) : 0u;
#pragma unroll
          for (int i = 0; i < 4; i++) f[i] = k + i < e ? front[u[i]] : 0ull;
#pragma unroll
          for (int i = 0; i < 4; i++) {
            const u64 m = f[i] & need;
            if (m) {
              if (par) ms_record((uint32_t)v, m, u[i], iter, lvl, par);
              acc |= m;
              need &= ~m;
            }
          }
        }
      }
      next[v] = acc;
      if (acc) {
        visit[v] = vis | acc;
        t_alive |= acc;
        t_edges += out_deg[v];
        t_touched += 1;
      }
    }
    // levels of this warp's 32 vertices (without parents; long lists are
    // marked by ms_big_finish)
    if constexpr (L) lc.push(acc, (uint32_t)v, iter, list, &mc->lpos);
    if (lane_sum) mark_rows_warp((uint32_t)v, acc, acc ? out_deg[v] : 0u, L ? nullptr : lvl, iter, ls);
  }
  if (L) lc.close(list);
  ms_flush(mc, t_alive, t_edges, t_touched);
  if (lane_sum) ls.flush(lane_sum);
}

// Long lists: one warp per PULL_CHUNK-edge chunk; a lane bit goes to the
// entry that wins the atomicOr on next[v] (any in-neighbour in that lane's
// frontier is a valid parent).  visit[v] is not touched here.
template <bool G>
__global__ void __launch_bounds__(256)
    ms_pull_chunks(Dir d, u64 alive, const u64 *__restrict__ front, const u64 *__restrict__ visit, u64 *next,
                   uint32_t *lvl, uint32_t *par, uint32_t iter, const MsState *st) {
  if (G) {
    alive = st->active;
    front = st->front;
    next = st->next;
    iter = st->iter;
  }
  const size_t nwarps = (size_t)gridDim.x * 8;
  const unsigned lane = lane_id();
  for (size_t c = (size_t)blockIdx.x * 8 + (threadIdx.x >> 5); c < d.nbigchunks; c += nwarps) {
    uint32_t v;
    unsigned long long lo, b, e;
    big_range(d, (uint32_t)c, d.chunk, &v, &lo, &b, &e);
    u64 need = ~visit[v] & alive;
    if (!need) continue;
    for (unsigned long long base = b; base < e; base += 32) {
      need &= ~*(volatile u64 *)(next + v);
      if (!need) break;
      const unsigned long long k = base + lane;
      u64 m = 0;
      uint32_t u = 0;
      if (k < e) {
        u = nbr_at(d, k, GG_SITE);
        m = front[u] & need;
      }
      if (m) {
        const u64 won = m & ~atomicOr(next + v, m);
        if (won && par) ms_record(v, won, u, iter, lvl, par);
      }
    }
  }
}

// The same for a sparse step, over its queue of newly reached vertices: a
// warp per vertex (thread t: lanes t and t + 32).
template <bool G>
__global__ void __launch_bounds__(256)
    ms_mark_levels_q(const uint32_t *__restrict__ q, const unsigned *n_dev, const u64 *__restrict__ next,
                     uint32_t *lvl, uint32_t iter, const uint32_t *__restrict__ out_deg, u64 *lane_sum,
                     const MsState *st) {
  if (G) {
    q = st->qb;
    next = st->next;
    iter = st->iter;
  }
  __shared__ u64 s_sum[2 * LANES];
  for (int i = threadIdx.x; i < 2 * LANES; i += blockDim.x) s_sum[i] = 0;
  __syncthreads();
  const uint32_t n = *n_dev;
  const size_t nwarps = (size_t)gridDim.x * 8;
  const unsigned lane = lane_id();
  u64 c0 = 0, c1 = 0, e0 = 0, e1 = 0;
  for (size_t i = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += nwarps) {
    const uint32_t v = q[i];
    const u64 m = next[v];
    const uint32_t dg = out_deg[v];
    uint32_t *row = lvl + (size_t)v * LANES;
    if ((m >> lane) & 1ull) {
      if (lvl) row[lane] = iter;
      c0 += 1;
      e0 += dg;
    }
    if ((m >> (lane + 32)) & 1ull) {
      if (lvl) row[lane + 32] = iter;
      c1 += 1;
      e1 += dg;
    }
  }
  if (c0) {
    atomicAdd(&s_sum[lane], c0);
    atomicAdd(&s_sum[LANES + lane], e0);
  }
  if (c1) {
    atomicAdd(&s_sum[lane + 32], c1);
    atomicAdd(&s_sum[LANES + lane + 32], e1);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < 2 * LANES; i += blockDim.x)
    if (s_sum[i]) atomicAdd(lane_sum + i, s_sum[i]);
}


// visit |= next for the long-list vertices, and their tallies.
template <bool G, bool L>
__global__ void ms_big_finish(Dir d, u64 *visit, const u64 *__restrict__ next, const uint32_t *__restrict__ out_deg,
                              MsCounters *mc, uint32_t *lvl, uint32_t iter, u64 *lane_sum, const MsState *st,
                              LevelEntry *list) {
  if (G) {
    next = st->next;
    iter = st->iter;
  }
  u64 t_alive = 0, t_edges = 0;
  unsigned t_touched = 0;
  LaneSums ls;
  ListCursor lc;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < ((size_t)d.nbig + 255) / 256 * 256;
       i += (size_t)gridDim.x * blockDim.x) {
    uint32_t v = 0;
    u64 nx = 0;
    if (i < d.nbig) {
      v = d.big[i];
      nx = next[v];
      if (nx) {
        visit[v] |= nx;
        t_alive |= nx;
        t_edges += out_deg[v];
        t_touched += 1;
      }
    }
    if constexpr (L) lc.push(nx, v, iter, list, &mc->lpos);
    if (lane_sum) mark_rows_warp(v, nx, nx ? out_deg[v] : 0u, L ? nullptr : lvl, iter, ls);
  }
  if (L) lc.close(list);
  ms_flush(mc, t_alive, t_edges, t_touched);
  if (lane_sum) ls.flush(lane_sum);
}

// ---------------------------------------------------------------- BFS push
// Edge-balanced over the union frontier queue (as push_lb): for edge (u, v)
// the lanes m = front[u] & ~visit[v] claim v through atomicOr on next[v];
// the first claimer of v appends it to the touched queue.
template <bool G>
__global__ void __launch_bounds__(PUSH_THREADS)
    ms_push(const uint32_t *__restrict__ q, const unsigned long long *__restrict__ P, uint32_t n,
            unsigned long long total, Dir d, const u64 *__restrict__ front, const u64 *__restrict__ visit, u64 *next,
            uint32_t *lvl, uint32_t *par, uint32_t iter, uint32_t *q_out, MsCounters *mc, const MsState *st) {
  if (G) {
    q = st->qa;
    n = st->nq;
    total = st->ae;
    front = st->front;
    next = st->next;
    iter = st->iter;
    q_out = st->qb;
  }
  __shared__ uint32_t s_lo, s_hi;
  const unsigned long long ntiles = (total + PUSH_TILE - 1) / PUSH_TILE;
  for (unsigned long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const unsigned long long e0 = tile * PUSH_TILE;
    const unsigned long long e1 = e0 + PUSH_TILE < total ? e0 + PUSH_TILE : total;
    if (threadIdx.x == 0) {
      uint32_t lo = upper_bound_idx<unsigned long long>(P, 0, n + 1, e0) - 1;
      s_lo = lo;
      s_hi = upper_bound_idx<unsigned long long>(P, lo, n + 1, e1 - 1);
    }
    __syncthreads();
    const uint32_t lo = s_lo, hi = s_hi;
    __syncthreads();
    for (unsigned long long base = e0; base < e1; base += PUSH_THREADS) {
      const unsigned long long e = base + threadIdx.x;
      bool fresh = false;
      uint32_t v = 0;
      if (e < e1) {
        const uint32_t i = upper_bound_idx<unsigned long long>(P, lo, hi, e) - 1;
        const uint32_t u = q[i];
        v = nbr_at(d, d.off[u] + (e - P[i]), GG_SITE);
        const u64 m = front[u] & ~visit[v];
        if (m && (m & ~*(volatile u64 *)(next + v))) {
          const u64 old = atomicOr(next + v, m);
          const u64 won = m & ~old;
          if (won && par) ms_record(v, won, u, iter, lvl, par);
          fresh = old == 0;
        }
      }
      queue_push(fresh, v, q_out, &mc->qlen);
    }
  }
}

// After a push: visit |= next over the touched queue, and the tallies.
// n_dev: the queue length the push kernel counted (read on the device, so
// the host does not wait between the two kernels).
// list: entry i of the level list for queue entry i (iteration iter).
template <bool G>
__global__ void ms_push_finish(const uint32_t *__restrict__ q, const unsigned *n_dev, u64 *visit,
                               const u64 *__restrict__ next, const uint32_t *__restrict__ out_deg, MsCounters *mc,
                               const MsState *st, LevelEntry *list, uint32_t iter) {
  if (G) {
    q = st->qb;
    next = st->next;
  }
  const uint32_t n = *n_dev;
  u64 t_alive = 0, t_edges = 0;
  unsigned t_touched = 0;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < ((size_t)n + 255) / 256 * 256;
       i += (size_t)gridDim.x * blockDim.x) {
    if (i < n) {
      const uint32_t v = q[i];
      const u64 nx = next[v];
      visit[v] |= nx;
      if (list) list[i] = make_uint4(v, iter, (unsigned)nx, (unsigned)(nx >> 32));
      t_alive |= nx;
      t_edges += out_deg[v];
      t_touched += 1;
    }
  }
  ms_flush(mc, t_alive, t_edges, t_touched);
}

// Clears mask entries of the n queued vertices.
template <bool G>
__global__ void ms_clear_queue(const uint32_t *__restrict__ q, uint32_t n, u64 *mask, const MsState *st) {
  if (G) {
    q = st->qa;
    n = st->nq;
    mask = st->front;
  }
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    mask[q[i]] = 0;
}

// Ordered queue of the vertices with a nonzero mask.
struct NonzeroMask {
  const u64 *m;
  __device__ __forceinline__ uint32_t operator()(size_t i) const { return m[i] ? 1u : 0u; }
};
// The frontier of a device-driven step (the mask array st->front).
struct NonzeroFront {
  const MsState *st;
  __device__ __forceinline__ uint32_t operator()(size_t i) const { return st->front[i] ? 1u : 0u; }
};
// G: the frontier is st->front, the queue st->qa, and the queue's length
// (pos[V]) is recorded in st as a valid queue.
template <bool G>
__global__ void ms_compact(const u64 *__restrict__ m, uint32_t V, const uint32_t *__restrict__ pos,
                           uint32_t *__restrict__ q, MsState *st) {
  if (G) {
    m = st->front;
    q = st->qa;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      st->nq = pos[V];
      st->qvalid = 1;
    }
  }
  for (size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (size_t)gridDim.x * blockDim.x)
    if (m[v]) q[pos[v]] = (uint32_t)v;
}

// next[v] = 0 for every v (a push step after a pull step).
__global__ void ms_clear_next(const MsState *st, uint32_t V) {
  u64 *next = st->next;
  for (size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (size_t)gridDim.x * blockDim.x)
    next[v] = 0;
}

// Degree of entry i of the frontier queue of a device-driven step.
struct QueueDegreeSt {
  const MsState *st;
  const uint32_t *deg;
  __device__ __forceinline__ unsigned long long operator()(size_t i) const {
    return (unsigned long long)deg[st->qa[i]];
  }
};


// ---------------------------------------------------------------- pool kernels
// visit[v] &= ~mask: lanes about to be reused start unvisited everywhere.
__global__ void lanes_reset_visit(u64 *visit, uint32_t V, u64 mask) {
  for (size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (size_t)gridDim.x * blockDim.x)
    visit[v] &= ~mask;
}

// dist[v][l] = 1e9 for the lanes in mask.
__global__ void lanes_reset_dist(float *dist, uint32_t V, u64 mask) {
  const size_t n = (size_t)V * LANES;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    if ((mask >> (i % LANES)) & 1ull) dist[i] = 1e9f;
}

// Roots into lanes: frontier bit, visited bit / distance 0, discovery iteration.
// list: the roots' level-list entries (instead of their level rows).
__global__ void lanes_admit(const uint32_t *roots, const int *lanes, int n, u64 *front, u64 *visit, uint32_t *lvl,
                            uint32_t *par, float *dist, uint32_t iter, const uint32_t *out_deg, MsCounters *mc,
                            u64 *lane_sum, LevelEntry *list) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  u64 edges = 0;
  for (int i = 0; i < n; i++) {
    const uint32_t r = roots[i];
    const int l = lanes[i];
    if (!front[r]) edges += out_deg[r];
    front[r] |= 1ull << l;
    if (visit) visit[r] |= 1ull << l;
    if (list) {
      const u64 m = 1ull << l;
      list[i] = make_uint4(r, iter, (unsigned)m, (unsigned)(m >> 32));
    } else if (lvl) {
      lvl[(size_t)r * LANES + l] = iter;
    }
    if (par) par[(size_t)r * LANES + l] = r;
    if (dist) dist[(size_t)r * LANES + l] = 0.0f;
    if (lane_sum) {
      lane_sum[l] = 1;
      lane_sum[LANES + l] = out_deg[r];
    }
  }
  mc->edges = edges;
}

// Levels of the lanes slot[l] >= 0 from the level lists, lane-major:
// levels[slot[l] * V + v] = entry iteration - start[l] (the arrays hold -1
// where a lane did not reach v).
__global__ void lanes_list_extract(const LevelEntry *__restrict__ list, size_t n, const int *__restrict__ slot,
                                   const uint32_t *__restrict__ start, uint32_t V, int32_t *levels) {
  __shared__ int s_slot[LANES];
  __shared__ uint32_t s_start[LANES];
  for (int i = threadIdx.x; i < LANES; i += blockDim.x) {
    s_slot[i] = slot[i];
    s_start[i] = start[i];
  }
  __syncthreads();
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const LevelEntry e = list[i];
    u64 m = ((u64)e.w << 32) | e.z;
    while (m) {
      const int l = __ffsll((long long)m) - 1;
      m &= m - 1;
      if (s_slot[l] >= 0) levels[(size_t)s_slot[l] * V + e.x] = (int32_t)(e.y - s_start[l]);
    }
  }
}

// The level rows from the level lists (lvl[v][l] = iteration).
__global__ void lanes_list_rows(const LevelEntry *__restrict__ list, size_t n, uint32_t *lvl) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const LevelEntry e = list[i];
    u64 m = ((u64)e.w << 32) | e.z;
    while (m) {
      const int l = __ffsll((long long)m) - 1;
      m &= m - 1;
      lvl[(size_t)e.x * LANES + l] = e.y;
    }
  }
}

// Checksum term of one result entry (matches gg_result_checksum).
__device__ __forceinline__ u64 result_term(uint32_t v, uint32_t x) {
  return gg_mix64((u64)v * 0x9E3779B97F4A7C15ull + x);
}

// ---------------------------------------------------------------- bucketed SSSP
static inline float host_float_of_bits(unsigned u) {
  float f;
  memcpy(&f, &u, sizeof f);
  return f;
}
// A lane whose distance at v was lowered waits in pend[v] until that distance
// is below the lane's threshold; then v expands for that lane (front[v]).
// Relaxing in rising distance buckets re-relaxes far less than plain rounds,
// and any relaxation order reaches the same fixpoint (every distance is the
// least rounded path sum), so results stay bit-identical.
__device__ __forceinline__ u64 shfl64(u64 x, int src) {
  const unsigned lo = __shfl_sync(GG_FULL, (unsigned)x, src), hi = __shfl_sync(GG_FULL, (unsigned)(x >> 32), src);
  return ((u64)hi << 32) | lo;
}

// Merges last step's lowered lanes (next) and admitted roots (front) into
// pend, moves the lanes below threshold to front and queues their vertices;
// per lane, the least distance still waiting (non-negative floats order like
// their bits).  A warp takes 32 vertices and serves the ones with pending
// lanes one at a time, thread t holding lanes t and t + 32.
__global__ void __launch_bounds__(256)
    msp_filter(uint32_t V, u64 *pend, u64 *next, u64 *front, const float *__restrict__ dist,
               const float *__restrict__ thr, uint32_t *q, const uint32_t *__restrict__ out_deg, MsCounters *mc,
               BucketCounters *bc) {
  __shared__ unsigned s_min[LANES];
  for (int i = threadIdx.x; i < LANES; i += blockDim.x) s_min[i] = 0xffffffffu;
  __syncthreads();
  const unsigned lane = lane_id();
  const float t0 = thr[lane], t1 = thr[lane + 32];
  unsigned mn0 = 0xffffffffu, mn1 = 0xffffffffu;
  u64 t_alive = 0, t_expand = 0, t_edges = 0;
  unsigned t_touched = 0;
  const size_t nwarps = (size_t)gridDim.x * (blockDim.x >> 5);
  for (size_t g = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; g * 32 < V; g += nwarps) {
    const size_t v = g * 32 + lane;
    u64 p = 0, nx = 0;
    if (v < V) {
      nx = next[v];
      p = pend[v] | nx | front[v];
    }
    unsigned bal = __ballot_sync(GG_FULL, p != 0);
    while (bal) {
      const int j = __ffs(bal) - 1;
      bal &= bal - 1;
      const size_t vj = g * 32 + j;
      const u64 pj = shfl64(p, j);
      const float *dv = dist + vj * LANES;
      bool e0 = false, e1 = false;
      if ((pj >> lane) & 1ull) {
        const float x = dv[lane];
        e0 = x < t0;
        if (!e0 && __float_as_uint(x) < mn0) mn0 = __float_as_uint(x);
      }
      if ((pj >> (lane + 32)) & 1ull) {
        const float x = dv[lane + 32];
        e1 = x < t1;
        if (!e1 && __float_as_uint(x) < mn1) mn1 = __float_as_uint(x);
      }
      const u64 E = (u64)__ballot_sync(GG_FULL, e0) | ((u64)__ballot_sync(GG_FULL, e1) << 32);
      if ((int)lane == j) {
        if (nx) next[vj] = 0;
        front[vj] = E;
        pend[vj] = pj & ~E;
        if (E) {
          q[atomicAdd(&mc->qlen, 1u)] = (uint32_t)vj;
          t_edges += out_deg[vj];
          t_touched += 1;
        }
      }
      t_alive |= pj;
      t_expand |= E;
    }
  }
  atomicMin(&s_min[lane], mn0);
  atomicMin(&s_min[lane + 32], mn1);
  t_expand = warp_or64(t_expand);
  if (lane == 0 && t_expand) atomicOr(&bc->expand, t_expand);
  __syncthreads();
  for (int i = threadIdx.x; i < LANES; i += blockDim.x)
    if (s_min[i] != 0xffffffffu) atomicMin(&bc->minp[i], s_min[i]);
  ms_flush(mc, t_alive, t_edges, t_touched);
}

__global__ void wmin_kernel(const float *__restrict__ w, size_t n, unsigned *out_bits_neg) {
  bool neg = false;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    neg |= w[i] < 0.0f;
  if (__any_sync(GG_FULL, neg) && lane_id() == 0) atomicOr(out_bits_neg, 1u);
}

// Per-lane digests of the lanes in mask: out[l] reached, out[64+l] checksum
// (SUM only), out[128+l] out-degree sum of reached vertices.  BFS: x = hop
// count; SSSP: x = the distance's float bits.  A warp walks vertices one at
// a time; thread t keeps traversal lanes t and t + 32, so the per-lane state
// of a vertex (64 consecutive entries) is read with two coalesced loads and
// the sums stay in registers until the end.
template <bool SUM>
__global__ void __launch_bounds__(256)
    lanes_digest(uint32_t V, u64 mask, const u64 *__restrict__ visit, const uint32_t *__restrict__ lvl,
                 const uint32_t *__restrict__ start, const float *__restrict__ dist,
                 const uint32_t *__restrict__ out_deg, u64 *out) {
  __shared__ u64 s_out[3 * LANES];
  for (int i = threadIdx.x; i < 3 * LANES; i += blockDim.x) s_out[i] = 0;
  __syncthreads();
  const unsigned t = lane_id();
  const bool m0 = (mask >> t) & 1ull, m1 = (mask >> (t + 32)) & 1ull;
  const uint32_t st0 = visit ? start[t] : 0u, st1 = visit ? start[t + 32] : 0u;
  u64 c0 = 0, c1 = 0, h0 = 0, h1 = 0, e0 = 0, e1 = 0;
  const size_t nwarps = (size_t)gridDim.x * (blockDim.x >> 5);
  for (size_t v = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; v < V; v += nwarps) {
    bool hit0, hit1;
    uint32_t x0 = 0, x1 = 0;
    if (visit) {
      const u64 vm = visit[v] & mask;
      if (!vm) continue;
      hit0 = (vm >> t) & 1ull;
      hit1 = (vm >> (t + 32)) & 1ull;
      if (SUM) {
        if (hit0) x0 = lvl[v * LANES + t] - st0;
        if (hit1) x1 = lvl[v * LANES + t + 32] - st1;
      }
    } else {
      const float d0 = dist[v * LANES + t], d1 = dist[v * LANES + t + 32];
      hit0 = m0 && d0 < 1e9f;
      hit1 = m1 && d1 < 1e9f;
      x0 = __float_as_uint(d0);
      x1 = __float_as_uint(d1);
      if (!__any_sync(GG_FULL, hit0 || hit1)) continue;
    }
    const uint32_t dg = out_deg[v];
    if (hit0) {
      c0 += 1;
      e0 += dg;
      if (SUM) h0 += result_term((uint32_t)v, x0);
    }
    if (hit1) {
      c1 += 1;
      e1 += dg;
      if (SUM) h1 += result_term((uint32_t)v, x1);
    }
  }
  if (m0) {
    if (c0) atomicAdd(&s_out[t], c0);
    if (h0) atomicAdd(&s_out[LANES + t], h0);
    if (e0) atomicAdd(&s_out[2 * LANES + t], e0);
  }
  if (m1) {
    if (c1) atomicAdd(&s_out[t + 32], c1);
    if (h1) atomicAdd(&s_out[LANES + t + 32], h1);
    if (e1) atomicAdd(&s_out[2 * LANES + t + 32], e1);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < 3 * LANES; i += blockDim.x)
    if (s_out[i]) atomicAdd(&out[i], s_out[i]);
}

// Lane-major results of lanes[0..n): levels[j*V + v] (hop count or -1),
// parents[j*V + v] (or V), dist_out[j*V + v], through a shared tile of 32
// vertices x n lanes.
__global__ void __launch_bounds__(256)
    lanes_extract(uint32_t V, const int *lanes, int n, const u64 *__restrict__ visit, const uint32_t *__restrict__ lvl,
                  const uint32_t *__restrict__ start, const uint32_t *__restrict__ par, const float *__restrict__ dist,
                  int32_t *levels, uint32_t *parents, float *dist_out) {
  __shared__ uint32_t s_a[32][LANES + 1];
  __shared__ uint32_t s_b[32][LANES + 1];
  __shared__ u64 s_vis[32];
  __shared__ int s_lane[LANES];
  if (threadIdx.x < (unsigned)n) s_lane[threadIdx.x] = lanes[threadIdx.x];
  __syncthreads();
  for (size_t v0 = (size_t)blockIdx.x * 32; v0 < V; v0 += (size_t)gridDim.x * 32) {
    for (int i = threadIdx.x; i < 32 * n; i += blockDim.x) {
      const int r = i / n, j = i % n;
      const size_t v = v0 + r;
      if (v >= V) continue;
      const int l = s_lane[j];
      if (levels) s_a[r][j] = lvl[v * LANES + l] - start[l];
      if (parents) s_b[r][j] = par[v * LANES + l];
      if (dist_out) s_a[r][j] = __float_as_uint(dist[v * LANES + l]);
    }
    if (threadIdx.x < 32) {
      const size_t v = v0 + threadIdx.x;
      s_vis[threadIdx.x] = (visit && v < V) ? visit[v] : 0ull;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 32 * n; i += blockDim.x) {
      const int j = i / 32, r = i % 32;
      const size_t v = v0 + r;
      if (v >= V) continue;
      if (dist_out) {
        dist_out[(size_t)j * V + v] = __uint_as_float(s_a[r][j]);
        continue;
      }
      const bool hit = (s_vis[r] >> s_lane[j]) & 1ull;
      if (levels) levels[(size_t)j * V + v] = hit ? (int32_t)s_a[r][j] : -1;
      if (parents) parents[(size_t)j * V + v] = hit ? s_b[r][j] : V;
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------- batched SSSP

// Relaxation of every out-edge (u, v, w) of the union frontier, one warp per
// edge: lane j handles SSSP lanes j and j + 32 of the edge (a coalesced 256 B
// row of dist[v]).  A lane whose distance at v was lowered gets v's next bit;
// the first setter of next[v] queues v.  Reads dist[u] as it is now (the
// fixpoint, hence every lane's result, does not depend on that order).
template <bool G>
__global__ void __launch_bounds__(PUSH_THREADS)
    msp_push(const uint32_t *__restrict__ q, const unsigned long long *__restrict__ P, uint32_t n,
             unsigned long long total, Dir d, const u64 *__restrict__ front, u64 *next, float *dist, uint32_t *q_out,
             MsCounters *mc, const MsState *st) {
  if (G) {
    q = st->qa;
    n = st->nq;
    total = st->ae;
    front = st->front;
    next = st->next;
    q_out = st->qb;
  }
  __shared__ unsigned long long s_P[PUSH_STAGE + 1];
  __shared__ unsigned long long s_base[PUSH_STAGE];
  __shared__ uint32_t s_src[PUSH_STAGE];
  __shared__ uint32_t s_lo, s_hi;
  const unsigned lane = lane_id(), w = threadIdx.x >> 5;
  const unsigned long long ntiles = (total + PUSH_TILE - 1) / PUSH_TILE;
  u64 t_alive = 0, t_edges = 0;
  for (unsigned long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const unsigned long long e0 = tile * PUSH_TILE;
    const unsigned long long e1 = e0 + PUSH_TILE < total ? e0 + PUSH_TILE : total;
    if (threadIdx.x == 0) {
      uint32_t lo = upper_bound_idx<unsigned long long>(P, 0, n + 1, e0) - 1;
      s_lo = lo;
      s_hi = upper_bound_idx<unsigned long long>(P, lo, n + 1, e1 - 1);
    }
    __syncthreads();
    const uint32_t lo = s_lo, hi = s_hi, cnt = hi - lo;
    const bool staged = cnt <= (uint32_t)PUSH_STAGE;
    if (staged) {
      for (uint32_t i = threadIdx.x; i < cnt; i += PUSH_THREADS) {
        const unsigned long long pi = P[lo + i];
        const uint32_t src = q[lo + i];
        s_P[i] = pi;
        s_src[i] = src;
        s_base[i] = d.off[src] - pi;
      }
    }
    __syncthreads();
    // each warp takes every eighth edge of the tile; its lanes cover the 64 SSSP lanes
    for (unsigned long long e = e0 + w; e < e1; e += PUSH_THREADS / 32) {
      uint32_t u;
      unsigned long long k;
      if (staged) {
        const uint32_t i = upper_bound_idx<unsigned long long>(s_P, 0, cnt, e) - 1;
        u = s_src[i];
        k = s_base[i] + e;
      } else {
        const uint32_t i = upper_bound_idx<unsigned long long>(P, lo, hi, e) - 1;
        u = q[i];
        k = d.off[u] + (e - P[i]);
      }
      const uint32_t v = nbr_at(d, k, GG_SITE);
      const float wt = d.w[k];
      const u64 fm = front[u];
      bool low0 = false, low1 = false;
      if ((fm >> lane) & 1ull) {
        const float nd = __fadd_rn(dist[(size_t)u * LANES + lane], wt);
        float *p = dist + (size_t)v * LANES + lane;
        if (nd < *(volatile float *)p) low0 = atomic_min_float_b(p, nd);
      }
      if ((fm >> (lane + 32)) & 1ull) {
        const float nd = __fadd_rn(dist[(size_t)u * LANES + lane + 32], wt);
        float *p = dist + (size_t)v * LANES + lane + 32;
        if (nd < *(volatile float *)p) low1 = atomic_min_float_b(p, nd);
      }
      const u64 low = (u64)__ballot_sync(GG_FULL, low0) | ((u64)__ballot_sync(GG_FULL, low1) << 32);
      if (low && lane == 0) {
        const u64 old = atomicOr(next + v, low);
        if (!old) {
          q_out[atomicAdd(&mc->qlen, 1u)] = v;
          t_edges += d.deg[v];
        }
        t_alive |= low;
      }
    }
    __syncthreads();
  }
  ms_flush(mc, t_alive, t_edges, 0);
}

// The same relaxation, one thread per edge, looping over the SSSP lanes in
// which the source is on the frontier: for steps with few lanes in flight,
// where a warp per edge would leave most of its threads idle.
template <bool G>
__global__ void __launch_bounds__(PUSH_THREADS, 8)
    msp_push_thread(const uint32_t *__restrict__ q, const unsigned long long *__restrict__ P, uint32_t n,
                    unsigned long long total, Dir d, const u64 *__restrict__ front, u64 *next, float *dist,
                    uint32_t *q_out, MsCounters *mc, const MsState *st) {
  if (G) {
    q = st->qa;
    n = st->nq;
    total = st->ae;
    front = st->front;
    next = st->next;
    q_out = st->qb;
  }
  __shared__ unsigned long long s_P[PUSH_STAGE + 1];
  __shared__ unsigned long long s_base[PUSH_STAGE];
  __shared__ uint32_t s_src[PUSH_STAGE];
  __shared__ uint32_t s_lo, s_hi;
  const unsigned long long ntiles = (total + PUSH_TILE - 1) / PUSH_TILE;
  u64 t_alive = 0, t_edges = 0;
  for (unsigned long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const unsigned long long e0 = tile * PUSH_TILE;
    const unsigned long long e1 = e0 + PUSH_TILE < total ? e0 + PUSH_TILE : total;
    if (threadIdx.x == 0) {
      uint32_t lo = upper_bound_idx<unsigned long long>(P, 0, n + 1, e0) - 1;
      s_lo = lo;
      s_hi = upper_bound_idx<unsigned long long>(P, lo, n + 1, e1 - 1);
    }
    __syncthreads();
    const uint32_t lo = s_lo, hi = s_hi, cnt = hi - lo;
    const bool staged = cnt <= (uint32_t)PUSH_STAGE;
    if (staged) {
      for (uint32_t i = threadIdx.x; i < cnt; i += PUSH_THREADS) {
        const unsigned long long pi = P[lo + i];
        const uint32_t src = q[lo + i];
        s_P[i] = pi;
        s_src[i] = src;
        s_base[i] = d.off[src] - pi;
      }
    }
    __syncthreads();
    for (unsigned long long e = e0 + threadIdx.x; e < e1; e += PUSH_THREADS) {
      uint32_t u;
      unsigned long long k;
      if (staged) {
        const uint32_t i = upper_bound_idx<unsigned long long>(s_P, 0, cnt, e) - 1;
        u = s_src[i];
        k = s_base[i] + e;
      } else {
        const uint32_t i = upper_bound_idx<unsigned long long>(P, lo, hi, e) - 1;
        u = q[i];
        k = d.off[u] + (e - P[i]);
      }
      const uint32_t v = nbr_at(d, k, GG_SITE);
      const float wt = d.w[k];
      u64 fm = front[u], low = 0;
      while (fm) {
        const int l = __ffsll((long long)fm) - 1;
        fm &= fm - 1;
        const float nd = __fadd_rn(dist[(size_t)u * LANES + l], wt);
        float *p = dist + (size_t)v * LANES + l;
        if (nd < *(volatile float *)p && atomic_min_float_b(p, nd)) low |= 1ull << l;
      }
      if (low) {
        const u64 old = atomicOr(next + v, low);
        if (!old) {
          q_out[atomicAdd(&mc->qlen, 1u)] = v;
          t_edges += d.deg[v];
        }
        t_alive |= low;
      }
    }
    __syncthreads();
  }
  ms_flush(mc, t_alive, t_edges, 0);
}

}  // namespace gg

// ---------------------------------------------------------------- LanePool
namespace gg {

size_t LanePool::bytes_needed(const gg_graph *g, Kind kind, bool parents) {
  const size_t V = g->V;
  size_t b = 3 * V * sizeof(u64) + 2 * (V + 1) * sizeof(uint32_t);            // masks, queues
  b += (V + 2) * sizeof(u64) + scan_scratch_elems(V + 1) * sizeof(u64);       // degree prefix + scan
  b += sizeof(MsState);                                                        // device-driven steps
  b += (bitmap_words32(g->V) + V + 1) * sizeof(uint32_t) + scan_scratch_elems(V) * sizeof(uint32_t);
  if (kind == BFS) b += V * LANES * sizeof(uint32_t) * (parents ? 2 : 1);
  else b += V * LANES * sizeof(float) + V * sizeof(u64);
  return b + (1 << 20);
}

int LanePool::open() {
  if (open_) return GG_OK;
  GG_CUDA(cudaSetDevice(g_->device));
  const size_t V = g_->V;
  auto fail = [&](cudaError_t e) {
    close();
    return cuda_status(e, "lane pool buffers");
  };
  cudaError_t e = cudaStreamCreateWithFlags(&s_, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc(&front_, V * sizeof(u64));
  if (e == cudaSuccess) e = cudaMalloc(&next_, V * sizeof(u64));
  if (e == cudaSuccess) e = cudaMalloc(&q_[0], (V + 1) * sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMalloc(&q_[1], (V + 1) * sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMalloc(&prefix_, (V + 2) * sizeof(u64));
  if (e == cudaSuccess) e = cudaMalloc(&scan64_, scan_scratch_elems(V + 1) * sizeof(u64));
  if (e == cudaSuccess) e = cudaMalloc(&qpos_, (V + 1) * sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMalloc(&scan32_, scan_scratch_elems(V) * sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMalloc(&roots_dev_, LANES * sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMalloc(&start_dev_, LANES * sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMalloc(&lanes_dev_, LANES * sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&mc_, 512);
  if (e == cudaSuccess) e = cudaMallocHost(&mc_host_, 512);
  if (e == cudaSuccess) e = cudaMalloc(&out_dev_, 3 * LANES * sizeof(u64));
  if (e == cudaSuccess) e = cudaMallocHost(&out_host_, 3 * LANES * sizeof(u64));
  if (e == cudaSuccess) e = cudaMalloc(&st_, sizeof(MsState));
  if (e == cudaSuccess) e = cudaMallocHost(&st_host_, sizeof(MsState));
  if (kind_ == BFS) {
    if (e == cudaSuccess && !parents_) e = cudaMalloc(&lane_sum_, 2 * LANES * sizeof(u64));
    if (e == cudaSuccess) e = cudaMalloc(&visit_, V * sizeof(u64));
    if (e == cudaSuccess) e = cudaMalloc(&lvl_, V * LANES * sizeof(uint32_t));
    if (e == cudaSuccess && parents_) e = cudaMalloc(&par_, V * LANES * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemsetAsync(visit_, 0, V * sizeof(u64), s_);
  } else {
    if (e == cudaSuccess) e = cudaMalloc(&dist_, V * LANES * sizeof(float));
    if (e == cudaSuccess) {
      fill_kernel<float><<<grid_for(V * LANES, 256, g_->num_sms, 16), 256, 0, s_>>>(dist_, V * LANES, 1e9f);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMalloc(&pend_, V * sizeof(u64));
    if (e == cudaSuccess) e = cudaMemsetAsync(pend_, 0, V * sizeof(u64), s_);
    if (e == cudaSuccess) e = cudaMalloc(&thr_dev_, LANES * sizeof(float));
    if (e == cudaSuccess && !g_->wmin_known && g_->out.w && g_->nadj) {
      unsigned *neg = nullptr;
      e = cudaMalloc(&neg, sizeof(unsigned));
      if (e == cudaSuccess) e = cudaMemsetAsync(neg, 0, sizeof(unsigned), s_);
      if (e == cudaSuccess) {
        wmin_kernel<<<grid_for(g_->nadj, 256, g_->num_sms, 8), 256, 0, s_>>>(g_->out.w, g_->nadj, neg);
        e = cudaGetLastError();
      }
      unsigned h = 0;
      if (e == cudaSuccess) e = cudaMemcpyAsync(&h, neg, sizeof(unsigned), cudaMemcpyDeviceToHost, s_);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s_);
      if (neg) cudaFree(neg);
      if (e == cudaSuccess) {
        g_->wmin = h ? -1.0f : 0.0f;
        g_->wmin_known = 1;
      }
    }
  }
  if (e == cudaSuccess) e = cudaMemsetAsync(front_, 0, V * sizeof(u64), s_);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s_);
  if (e != cudaSuccess) return fail(e);
  used_ = active_ = 0;
  ae_ = 0;
  nq_ = 0;
  qvalid_ = true;
  next_clear_ = false;
  cur_ = 0;
  iter_ = 0;
  open_ = true;
  return GG_OK;
}

void LanePool::close() {
  if (s_) cudaStreamSynchronize(s_);
  destroy_step_graph();
  void *bufs[] = {visit_, front_, next_, lvl_, par_, dist_, q_[0], q_[1], prefix_, scan64_, qpos_, scan32_,
                  roots_dev_, start_dev_, lanes_dev_, mc_, out_dev_, pend_, thr_dev_, lane_sum_, st_};
  for (void *p : bufs)
    if (p) cudaFree(p);
  if (mc_host_) cudaFreeHost(mc_host_);
  if (out_host_) cudaFreeHost(out_host_);
  if (st_host_) cudaFreeHost(st_host_);
  if (list_) cudaFree(list_);
  list_ = nullptr;
  list_n_ = list_cap_ = 0;
  list_mode_ = false;
  if (s_) cudaStreamDestroy(s_);
  visit_ = front_ = next_ = nullptr;
  lvl_ = par_ = nullptr;
  dist_ = nullptr;
  pend_ = nullptr;
  thr_dev_ = nullptr;
  lane_sum_ = nullptr;
  q_[0] = q_[1] = nullptr;
  prefix_ = scan64_ = nullptr;
  qpos_ = scan32_ = roots_dev_ = start_dev_ = nullptr;
  lanes_dev_ = nullptr;
  mc_ = mc_host_ = nullptr;
  out_dev_ = out_host_ = nullptr;
  st_ = st_host_ = nullptr;
  s_ = nullptr;
  open_ = false;
}

int LanePool::read_counters(LaneCounters *h) {
  GG_CUDA(cudaMemcpyAsync(mc_host_, mc_, sizeof(LaneCounters), cudaMemcpyDeviceToHost, s_));
  GG_CUDA(cudaStreamSynchronize(s_));
  *h = *mc_host_;
  return GG_OK;
}

int LanePool::admit(const uint32_t *roots, const int *lanes, int n) {
  if (n <= 0) return GG_OK;
  u64 mask = 0;
  for (int i = 0; i < n; i++) {
    if (lanes[i] < 0 || lanes[i] >= LANES || ((used_ >> lanes[i]) & 1ull) || roots[i] >= g_->V) {
      set_error("bad lane or root in admit");
      return GG_ERR_INVALID;
    }
    mask |= 1ull << lanes[i];
    start_[lanes[i]] = iter_;
  }
  if (kind_ == SSSP) {
    // bucketing needs non-negative weights; the width is read per admission
    if (used_ == 0) {
      delta_ = g_->sssp_delta;
      bucket_ = delta_ > 0.0f && g_->wmin_known && g_->wmin >= 0.0f;
    }
    for (int i = 0; i < n; i++) thr_[lanes[i]] = delta_;
  }
  if (used_ == 0) {
    list_mode_ = want_lists_ && kind_ == BFS && !parents_;
    list_n_ = 0;
  }
  if (list_mode_) GG_TRY(list_room((size_t)n));
  const uint32_t V = g_->V;
  GG_CUDA(cudaMemcpyAsync(roots_dev_, roots, sizeof(uint32_t) * n, cudaMemcpyHostToDevice, s_));
  GG_CUDA(cudaMemcpyAsync(lanes_dev_, lanes, sizeof(int) * n, cudaMemcpyHostToDevice, s_));
  GG_CUDA(cudaMemcpyAsync(start_dev_, start_, sizeof(uint32_t) * LANES, cudaMemcpyHostToDevice, s_));
  if (kind_ == BFS)
    lanes_reset_visit<<<grid_for(V, 256, g_->num_sms, 8), 256, 0, s_>>>(visit_, V, mask);
  else
    lanes_reset_dist<<<grid_for((size_t)V * LANES, 256, g_->num_sms, 16), 256, 0, s_>>>(dist_, V, mask);
  GG_CUDA(cudaMemsetAsync(mc_, 0, sizeof(LaneCounters), s_));
  lanes_admit<<<1, 32, 0, s_>>>(roots_dev_, lanes_dev_, n, front_, visit_, lvl_, par_, dist_, iter_, g_->out.deg, mc_,
                                lane_sum_, list_mode_ ? list_ + list_n_ : nullptr);
  launches += 2;
  GG_CUDA(cudaGetLastError());
  LaneCounters h;
  GG_TRY(read_counters(&h));
  if (list_mode_) list_n_ += (size_t)n;
  ae_ += h.edges;
  qvalid_ = false;
  used_ |= mask;
  active_ |= mask;
  return GG_OK;
}

template <bool G>
int LanePool::queue_kernels(int *n) {
  const uint32_t V = g_->V;
  if (G)
    GG_CUDA((exclusive_scan<uint32_t, NonzeroFront>(NonzeroFront{st_}, V, qpos_, scan32_, s_, n)));
  else
    GG_CUDA((exclusive_scan<uint32_t, NonzeroMask>(NonzeroMask{front_}, V, qpos_, scan32_, s_, n)));
  ms_compact<G><<<grid_for(V, 256, g_->num_sms), 256, 0, s_>>>(front_, V, qpos_, q_[cur_], st_);
  *n += 1;
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

int LanePool::build_queue() {
  const uint32_t V = g_->V;
  GG_TRY(queue_kernels<false>(&launches));
  GG_CUDA(cudaMemcpyAsync(mc_host_, qpos_ + V, sizeof(uint32_t), cudaMemcpyDeviceToHost, s_));
  GG_CUDA(cudaStreamSynchronize(s_));
  nq_ = *(uint32_t *)mc_host_;
  qvalid_ = true;
  return GG_OK;
}

static unsigned push_grid_for(const gg_graph *g, unsigned long long total) {
  unsigned long long tiles = (total + PUSH_TILE - 1) / PUSH_TILE;
  unsigned long long cap = (unsigned long long)g->num_sms * 8;
  return (unsigned)(tiles < 1 ? 1 : (tiles > cap ? cap : tiles));
}

// Dense BFS step: the light lists, then the long lists' chunks and their finish.
template <bool G>
int LanePool::pull_kernels(int *n) {
  const uint32_t V = g_->V;
  u64 *ls = par_ ? nullptr : lane_sum_;
  // level lists: entries of this step from list_ + list_n_ (host-driven only)
  const bool lists = !G && list_mode_;
  LevelEntry *list = lists ? list_ + list_n_ : nullptr;
  const unsigned grid = grid_for(((size_t)V + 31) / 32 * 32, 256, g_->num_sms, 8);
  if (lists)
    ms_pull_light<G, true><<<grid, 256, 0, s_>>>(g_->in, V, active_, front_, visit_, next_, lvl_, par_, iter_,
                                                g_->out.deg, mc_, ls, st_, list);
  else
    ms_pull_light<G, false><<<grid, 256, 0, s_>>>(g_->in, V, active_, front_, visit_, next_, lvl_, par_, iter_,
                                                 g_->out.deg, mc_, ls, st_, nullptr);
  *n += 1;
  if (g_->in.nbig) {
    ms_pull_chunks<G><<<grid_for((size_t)g_->in.nbigchunks * 32, 256, g_->num_sms, 8), 256, 0, s_>>>(
        g_->in, active_, front_, visit_, next_, lvl_, par_, iter_, st_);
    const unsigned fg = grid_for(g_->in.nbig, 256, g_->num_sms);
    if (lists)
      ms_big_finish<G, true><<<fg, 256, 0, s_>>>(g_->in, visit_, next_, g_->out.deg, mc_, lvl_, iter_, ls, st_, list);
    else
      ms_big_finish<G, false><<<fg, 256, 0, s_>>>(g_->in, visit_, next_, g_->out.deg, mc_, lvl_, iter_, ls, st_,
                                                  nullptr);
    *n += 2;
  }
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

// Push over the frontier queue: the prefix of its out-degrees, then the
// edge-balanced push (BFS), or the warp- or thread-per-edge relaxation (SSSP).
template <bool G>
int LanePool::push_kernels(bool per_thread, int *n) {
  if (G)
    GG_CUDA((exclusive_scan_dn<unsigned long long, QueueDegreeSt>(QueueDegreeSt{st_, g_->out.deg}, &st_->nq, g_->V,
                                                                  prefix_, scan64_, s_, n)));
  else
    GG_CUDA((exclusive_scan<unsigned long long, QueueDegreeIn>(QueueDegreeIn{q_[cur_], g_->out.deg}, nq_, prefix_,
                                                               scan64_, s_, n)));
  const unsigned grid = G ? (unsigned)g_->num_sms * 8 : push_grid_for(g_, ae_);
  if (!G && tr_) GG_TRY(tr_->kbegin());
  if (kind_ == BFS)
    ms_push<G><<<grid, PUSH_THREADS, 0, s_>>>(q_[cur_], prefix_, nq_, ae_, g_->out, front_, visit_, next_, lvl_,
                                              par_, iter_, q_[cur_ ^ 1], mc_, st_);
  else
    (per_thread ? msp_push_thread<G> : msp_push<G>)<<<grid, PUSH_THREADS, 0, s_>>>(
        q_[cur_], prefix_, nq_, ae_, g_->out, front_, next_, dist_, q_[cur_ ^ 1], mc_, st_);
  if (!G && tr_) GG_TRY(tr_->kend());
  *n += 1;
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

// After a push: (BFS) visit |= next over the reached queue and its levels;
// the frontier's masks cleared through its queue.
template <bool G>
int LanePool::push_tail(int *n) {
  // the reached queue's length stays on the device
  const unsigned *qlen_dev = &mc_->qlen;
  const bool lists = !G && list_mode_;
  if (kind_ == BFS) {
    ms_push_finish<G><<<g_->num_sms * 4, 256, 0, s_>>>(q_[cur_ ^ 1], qlen_dev, visit_, next_, g_->out.deg, mc_, st_,
                                                       lists ? list_ + list_n_ : nullptr, iter_);
    *n += 1;
  }
  const unsigned grid = G ? grid_for(g_->V, 256, g_->num_sms) : grid_for(nq_ ? nq_ : 1, 256, g_->num_sms);
  ms_clear_queue<G><<<grid, 256, 0, s_>>>(q_[cur_], nq_, front_, st_);
  *n += 1;
  if (kind_ == BFS && !par_) {
    ms_mark_levels_q<G><<<g_->num_sms * 4, 256, 0, s_>>>(q_[cur_ ^ 1], qlen_dev, next_, lists ? nullptr : lvl_,
                                                        iter_, g_->out.deg,
                                                        lane_sum_, st_);
    *n += 1;
  }
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

int LanePool::bfs_step() {
  const uint32_t V = g_->V;
  // a step appends at most one level-list entry per vertex; a pull step
  // leaves fewer than 32 empty slots per slot range it takes (ranges hold
  // LIST_CHUNK) and fewer than LIST_CHUNK at the end of each warp of its two
  // kernels (at most 64 warps per SM each)
  if (list_mode_) GG_TRY(list_room(2 * (size_t)V + (size_t)2 * g_->num_sms * 64 * LIST_CHUNK));
  const bool sparse = ae_ < g_->E / g_->batched_switch_div;
  if (tr_) tr_->add(sparse ? 0 : 1, ae_, 0);
  iter_ += 1;
  LaneCounters h;
  GG_CUDA(cudaMemsetAsync(mc_, 0, sizeof(LaneCounters), s_));
  if (sparse) {
    if (!qvalid_) GG_TRY(build_queue());
    if (!next_clear_) GG_CUDA(cudaMemsetAsync(next_, 0, sizeof(u64) * V, s_));
    if (ae_ > 0) GG_TRY(push_kernels<false>(false, &launches));
    GG_TRY(push_tail<false>(&launches));
    // one host wait per step
    GG_TRY(read_counters(&h));
    nq_ = h.qlen;
    qvalid_ = true;
    cur_ ^= 1;
    next_clear_ = true;
  } else {
    if (tr_) GG_TRY(tr_->kbegin());
    GG_TRY(pull_kernels<false>(&launches));
    if (tr_) GG_TRY(tr_->kend());
    GG_TRY(read_counters(&h));
    qvalid_ = false;
    next_clear_ = false;
  }
  if (tr_) tr_->set_activated(h.touched);
  // every vertex the step reached has one entry (pull: in the slots taken
  // from mc->lpos, some left empty; push: in the reached queue's order)
  if (list_mode_) list_n_ += sparse ? h.touched : h.lpos;
  active_ &= h.alive;
  ae_ = h.edges;
  u64 *t = front_;
  front_ = next_;
  next_ = t;
  return GG_OK;
}

// Room for `more` level-list entries: the list grows by doubling up to 16
// entries per vertex (the level rows' 256 bytes); past that the entries so
// far go into the level rows and the traversals continue on the rows.
int LanePool::list_room(size_t more) {
  if (list_n_ + more <= list_cap_) return GG_OK;
  const size_t V = g_->V;
  size_t want = list_cap_ ? 2 * list_cap_ : 4 * V + 64;
  while (want < list_n_ + more) want *= 2;
  if (want > 16 * V + 64) return lists_to_rows();
  LevelEntry *p = nullptr;
  cudaError_t e = cudaMalloc(&p, sizeof(LevelEntry) * want);
  if (e != cudaSuccess) {
    cudaGetLastError();  // out of memory: the rows take over
    return lists_to_rows();
  }
  if (list_n_) GG_CUDA(cudaMemcpyAsync(p, list_, sizeof(LevelEntry) * list_n_, cudaMemcpyDeviceToDevice, s_));
  GG_CUDA(cudaStreamSynchronize(s_));
  if (list_) cudaFree(list_);
  list_ = p;
  list_cap_ = want;
  return GG_OK;
}

// The level lists into the level rows; the running traversals go on with
// the rows (the per-lane sums are kept by the steps either way).
int LanePool::lists_to_rows() {
  if (!list_mode_) return GG_OK;
  if (list_n_) {
    lanes_list_rows<<<grid_for(list_n_, 256, g_->num_sms, 8), 256, 0, s_>>>(list_, list_n_, lvl_);
    launches += 1;
  }
  GG_CUDA(cudaGetLastError());
  list_mode_ = false;
  list_n_ = 0;
  return GG_OK;
}

int LanePool::sssp_step() {
  if (tr_) tr_->add(0, ae_, 0);
  iter_ += 1;
  if (!qvalid_) GG_TRY(build_queue());
  GG_CUDA(cudaMemsetAsync(mc_, 0, sizeof(LaneCounters), s_));
  if (!next_clear_) GG_CUDA(cudaMemsetAsync(next_, 0, sizeof(u64) * g_->V, s_));
  if (ae_ > 0 && nq_ > 0)
    GG_TRY(push_kernels<false>(__builtin_popcountll(active_) <= (int)g_->batched_thread_lanes, &launches));
  GG_TRY(push_tail<false>(&launches));
  LaneCounters h;
  GG_TRY(read_counters(&h));
  if (tr_) tr_->set_activated(h.qlen);
  nq_ = h.qlen;
  qvalid_ = true;
  next_clear_ = true;
  cur_ ^= 1;
  active_ &= h.alive;
  ae_ = h.edges;
  u64 *t = front_;
  front_ = next_;
  next_ = t;
  return GG_OK;
}

int LanePool::sssp_bucket_step() {
  const uint32_t V = g_->V;
  iter_ += 1;
  BucketCounters *bc_dev = reinterpret_cast<BucketCounters *>(reinterpret_cast<char *>(mc_) + BUCKET_OFFSET);
  const BucketCounters *bc_host =
      reinterpret_cast<const BucketCounters *>(reinterpret_cast<const char *>(mc_host_) + BUCKET_OFFSET);
  LaneCounters h;
  u64 expand = 0;
  // at most two rounds: a round that expands nothing raises every waiting
  // lane's threshold past its least waiting distance
  for (int round = 0; round < 2; round++) {
    GG_CUDA(cudaMemcpyAsync(thr_dev_, thr_, sizeof(float) * LANES, cudaMemcpyHostToDevice, s_));
    GG_CUDA(cudaMemsetAsync(mc_, 0, BUCKET_OFFSET + sizeof(u64), s_));
    GG_CUDA(cudaMemsetAsync(bc_dev->minp, 0xff, sizeof(bc_dev->minp), s_));
    msp_filter<<<grid_for(((size_t)V + 31) / 32 * 32, 256, g_->num_sms, 8), 256, 0, s_>>>(
        V, pend_, next_, front_, dist_, thr_dev_, q_[cur_], g_->out.deg, mc_, bc_dev);
    launches += 1;
    GG_CUDA(cudaGetLastError());
    GG_CUDA(cudaMemcpyAsync(mc_host_, mc_, BUCKET_OFFSET + sizeof(BucketCounters), cudaMemcpyDeviceToHost, s_));
    GG_CUDA(cudaStreamSynchronize(s_));
    h = *mc_host_;
    expand = bc_host->expand;
    const u64 waiting = h.alive & ~expand;
    for (int l = 0; l < LANES; l++) {
      if (!((waiting >> l) & 1ull) || bc_host->minp[l] == 0xffffffffu) continue;
      const float m = host_float_of_bits(bc_host->minp[l]);
      float t = (floorf(m / delta_) + 1.0f) * delta_;
      if (!(t > m)) t = nextafterf(m, 3.0e38f);
      thr_[l] = t;
    }
    if (expand || !h.alive) break;
  }
  nq_ = h.qlen;
  ae_ = h.edges;
  if (tr_) tr_->add(0, ae_, h.touched);
  active_ &= h.alive;
  if (expand && nq_ && ae_) {
    GG_CUDA((exclusive_scan<unsigned long long, QueueDegreeIn>(QueueDegreeIn{q_[cur_], g_->out.deg}, nq_, prefix_,
                                                               scan64_, s_, &launches)));
    if (tr_) GG_TRY(tr_->kbegin());
    (__builtin_popcountll(active_) <= (int)g_->batched_thread_lanes ? msp_push_thread<false> : msp_push<false>)<<<
        push_grid_for(g_, ae_), PUSH_THREADS, 0, s_>>>(q_[cur_], prefix_, nq_, ae_, g_->out, front_, next_,
                                                              dist_, q_[cur_ ^ 1], mc_, nullptr);
    if (tr_) GG_TRY(tr_->kend());
    launches += 1;
  }
  if (nq_) {
    ms_clear_queue<false><<<grid_for(nq_, 256, g_->num_sms), 256, 0, s_>>>(q_[cur_], nq_, front_, nullptr);
    launches += 1;
  }
  GG_CUDA(cudaGetLastError());
  qvalid_ = false;
  return GG_OK;
}

int LanePool::step() {
  if (!active_) return GG_OK;
  calls_ += 1;
  if (kind_ == BFS) return bfs_step();
  return bucket_ ? sssp_bucket_step() : sssp_step();
}

// ---------------------------------------------------------------- device-driven steps
constexpr uint32_t MS_NO_STEP = 0xffffffffu;

// First kernel of a step of the loop: the step's mode by the rule of
// bfs_step / sssp_step, from the state the last step left; the step graph's
// branches switched on or off; the step's counters cleared.
__global__ void ms_decide(MsState *st, MsCounters *mc, unsigned long long dense_edges, int bfs, uint32_t thread_lanes,
                          cudaGraphConditionalHandle h_dense, cudaGraphConditionalHandle h_sparse,
                          cudaGraphConditionalHandle h_build, cudaGraphConditionalHandle h_clear,
                          cudaGraphConditionalHandle h_push, cudaGraphConditionalHandle h_push_t) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const bool go = st->active != 0 && st->steps < st->cap;
  const bool dense = go && bfs && st->ae >= dense_edges;
  const bool sparse = go && !dense;
  const bool build = sparse && !st->qvalid;
  const bool clear = sparse && !st->next_clear;
  const bool push = sparse && st->ae > 0;
  const bool per_thread = push && !bfs && __popcll(st->active) <= (int)thread_lanes;
  if (bfs) cudaGraphSetConditional(h_dense, dense);
  cudaGraphSetConditional(h_sparse, sparse);
  cudaGraphSetConditional(h_build, build);
  cudaGraphSetConditional(h_clear, clear);
  cudaGraphSetConditional(h_push, push && !per_thread);
  if (!bfs) cudaGraphSetConditional(h_push_t, per_thread);
  if (!go) {
    st->mode = MS_NO_STEP;
    return;
  }
  st->mode = (dense ? MS_ROW_DENSE : 0u) | (build ? MS_ROW_BUILD : 0u) | (clear ? MS_ROW_CLEAR : 0u) |
             (push && !per_thread ? MS_ROW_PUSH : 0u) | (per_thread ? MS_ROW_PUSH_THREAD : 0u);
  st->iter += 1;
  mc->alive = 0;
  mc->edges = 0;
  mc->touched = 0;
  mc->qlen = 0;
}

// Last kernel of a step: its row; the lanes left, the frontier's out-edges
// and queue; front / next and the two queues swapped; the loop goes on while
// a lane is active and rows are left.
__global__ void ms_advance(MsState *st, const MsCounters *mc, int bfs, cudaGraphConditionalHandle h_loop) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const uint32_t mode = st->mode;
  if (mode == MS_NO_STEP) {
    cudaGraphSetConditional(h_loop, 0);
    return;
  }
  const uint32_t r = st->steps;
  st->row_mode[r] = mode;
  st->row_ae[r] = st->ae;
  st->row_reached[r] = bfs ? mc->touched : mc->qlen;
  st->steps = r + 1;
  if (mode & MS_ROW_DENSE) {
    st->qvalid = 0;
    st->next_clear = 0;
  } else {
    // the reached queue is the next frontier's; the push epilogue cleared
    // the old frontier's masks through its queue
    st->nq = mc->qlen;
    st->qvalid = 1;
    st->next_clear = 1;
    uint32_t *t = st->qa;
    st->qa = st->qb;
    st->qb = t;
  }
  st->active &= mc->alive;
  st->ae = mc->edges;
  u64 *t = st->front;
  st->front = st->next;
  st->next = t;
  cudaGraphSetConditional(h_loop, st->active != 0 && st->steps < st->cap);
}

static bool same_dir(const Dir &a, const Dir &b) {
  return a.light == b.light && a.chunk == b.chunk && a.vec == b.vec && a.off == b.off && a.nbr == b.nbr &&
         a.w == b.w && a.deg == b.deg && a.nz == b.nz && a.med == b.med && a.nmed == b.nmed && a.heavy == b.heavy &&
         a.nheavy == b.nheavy && a.heavy_chunk == b.heavy_chunk && a.chunk_owner == b.chunk_owner &&
         a.nchunks == b.nchunks && a.big == b.big && a.nbig == b.nbig && a.big_chunk == b.big_chunk &&
         a.big_owner == b.big_owner && a.nbigchunks == b.nbigchunks && a.nv == b.nv && a.ne == b.ne &&
         a.err == b.err;
}

bool LanePool::step_graph_current() const {
  return step_exec_ && same_dir(key_in_, g_->in) && same_dir(key_out_, g_->out) &&
         key_div_ == g_->batched_switch_div && key_tl_ == g_->batched_thread_lanes;
}

void LanePool::destroy_step_graph() {
  if (step_exec_) cudaGraphExecDestroy(step_exec_);
  if (step_graph_) cudaGraphDestroy(step_graph_);
  step_exec_ = nullptr;
  step_graph_ = nullptr;
}

// The step graph: a loop node whose body is
//   decide -> [pull] | [push: (queue build) (clear next) -> (push | thread push) -> epilogue] -> advance
// with every bracket a conditional node that decide switches.  Built once per
// pool and adjacency (the bins are launch arguments), replayed for every batch.
int LanePool::build_step_graph() {
  destroy_step_graph();
  GG_CUDA(cudaStreamSynchronize(s_));
  const bool bfs = kind_ == BFS;
  cudaGraph_t top = nullptr;
  GG_CUDA(cudaGraphCreate(&top, 0));
  step_graph_ = top;
  auto handle = [&](cudaGraphConditionalHandle *h, unsigned dflt, unsigned flags) -> int {
    GG_CUDA(cudaGraphConditionalHandleCreate(h, top, dflt, flags));
    return GG_OK;
  };
  auto cond = [&](cudaGraph_t g, const std::vector<cudaGraphNode_t> &deps, cudaGraphConditionalHandle h,
                  cudaGraphConditionalNodeType type, cudaGraphNode_t *node, cudaGraph_t *body) -> int {
    cudaGraphNodeParams np = {};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = h;
    np.conditional.type = type;
    np.conditional.size = 1;
    GG_CUDA(cudaGraphAddNode(node, g, deps.empty() ? nullptr : deps.data(), nullptr, deps.size(), &np));
    *body = np.conditional.phGraph_out[0];
    return GG_OK;
  };
  // kernels launched by fn, captured into g after deps; sinks: the captured
  // nodes nothing else depends on
  auto capture = [&](cudaGraph_t g, const std::vector<cudaGraphNode_t> &deps, auto &&fn,
                     std::vector<cudaGraphNode_t> *sinks) -> int {
    GG_CUDA(cudaStreamBeginCaptureToGraph(s_, g, deps.empty() ? nullptr : deps.data(), nullptr, deps.size(),
                                          cudaStreamCaptureModeThreadLocal));
    const int status = fn();
    cudaStreamCaptureStatus cs;
    const cudaGraphNode_t *d = nullptr;
    size_t nd = 0;
    const cudaError_t e = cudaStreamGetCaptureInfo(s_, &cs, nullptr, nullptr, &d, nullptr, &nd);
    if (e == cudaSuccess && sinks) sinks->assign(d, d + nd);
    cudaGraph_t captured = nullptr;
    const cudaError_t e2 = cudaStreamEndCapture(s_, &captured);
    if (status != GG_OK) return status;
    GG_CUDA(e);
    GG_CUDA(e2);
    return GG_OK;
  };
  cudaGraphConditionalHandle h_loop, h_dense = 0, h_sparse, h_build, h_clear, h_push, h_push_t = 0;
  GG_TRY(handle(&h_loop, 1, cudaGraphCondAssignDefault));
  if (bfs) GG_TRY(handle(&h_dense, 0, 0));
  GG_TRY(handle(&h_sparse, 0, 0));
  GG_TRY(handle(&h_build, 0, 0));
  GG_TRY(handle(&h_clear, 0, 0));
  GG_TRY(handle(&h_push, 0, 0));
  if (!bfs) GG_TRY(handle(&h_push_t, 0, 0));
  n_ctl_ = 2;
  n_dense_ = n_build_ = n_clear_ = n_push_ = n_push_t_ = n_tail_ = 0;

  cudaGraphNode_t loop;
  cudaGraph_t body;
  GG_TRY(cond(top, {}, h_loop, cudaGraphCondTypeWhile, &loop, &body));
  std::vector<cudaGraphNode_t> decided, branches;
  const unsigned long long dense_edges = g_->E / g_->batched_switch_div;
  GG_TRY(capture(body, {}, [&]() -> int {
    ms_decide<<<1, 32, 0, s_>>>(st_, mc_, dense_edges, bfs ? 1 : 0, g_->batched_thread_lanes, h_dense, h_sparse,
                                h_build, h_clear, h_push, h_push_t);
    GG_CUDA(cudaGetLastError());
    return GG_OK;
  }, &decided));
  cudaGraphNode_t node;
  cudaGraph_t sub;
  if (bfs) {
    GG_TRY(cond(body, decided, h_dense, cudaGraphCondTypeIf, &node, &sub));
    GG_TRY(capture(sub, {}, [&]() { return pull_kernels<true>(&n_dense_); }, nullptr));
    branches.push_back(node);
  }
  cudaGraph_t sparse;
  GG_TRY(cond(body, decided, h_sparse, cudaGraphCondTypeIf, &node, &sparse));
  branches.push_back(node);
  std::vector<cudaGraphNode_t> ready, pushed;
  GG_TRY(cond(sparse, {}, h_build, cudaGraphCondTypeIf, &node, &sub));
  GG_TRY(capture(sub, {}, [&]() { return queue_kernels<true>(&n_build_); }, nullptr));
  ready.push_back(node);
  GG_TRY(cond(sparse, {}, h_clear, cudaGraphCondTypeIf, &node, &sub));
  GG_TRY(capture(sub, {}, [&]() -> int {
    ms_clear_next<<<grid_for(g_->V, 256, g_->num_sms), 256, 0, s_>>>(st_, g_->V);
    n_clear_ += 1;
    GG_CUDA(cudaGetLastError());
    return GG_OK;
  }, nullptr));
  ready.push_back(node);
  GG_TRY(cond(sparse, ready, h_push, cudaGraphCondTypeIf, &node, &sub));
  GG_TRY(capture(sub, {}, [&]() { return push_kernels<true>(false, &n_push_); }, nullptr));
  pushed.push_back(node);
  if (!bfs) {
    GG_TRY(cond(sparse, ready, h_push_t, cudaGraphCondTypeIf, &node, &sub));
    GG_TRY(capture(sub, {}, [&]() { return push_kernels<true>(true, &n_push_t_); }, nullptr));
    pushed.push_back(node);
  }
  GG_TRY(capture(sparse, pushed, [&]() { return push_tail<true>(&n_tail_); }, nullptr));
  GG_TRY(capture(body, branches, [&]() -> int {
    ms_advance<<<1, 32, 0, s_>>>(st_, mc_, bfs ? 1 : 0, h_loop);
    GG_CUDA(cudaGetLastError());
    return GG_OK;
  }, nullptr));
  GG_CUDA(cudaGraphInstantiate(&step_exec_, top, 0));
  key_in_ = g_->in;
  key_out_ = g_->out;
  key_div_ = g_->batched_switch_div;
  key_tl_ = g_->batched_thread_lanes;
  return GG_OK;
}

// Runs the step graph until no lane is active: the host state goes to the
// device before each launch and comes back after it, with one row per step
// for the trace.  A launch runs at most MS_ROWS steps.
int LanePool::run_device_steps() {
  if (!step_graph_current()) GG_TRY(build_step_graph());
  MsState *h = st_host_;
  while (active_) {
    h->front = front_;
    h->next = next_;
    h->qa = q_[cur_];
    h->qb = q_[cur_ ^ 1];
    h->active = active_;
    h->ae = ae_;
    h->nq = nq_;
    h->iter = iter_;
    h->qvalid = qvalid_ ? 1u : 0u;
    h->next_clear = next_clear_ ? 1u : 0u;
    h->steps = 0;
    h->cap = MS_ROWS;
    h->mode = 0;
    GG_CUDA(cudaMemcpyAsync(st_, h, MS_HEADER, cudaMemcpyHostToDevice, s_));
    GG_CUDA(cudaGraphLaunch(step_exec_, s_));
    GG_CUDA(cudaMemcpyAsync(h, st_, sizeof(MsState), cudaMemcpyDeviceToHost, s_));
    GG_CUDA(cudaStreamSynchronize(s_));
    const uint32_t steps = h->steps;
    if (steps == 0 || steps > MS_ROWS) {
      set_error("device-driven batch ran %u steps", steps);
      return GG_ERR_CUDA;
    }
    for (uint32_t r = 0; r < steps; r++) {
      const uint32_t m = h->row_mode[r];
      if (tr_) tr_->add((m & MS_ROW_DENSE) ? 1 : 0, h->row_ae[r], h->row_reached[r]);
      launches += n_ctl_;
      if (m & MS_ROW_DENSE) {
        launches += n_dense_;
        continue;
      }
      if (m & MS_ROW_BUILD) launches += n_build_;
      if (m & MS_ROW_CLEAR) launches += n_clear_;
      if (m & MS_ROW_PUSH) launches += n_push_;
      if (m & MS_ROW_PUSH_THREAD) launches += n_push_t_;
      launches += n_tail_;
    }
    calls_ += (int)steps;
    front_ = h->front;
    next_ = h->next;
    cur_ = h->qa == q_[0] ? 0 : 1;
    active_ = h->active;
    ae_ = h->ae;
    nq_ = h->nq;
    iter_ = h->iter;
    qvalid_ = h->qvalid != 0;
    next_clear_ = h->next_clear != 0;
  }
  return GG_OK;
}

int LanePool::run(bool per_step_timing) {
  const bool device = g_->batched_graph && !per_step_timing && !(kind_ == SSSP && bucket_) && !list_mode_;
  if (device && active_) return run_device_steps();
  while (active_) GG_TRY(step());
  return GG_OK;
}

int LanePool::digest(u64 mask, u64 *reached, u64 *checksum, u64 *edges) {
  mask &= used_;
  if (!mask) return GG_OK;
  const uint32_t V = g_->V;
  if (list_mode_ && checksum) GG_TRY(lists_to_rows());
  if (kind_ == BFS && lane_sum_ && !checksum) {
    // the level passes kept the sums: no scan of the graph
    GG_CUDA(cudaMemcpyAsync(out_host_, lane_sum_, 2 * LANES * sizeof(u64), cudaMemcpyDeviceToHost, s_));
    GG_CUDA(cudaStreamSynchronize(s_));
    for (int l = 0; l < LANES; l++) {
      if (!((mask >> l) & 1ull)) continue;
      if (reached) reached[l] = out_host_[l];
      if (edges) edges[l] = out_host_[LANES + l];
    }
    return GG_OK;
  }
  GG_CUDA(cudaMemcpyAsync(start_dev_, start_, sizeof(uint32_t) * LANES, cudaMemcpyHostToDevice, s_));
  GG_CUDA(cudaMemsetAsync(out_dev_, 0, 3 * LANES * sizeof(u64), s_));
  const unsigned grid = grid_for((size_t)V * 32, 256, g_->num_sms, 8);
  if (checksum)
    lanes_digest<true><<<grid, 256, 0, s_>>>(V, mask, kind_ == BFS ? visit_ : nullptr, lvl_, start_dev_, dist_,
                                             g_->out.deg, out_dev_);
  else
    lanes_digest<false><<<grid, 256, 0, s_>>>(V, mask, kind_ == BFS ? visit_ : nullptr, lvl_, start_dev_, dist_,
                                              g_->out.deg, out_dev_);
  launches += 1;
  GG_CUDA(cudaGetLastError());
  GG_CUDA(cudaMemcpyAsync(out_host_, out_dev_, 3 * LANES * sizeof(u64), cudaMemcpyDeviceToHost, s_));
  GG_CUDA(cudaStreamSynchronize(s_));
  for (int l = 0; l < LANES; l++) {
    if (!((mask >> l) & 1ull)) continue;
    if (reached) reached[l] = out_host_[l];
    if (checksum) checksum[l] = out_host_[LANES + l];
    if (edges) edges[l] = out_host_[2 * LANES + l];
  }
  return GG_OK;
}

int LanePool::extract(u64 mask, int32_t *levels, uint32_t *parents, float *dist) {
  mask &= used_;
  int lanes[LANES], n = 0;
  for (int l = 0; l < LANES; l++)
    if ((mask >> l) & 1ull) lanes[n++] = l;
  if (!n) return GG_OK;
  const uint32_t V = g_->V;
  if (list_mode_ && kind_ == BFS) {
    // lane-major levels from the level lists: slot[l] = output row of lane l
    int slot[LANES];
    for (int l = 0; l < LANES; l++) slot[l] = -1;
    for (int j = 0; j < n; j++) slot[lanes[j]] = j;
    GG_CUDA(cudaMemcpyAsync(lanes_dev_, slot, sizeof(int) * LANES, cudaMemcpyHostToDevice, s_));
    GG_CUDA(cudaMemcpyAsync(start_dev_, start_, sizeof(uint32_t) * LANES, cudaMemcpyHostToDevice, s_));
    if (levels) {
      GG_CUDA(cudaMemsetAsync(levels, 0xff, sizeof(int32_t) * (size_t)V * n, s_));
      if (list_n_)
        lanes_list_extract<<<grid_for(list_n_, 256, g_->num_sms, 8), 256, 0, s_>>>(list_, list_n_, lanes_dev_,
                                                                                   start_dev_, V, levels);
      launches += 1;
    }
    GG_CUDA(cudaGetLastError());
    GG_CUDA(cudaStreamSynchronize(s_));
    return GG_OK;
  }
  GG_CUDA(cudaMemcpyAsync(lanes_dev_, lanes, sizeof(int) * n, cudaMemcpyHostToDevice, s_));
  GG_CUDA(cudaMemcpyAsync(start_dev_, start_, sizeof(uint32_t) * LANES, cudaMemcpyHostToDevice, s_));
  lanes_extract<<<grid_for(((size_t)V + 31) / 32, 1, g_->num_sms, 16), 256, 0, s_>>>(
      V, lanes_dev_, n, visit_, lvl_, start_dev_, par_, dist_, kind_ == BFS ? levels : nullptr,
      kind_ == BFS ? parents : nullptr, kind_ == SSSP ? dist : nullptr);
  launches += 1;
  GG_CUDA(cudaGetLastError());
  GG_CUDA(cudaStreamSynchronize(s_));
  return GG_OK;
}

// The graph's own pools for the batched calls (created on first use).
static LanePool *graph_pool(gg_graph *g, LanePool::Kind kind, bool parents, int *status) {
  LanePool *&p = kind == LanePool::BFS ? g->pool_bfs : g->pool_sssp;
  if (p && kind == LanePool::BFS && parents && !p->parents()) {
    delete p;
    p = nullptr;
  }
  if (!p) p = new LanePool(g, kind, parents);
  *status = p->open();
  return p;
}

void pools_destroy(gg_graph *g) {
  delete g->pool_bfs;
  delete g->pool_sssp;
  g->pool_bfs = g->pool_sssp = nullptr;
}

// Runs one batch of roots to completion on the graph's pool.
static int run_batch(gg_graph *g, LanePool::Kind kind, const uint32_t *roots, int nroots, bool parents,
                     int32_t *levels, uint32_t *par_out, float *dist_out, uint64_t *reached, uint64_t *checksum,
                     uint64_t *lane_edges, gg_run_stats *stats) {
  if (!g || !roots || nroots < 1 || nroots > LANES) {
    set_error("need a graph and 1..64 roots");
    return GG_ERR_INVALID;
  }
  if (kind == LanePool::SSSP && !g->weighted) {
    set_error("sssp needs a weighted graph");
    return GG_ERR_UNWEIGHTED;
  }
  for (int i = 0; i < nroots; i++)
    if (roots[i] >= g->V) {
      set_error("root %u >= vertices %u", roots[i], g->V);
      return GG_ERR_INVALID;
    }
  GG_CUDA(cudaSetDevice(g->device));
  int status = GG_OK;
  LanePool *p = graph_pool(g, kind, parents, &status);
  if (status != GG_OK) return status;
  Trace tr(stats, g, kind == LanePool::BFS ? "gg_bfs_batched" : "gg_sssp_batched");
  p->set_trace(&tr);
  p->set_level_lists(kind == LanePool::BFS && !parents && g->batched_lists);
  p->launches = 0;
  const uint32_t V = g->V;
  int lanes[LANES];
  for (int i = 0; i < nroots; i++) lanes[i] = i;
  cudaStream_t gs = g->stream;
  g->stream = p->stream();  // events and traces on the pool's stream
  status = timed_begin(g);
  if (status == GG_OK) status = p->admit(roots, lanes, nroots);
  if (status == GG_OK) status = p->run(tr.timing_requested() != 0);
  const u64 mask = nroots == 64 ? ~0ull : ((1ull << nroots) - 1);
  u64 r[LANES], c[LANES], e[LANES];
  if (status == GG_OK) status = p->digest(mask, r, checksum ? c : nullptr, e);
  int32_t *d_lv = nullptr;
  uint32_t *d_pa = nullptr;
  float *d_di = nullptr;
  if (status == GG_OK && levels) status = ws(g, WS_MS_OUT0, (size_t)V * nroots, &d_lv);
  if (status == GG_OK && par_out) status = ws(g, WS_MS_OUT1, (size_t)V * nroots, &d_pa);
  if (status == GG_OK && dist_out) status = ws(g, WS_MS_OUT0, (size_t)V * nroots, &d_di);
  if (status == GG_OK && (d_lv || d_pa || d_di)) status = p->extract(mask, d_lv, d_pa, d_di);
  if (status == GG_OK) status = timed_end(g, stats, p->launches);
  if (status == GG_OK) status = tr.collect();
  g->stream = gs;
  p->retire(mask);
  p->set_trace(nullptr);
  if (status != GG_OK) return status;
  if (levels) GG_CUDA(cudaMemcpy(levels, d_lv, sizeof(int32_t) * V * nroots, cudaMemcpyDeviceToHost));
  if (par_out) GG_CUDA(cudaMemcpy(par_out, d_pa, sizeof(uint32_t) * V * nroots, cudaMemcpyDeviceToHost));
  if (dist_out) GG_CUDA(cudaMemcpy(dist_out, d_di, sizeof(float) * V * nroots, cudaMemcpyDeviceToHost));
  for (int i = 0; i < nroots; i++) {
    if (reached) reached[i] = r[i];
    if (checksum) checksum[i] = c[i];
    if (lane_edges) lane_edges[i] = e[i];
  }
  g->result[0] = d_lv ? (const void *)d_lv : (const void *)d_di;
  g->result[1] = d_pa;
  return GG_OK;
}

}  // namespace gg

using namespace gg;

extern "C" int gg_bfs_batched(gg_graph *g, const uint32_t *roots, int nroots, int32_t *levels, uint32_t *parents,
                              uint64_t *reached, uint64_t *lane_edges, gg_run_stats *stats) {
  return run_batch(g, LanePool::BFS, roots, nroots, parents != nullptr, levels, parents, nullptr, reached, nullptr,
                   lane_edges, stats);
}

extern "C" int gg_sssp_batched(gg_graph *g, const uint32_t *roots, int nroots, float *distances, uint64_t *reached,
                               gg_run_stats *stats) {
  return run_batch(g, LanePool::SSSP, roots, nroots, false, nullptr, nullptr, distances, reached, nullptr, nullptr,
                   stats);
}

extern "C" uint64_t gg_result_checksum(const void *values, uint32_t vertices, int kind) {
  uint64_t sum = 0;
  for (uint32_t v = 0; v < vertices; v++) {
    uint32_t x;
    if (kind == 0) {
      int32_t lv = ((const int32_t *)values)[v];
      if (lv < 0) continue;
      x = (uint32_t)lv;
    } else {
      float d = ((const float *)values)[v];
      if (!(d < 1e9f)) continue;
      memcpy(&x, &d, 4);
    }
    sum += gg_mix64((uint64_t)v * 0x9E3779B97F4A7C15ull + x);
  }
  return sum;
}

extern "C" int gg_graph_set_batched_switch(gg_graph *g, uint32_t divisor) {
  if (!g) {
    set_error("null graph");
    return GG_ERR_INVALID;
  }
  g->batched_switch_div = divisor ? divisor : 20;
  return GG_OK;
}

extern "C" int gg_graph_set_batched_thread_lanes(gg_graph *g, uint32_t lanes) {
  if (!g || lanes > 64) {
    set_error("need a graph and at most 64 lanes");
    return GG_ERR_INVALID;
  }
  g->batched_thread_lanes = lanes;
  return GG_OK;
}

extern "C" int gg_graph_set_batched_lists(gg_graph *g, int on) {
  if (!g) {
    set_error("null graph");
    return GG_ERR_INVALID;
  }
  g->batched_lists = on ? 1 : 0;
  return GG_OK;
}

extern "C" int gg_graph_set_batched_graph(gg_graph *g, int on) {
  if (!g) {
    set_error("null graph");
    return GG_ERR_INVALID;
  }
  g->batched_graph = on ? 1 : 0;
  return GG_OK;
}

int gg_graph_set_sssp_delta(gg_graph *g, float delta) {
  if (!g || !(delta >= 0.0f)) {
    gg::set_error("the bucket width must be >= 0");
    return GG_ERR_INVALID;
  }
  g->sssp_delta = delta;
  return GG_OK;
}
