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
#include <vector>

#include "gg_engine.cuh"

namespace gg {

typedef unsigned long long u64;
constexpr int LANES = 64;

struct MsCounters {
  u64 alive;           // OR of the lanes activated this iteration
  u64 edges;           // sum of out_degree over vertices touched this iteration
  unsigned int touched;
  unsigned int qlen;
};

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

__global__ void ms_roots(const uint32_t *roots, int n, u64 *front, u64 *visit, uint32_t *lvl, uint32_t *par,
                         uint32_t iter, const uint32_t *out_deg, MsCounters *mc) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  u64 alive = 0, edges = 0;
  unsigned touched = 0;
  for (int l = 0; l < n; l++) {
    uint32_t r = roots[l];
    if (!front[r]) {
      edges += out_deg[r];
      touched += 1;
    }
    front[r] |= 1ull << l;
    visit[r] |= 1ull << l;
    lvl[(size_t)r * LANES + l] = iter;
    if (par) par[(size_t)r * LANES + l] = r;
    alive |= 1ull << l;
  }
  mc->alive = alive;
  mc->edges = edges;
  mc->touched = touched;
}

// ---------------------------------------------------------------- BFS pull
// Light lists (<= LIGHT_DEG): the lane's own vertex, in CSC order, so each
// lane bit takes the first in-neighbour that has it (as bfs.cpp:63-66 does for
// one root).  next[v] is written for every v (0 for long lists, which the
// chunk kernel then ORs into).
__global__ void __launch_bounds__(256)
    ms_pull_light(Dir d, uint32_t V, u64 alive, const u64 *__restrict__ front, u64 *visit, u64 *next, uint32_t *lvl,
                  uint32_t *par, uint32_t iter, const uint32_t *__restrict__ out_deg, MsCounters *mc) {
  u64 t_alive = 0, t_edges = 0;
  unsigned t_touched = 0;
  for (size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x; v < ((size_t)V + 255) / 256 * 256;
       v += (size_t)gridDim.x * blockDim.x) {
    u64 acc = 0;
    if (v < V) {
      const u64 vis = visit[v];
      u64 need = ~vis & alive;
      const unsigned long long b = d.off[v], e = d.off[v + 1];
      if (need && e - b <= LIGHT_DEG) {
        for (unsigned long long k = b; k < e && need; k++) {
          const uint32_t u = d.nbr[k];
          const u64 m = front[u] & need;
          if (m) {
            ms_record((uint32_t)v, m, u, iter, lvl, par);
            acc |= m;
            need &= ~m;
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
  }
  ms_flush(mc, t_alive, t_edges, t_touched);
}

// Long lists: one warp per PULL_CHUNK-edge chunk; a lane bit goes to the
// entry that wins the atomicOr on next[v] (any in-neighbour in that lane's
// frontier is a valid parent).  visit[v] is not touched here.
__global__ void __launch_bounds__(256)
    ms_pull_chunks(Dir d, u64 alive, const u64 *__restrict__ front, const u64 *__restrict__ visit, u64 *next,
                   uint32_t *lvl, uint32_t *par, uint32_t iter) {
  const size_t nwarps = (size_t)gridDim.x * 8;
  const unsigned lane = lane_id();
  for (size_t c = (size_t)blockIdx.x * 8 + (threadIdx.x >> 5); c < d.nbigchunks; c += nwarps) {
    const uint32_t o = d.big_owner[c];
    const uint32_t v = d.big[o];
    u64 need = ~visit[v] & alive;
    if (!need) continue;
    const unsigned long long b = d.off[v] + (unsigned long long)(c - d.big_chunk[o]) * PULL_CHUNK;
    const unsigned long long end = d.off[v + 1];
    const unsigned long long e = b + PULL_CHUNK < end ? b + PULL_CHUNK : end;
    for (unsigned long long base = b; base < e; base += 32) {
      need &= ~*(volatile u64 *)(next + v);
      if (!need) break;
      const unsigned long long k = base + lane;
      u64 m = 0;
      uint32_t u = 0;
      if (k < e) {
        u = d.nbr[k];
        m = front[u] & need;
      }
      if (m) {
        const u64 won = m & ~atomicOr(next + v, m);
        if (won) ms_record(v, won, u, iter, lvl, par);
      }
    }
  }
}

// visit |= next for the long-list vertices, and their tallies.
__global__ void ms_big_finish(Dir d, u64 *visit, const u64 *__restrict__ next, const uint32_t *__restrict__ out_deg,
                              MsCounters *mc) {
  u64 t_alive = 0, t_edges = 0;
  unsigned t_touched = 0;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < ((size_t)d.nbig + 255) / 256 * 256;
       i += (size_t)gridDim.x * blockDim.x) {
    if (i < d.nbig) {
      const uint32_t v = d.big[i];
      const u64 nx = next[v];
      if (nx) {
        visit[v] |= nx;
        t_alive |= nx;
        t_edges += out_deg[v];
        t_touched += 1;
      }
    }
  }
  ms_flush(mc, t_alive, t_edges, t_touched);
}

// ---------------------------------------------------------------- BFS push
// Edge-balanced over the union frontier queue (as push_lb): for edge (u, v)
// the lanes m = front[u] & ~visit[v] claim v through atomicOr on next[v];
// the first claimer of v appends it to the touched queue.
__global__ void __launch_bounds__(PUSH_THREADS)
    ms_push(const uint32_t *__restrict__ q, const unsigned long long *__restrict__ P, uint32_t n,
            unsigned long long total, Dir d, const u64 *__restrict__ front, const u64 *__restrict__ visit, u64 *next,
            uint32_t *lvl, uint32_t *par, uint32_t iter, uint32_t *q_out, MsCounters *mc) {
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
        v = d.nbr[d.off[u] + (e - P[i])];
        const u64 m = front[u] & ~visit[v];
        if (m && (m & ~*(volatile u64 *)(next + v))) {
          const u64 old = atomicOr(next + v, m);
          const u64 won = m & ~old;
          if (won) ms_record(v, won, u, iter, lvl, par);
          fresh = old == 0;
        }
      }
      queue_push(fresh, v, q_out, &mc->qlen);
    }
  }
}

// After a push: visit |= next over the touched queue, and the tallies.
__global__ void ms_push_finish(const uint32_t *__restrict__ q, uint32_t n, u64 *visit, const u64 *__restrict__ next,
                               const uint32_t *__restrict__ out_deg, MsCounters *mc) {
  u64 t_alive = 0, t_edges = 0;
  unsigned t_touched = 0;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < ((size_t)n + 255) / 256 * 256;
       i += (size_t)gridDim.x * blockDim.x) {
    if (i < n) {
      const uint32_t v = q[i];
      const u64 nx = next[v];
      visit[v] |= nx;
      t_alive |= nx;
      t_edges += out_deg[v];
      t_touched += 1;
    }
  }
  ms_flush(mc, t_alive, t_edges, t_touched);
}

// Clears mask entries of the n queued vertices.
__global__ void ms_clear_queue(const uint32_t *__restrict__ q, uint32_t n, u64 *mask) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    mask[q[i]] = 0;
}

// Ordered queue of the vertices with a nonzero mask.
struct NonzeroMask {
  const u64 *m;
  __device__ __forceinline__ uint32_t operator()(size_t i) const { return m[i] ? 1u : 0u; }
};
__global__ void ms_compact(const u64 *__restrict__ m, uint32_t V, const uint32_t *__restrict__ pos,
                           uint32_t *__restrict__ q) {
  for (size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (size_t)gridDim.x * blockDim.x)
    if (m[v]) q[pos[v]] = (uint32_t)v;
}

// Per-lane results in the caller's layout (lane-major), through a shared
// tile of 32 vertices x 64 lanes; also per-lane reached counts and edge sums.
__global__ void __launch_bounds__(256)
    ms_extract(uint32_t V, int n, const u64 *__restrict__ visit, const uint32_t *__restrict__ lvl,
               const uint32_t *__restrict__ par, const uint32_t *__restrict__ out_deg, int32_t *levels,
               uint32_t *parents, u64 *reached, u64 *edges) {
  __shared__ uint32_t s_lvl[32][LANES + 1];
  __shared__ uint32_t s_par[32][LANES + 1];
  __shared__ u64 s_vis[32];
  __shared__ uint32_t s_deg[32];
  __shared__ u64 s_reach[LANES], s_edge[LANES];
  if (threadIdx.x < LANES) {
    s_reach[threadIdx.x] = 0;
    s_edge[threadIdx.x] = 0;
  }
  __syncthreads();
  for (size_t v0 = (size_t)blockIdx.x * 32; v0 < V; v0 += (size_t)gridDim.x * 32) {
    for (int i = threadIdx.x; i < 32 * LANES; i += blockDim.x) {
      const int r = i / LANES, l = i % LANES;
      const size_t v = v0 + r;
      if (v < V) {
        s_lvl[r][l] = lvl[v * LANES + l];
        if (par) s_par[r][l] = par[v * LANES + l];
      }
    }
    if (threadIdx.x < 32) {
      const size_t v = v0 + threadIdx.x;
      s_vis[threadIdx.x] = v < V ? visit[v] : 0ull;
      s_deg[threadIdx.x] = v < V ? out_deg[v] : 0u;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 32 * n; i += blockDim.x) {
      const int l = i / 32, r = i % 32;
      const size_t v = v0 + r;
      if (v >= V) continue;
      const bool hit = (s_vis[r] >> l) & 1ull;
      if (levels) levels[(size_t)l * V + v] = hit ? (int32_t)s_lvl[r][l] : -1;
      if (parents) parents[(size_t)l * V + v] = hit ? s_par[r][l] : V;
      if (hit) {
        atomicAdd(&s_reach[l], 1ull);
        atomicAdd(&s_edge[l], (u64)s_deg[r]);
      }
    }
    __syncthreads();
  }
  if (threadIdx.x < (unsigned)n) {
    if (s_reach[threadIdx.x]) atomicAdd(&reached[threadIdx.x], s_reach[threadIdx.x]);
    if (s_edge[threadIdx.x]) atomicAdd(&edges[threadIdx.x], s_edge[threadIdx.x]);
  }
}

}  // namespace gg

using namespace gg;

namespace {

struct BatchBuffers {
  u64 *visit, *front, *next;
  uint32_t *lvl, *par, *q[2];
  MsCounters *mc;
  u64 *lane_reached, *lane_edges;
};

int ms_buffers(gg_graph *g, bool want_par, BatchBuffers *b) {
  const uint32_t V = g->V;
  GG_TRY(ws(g, WS_MS_VISIT, V, &b->visit));
  GG_TRY(ws(g, WS_MS_FRONT, V, &b->front));
  GG_TRY(ws(g, WS_MS_NEXT, V, &b->next));
  GG_TRY(ws(g, WS_MS_LVL, (size_t)V * LANES, &b->lvl));
  b->par = nullptr;
  if (want_par) GG_TRY(ws(g, WS_MS_PAR, (size_t)V * LANES, &b->par));
  GG_TRY(ws(g, WS_Q0, (size_t)V + 1, &b->q[0]));
  GG_TRY(ws(g, WS_Q1, (size_t)V + 1, &b->q[1]));
  char *blob;
  GG_TRY(ws(g, WS_MS_MISC, 256 + sizeof(u64) * 2 * LANES, &blob));
  b->mc = (MsCounters *)blob;
  b->lane_reached = (u64 *)(blob + 256);
  b->lane_edges = b->lane_reached + LANES;
  return GG_OK;
}

int ms_read(gg_graph *g, MsCounters *mc, MsCounters *h) {
  GG_CUDA(cudaMemcpyAsync(g->ws.ctr_host, mc, sizeof(MsCounters), cudaMemcpyDeviceToHost, g->stream));
  GG_CUDA(cudaStreamSynchronize(g->stream));
  memcpy(h, g->ws.ctr_host, sizeof(MsCounters));
  return GG_OK;
}

}  // namespace

extern "C" int gg_bfs_batched(gg_graph *g, const uint32_t *roots, int nroots, int32_t *levels, uint32_t *parents,
                              uint64_t *reached, uint64_t *lane_edges, gg_run_stats *stats) {
  if (!g || !roots || nroots < 1 || nroots > LANES) {
    set_error("need a graph and 1..64 roots");
    return GG_ERR_INVALID;
  }
  for (int i = 0; i < nroots; i++)
    if (roots[i] >= g->V) {
      set_error("root %u >= vertices %u", roots[i], g->V);
      return GG_ERR_INVALID;
    }
  GG_CUDA(cudaSetDevice(g->device));
  const uint32_t V = g->V;
  BatchBuffers b;
  GG_TRY(ms_buffers(g, parents != nullptr, &b));
  Launch L(g);
  Trace tr(stats, g);
  cudaStream_t s = g->stream;
  uint32_t *d_roots;
  GG_TRY(ws(g, WS_MS_ROOTS, LANES, &d_roots));
  GG_TRY(timed_begin(g));
  GG_CUDA(cudaMemcpyAsync(d_roots, roots, sizeof(uint32_t) * nroots, cudaMemcpyHostToDevice, s));
  GG_CUDA(cudaMemsetAsync(b.visit, 0, sizeof(u64) * V, s));
  GG_CUDA(cudaMemsetAsync(b.front, 0, sizeof(u64) * V, s));
  GG_CUDA(cudaMemsetAsync(b.mc, 0, 256 + sizeof(u64) * 2 * LANES, s));
  ms_roots<<<1, 32, 0, s>>>(d_roots, nroots, b.front, b.visit, b.lvl, b.par, 0, g->out.deg, b.mc);
  L.launches += 1;
  GG_CUDA(cudaGetLastError());
  MsCounters h;
  GG_TRY(ms_read(g, b.mc, &h));
  // queue of the union frontier, when the next iteration pushes
  {
    uint32_t *pos, *scratch;
    GG_TRY(ws(g, WS_QPOS, (size_t)V + 1, &pos));
    GG_TRY(ws(g, WS_SCAN32, scan_scratch_elems(V), &scratch));
    GG_CUDA((exclusive_scan<uint32_t, NonzeroMask>(NonzeroMask{b.front}, V, pos, scratch, s, &L.launches)));
    ms_compact<<<grid_for(V, 256, g->num_sms), 256, 0, s>>>(b.front, V, pos, b.q[0]);
    L.launches += 1;
  }
  uint32_t nq = h.touched;
  bool qvalid = true;
  u64 alive = h.alive;
  unsigned long long ae = h.edges;
  int cur = 0;
  bool next_clear = false;  // next[] is all zero
  for (uint32_t iter = 1; alive; iter++) {
    const bool sparse = ae < g->E / 20;
    tr.add(sparse ? 0 : 1, ae, 0);
    GG_CUDA(cudaMemsetAsync(b.mc, 0, sizeof(MsCounters), s));
    if (sparse) {
      if (!qvalid) {
        uint32_t *pos, *scratch;
        GG_TRY(ws(g, WS_QPOS, (size_t)V + 1, &pos));
        GG_TRY(ws(g, WS_SCAN32, scan_scratch_elems(V), &scratch));
        GG_CUDA((exclusive_scan<uint32_t, NonzeroMask>(NonzeroMask{b.front}, V, pos, scratch, s, &L.launches)));
        ms_compact<<<grid_for(V, 256, g->num_sms), 256, 0, s>>>(b.front, V, pos, b.q[cur]);
        GG_CUDA(cudaMemcpyAsync(g->ws.ctr_host, pos + V, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
        GG_CUDA(cudaStreamSynchronize(s));
        nq = *(uint32_t *)g->ws.ctr_host;
        L.launches += 1;
      }
      if (!next_clear) GG_CUDA(cudaMemsetAsync(b.next, 0, sizeof(u64) * V, s));
      if (ae > 0) {
        unsigned long long *P;
        GG_TRY(L.scan_queue_degrees(b.q[cur], nq, g->out.deg, &P));
        GG_TRY(tr.kbegin());
        ms_push<<<L.push_grid(ae), PUSH_THREADS, 0, s>>>(b.q[cur], P, nq, ae, g->out, b.front, b.visit, b.next, b.lvl,
                                                          b.par, iter, b.q[cur ^ 1], b.mc);
        GG_TRY(tr.kend());
        L.launches += 1;
      }
      MsCounters hq;
      GG_TRY(ms_read(g, b.mc, &hq));
      if (hq.qlen)
        ms_push_finish<<<grid_for(hq.qlen, 256, g->num_sms), 256, 0, s>>>(b.q[cur ^ 1], hq.qlen, b.visit, b.next,
                                                                         g->out.deg, b.mc);
      // the old frontier becomes next: clear it through its queue
      ms_clear_queue<<<grid_for(nq ? nq : 1, 256, g->num_sms), 256, 0, s>>>(b.q[cur], nq, b.front);
      L.launches += 2;
      GG_TRY(ms_read(g, b.mc, &h));
      nq = h.qlen;
      qvalid = true;
      cur ^= 1;
      next_clear = true;
    } else {
      GG_TRY(tr.kbegin());
      ms_pull_light<<<L.pull_grid(), 256, 0, s>>>(g->in, V, alive, b.front, b.visit, b.next, b.lvl, b.par, iter,
                                                  g->out.deg, b.mc);
      L.launches += 1;
      if (g->in.nbig) {
        ms_pull_chunks<<<grid_for((size_t)g->in.nbigchunks * 32, 256, g->num_sms, 8), 256, 0, s>>>(
            g->in, alive, b.front, b.visit, b.next, b.lvl, b.par, iter);
        ms_big_finish<<<grid_for(g->in.nbig, 256, g->num_sms), 256, 0, s>>>(g->in, b.visit, b.next, g->out.deg,
                                                                          b.mc);
        L.launches += 2;
      }
      GG_TRY(tr.kend());
      GG_TRY(ms_read(g, b.mc, &h));
      qvalid = false;
      next_clear = false;
    }
    GG_CUDA(cudaGetLastError());
    tr.set_activated(h.touched);
    alive = h.alive;
    ae = h.edges;
    u64 *t = b.front;
    b.front = b.next;
    b.next = t;
  }
  GG_CUDA(cudaMemsetAsync(b.lane_reached, 0, sizeof(u64) * 2 * LANES, s));
  int32_t *d_levels = nullptr;
  uint32_t *d_parents = nullptr;
  if (levels) GG_TRY(ws(g, WS_MS_OUT0, (size_t)V * nroots, &d_levels));
  if (parents) GG_TRY(ws(g, WS_MS_OUT1, (size_t)V * nroots, &d_parents));
  ms_extract<<<grid_for(((size_t)V + 31) / 32, 1, g->num_sms, 16), 256, 0, s>>>(
      V, nroots, b.visit, b.lvl, b.par, g->out.deg, d_levels, d_parents, b.lane_reached, b.lane_edges);
  L.launches += 1;
  GG_CUDA(cudaGetLastError());
  GG_TRY(timed_end(g, stats, L.launches));
  GG_TRY(tr.collect());
  if (levels) GG_CUDA(cudaMemcpy(levels, d_levels, sizeof(int32_t) * V * nroots, cudaMemcpyDeviceToHost));
  if (parents) GG_CUDA(cudaMemcpy(parents, d_parents, sizeof(uint32_t) * V * nroots, cudaMemcpyDeviceToHost));
  u64 hr[2 * LANES];
  GG_CUDA(cudaMemcpy(hr, b.lane_reached, sizeof(u64) * 2 * LANES, cudaMemcpyDeviceToHost));
  if (reached) memcpy(reached, hr, sizeof(u64) * nroots);
  if (lane_edges) memcpy(lane_edges, hr + LANES, sizeof(u64) * nroots);
  g->result[0] = d_levels;
  g->result[1] = d_parents;
  return GG_OK;
}

// ---------------------------------------------------------------- batched SSSP
namespace gg {

__global__ void msp_roots(const uint32_t *roots, int n, u64 *front, float *dist, const uint32_t *out_deg,
                          MsCounters *mc, uint32_t *q) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  u64 alive = 0, edges = 0;
  unsigned nq = 0;
  for (int l = 0; l < n; l++) {
    uint32_t r = roots[l];
    if (!front[r]) {
      edges += out_deg[r];
      if (out_deg[r]) q[nq++] = r;
    }
    front[r] |= 1ull << l;
    dist[(size_t)r * LANES + l] = 0.0f;
    alive |= 1ull << l;
  }
  mc->alive = alive;
  mc->edges = edges;
  mc->qlen = nq;
}

// Relaxation of every out-edge (u, v, w) of the union frontier, one warp per
// edge: lane j handles SSSP lanes j and j + 32 of the edge (a coalesced 256 B
// row of dist[v]).  A lane whose distance at v was lowered gets v's next bit;
// the first setter of next[v] queues v.  Reads dist[u] as it is now (the
// fixpoint, hence every lane's result, does not depend on that order).
__global__ void __launch_bounds__(PUSH_THREADS)
    msp_push(const uint32_t *__restrict__ q, const unsigned long long *__restrict__ P, uint32_t n,
             unsigned long long total, Dir d, const u64 *__restrict__ front, u64 *next, float *dist, uint32_t *q_out,
             MsCounters *mc) {
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
    const uint32_t lo = s_lo, hi = s_hi;
    __syncthreads();
    for (unsigned long long e = e0 + w; e < e1; e += PUSH_THREADS / 32) {
      const uint32_t i = upper_bound_idx<unsigned long long>(P, lo, hi, e) - 1;
      const uint32_t u = q[i];
      const unsigned long long k = d.off[u] + (e - P[i]);
      const uint32_t v = d.nbr[k];
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
  }
  ms_flush(mc, t_alive, t_edges, 0);
}

// dist, lane-major, and per-lane reached counts (distance < 1e9).
__global__ void __launch_bounds__(256)
    msp_extract(uint32_t V, int n, const float *__restrict__ dist, float *out, u64 *reached) {
  __shared__ float s_d[32][LANES + 1];
  __shared__ u64 s_reach[LANES];
  if (threadIdx.x < LANES) s_reach[threadIdx.x] = 0;
  __syncthreads();
  for (size_t v0 = (size_t)blockIdx.x * 32; v0 < V; v0 += (size_t)gridDim.x * 32) {
    for (int i = threadIdx.x; i < 32 * LANES; i += blockDim.x) {
      const int r = i / LANES, l = i % LANES;
      if (v0 + r < V) s_d[r][l] = dist[(v0 + r) * LANES + l];
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 32 * n; i += blockDim.x) {
      const int l = i / 32, r = i % 32;
      const size_t v = v0 + r;
      if (v >= V) continue;
      const float x = s_d[r][l];
      if (out) out[(size_t)l * V + v] = x;
      if (x < 1e9f) atomicAdd(&s_reach[l], 1ull);
    }
    __syncthreads();
  }
  if (threadIdx.x < (unsigned)n && s_reach[threadIdx.x]) atomicAdd(&reached[threadIdx.x], s_reach[threadIdx.x]);
}

}  // namespace gg

extern "C" int gg_sssp_batched(gg_graph *g, const uint32_t *roots, int nroots, float *distances, uint64_t *reached,
                               gg_run_stats *stats) {
  if (!g || !roots || nroots < 1 || nroots > LANES) {
    set_error("need a graph and 1..64 roots");
    return GG_ERR_INVALID;
  }
  if (!g->weighted) {
    set_error("sssp needs a weighted graph");
    return GG_ERR_UNWEIGHTED;
  }
  for (int i = 0; i < nroots; i++)
    if (roots[i] >= g->V) {
      set_error("root %u >= vertices %u", roots[i], g->V);
      return GG_ERR_INVALID;
    }
  GG_CUDA(cudaSetDevice(g->device));
  const uint32_t V = g->V;
  u64 *front, *next;
  float *dist;
  uint32_t *q[2], *d_roots;
  char *blob;
  GG_TRY(ws(g, WS_MS_FRONT, V, &front));
  GG_TRY(ws(g, WS_MS_NEXT, V, &next));
  GG_TRY(ws(g, WS_MS_DIST, (size_t)V * LANES, &dist));
  GG_TRY(ws(g, WS_Q0, (size_t)V + 1, &q[0]));
  GG_TRY(ws(g, WS_Q1, (size_t)V + 1, &q[1]));
  GG_TRY(ws(g, WS_MS_ROOTS, LANES, &d_roots));
  GG_TRY(ws(g, WS_MS_MISC, 256 + sizeof(u64) * 2 * LANES, &blob));
  MsCounters *mc = (MsCounters *)blob;
  u64 *lane_reached = (u64 *)(blob + 256);
  Launch L(g);
  Trace tr(stats, g);
  cudaStream_t s = g->stream;
  GG_TRY(timed_begin(g));
  GG_CUDA(cudaMemcpyAsync(d_roots, roots, sizeof(uint32_t) * nroots, cudaMemcpyHostToDevice, s));
  GG_CUDA(cudaMemsetAsync(front, 0, sizeof(u64) * V, s));
  GG_CUDA(cudaMemsetAsync(next, 0, sizeof(u64) * V, s));
  GG_CUDA(cudaMemsetAsync(blob, 0, 256 + sizeof(u64) * 2 * LANES, s));
  fill_kernel<float><<<grid_for((size_t)V * LANES, 256, g->num_sms, 16), 256, 0, s>>>(dist, (size_t)V * LANES, 1e9f);
  msp_roots<<<1, 32, 0, s>>>(d_roots, nroots, front, dist, g->out.deg, mc, q[0]);
  L.launches += 2;
  GG_CUDA(cudaGetLastError());
  MsCounters h;
  GG_TRY(ms_read(g, mc, &h));
  uint32_t nq = h.qlen;
  unsigned long long ae = h.edges;
  int cur = 0;
  while (nq > 0 && ae > 0) {
    tr.add(0, ae, 0);
    GG_CUDA(cudaMemsetAsync(mc, 0, sizeof(MsCounters), s));
    unsigned long long *P;
    GG_TRY(L.scan_queue_degrees(q[cur], nq, g->out.deg, &P));
    GG_TRY(tr.kbegin());
    msp_push<<<L.push_grid(ae), PUSH_THREADS, 0, s>>>(q[cur], P, nq, ae, g->out, front, next, dist, q[cur ^ 1], mc);
    GG_TRY(tr.kend());
    // the old frontier becomes next: clear its entries
    ms_clear_queue<<<grid_for(nq, 256, g->num_sms), 256, 0, s>>>(q[cur], nq, front);
    L.launches += 2;
    GG_CUDA(cudaGetLastError());
    GG_TRY(ms_read(g, mc, &h));
    tr.set_activated(h.qlen);
    nq = h.qlen;
    ae = h.edges;
    u64 *t = front;
    front = next;
    next = t;
    cur ^= 1;
  }
  float *d_out = nullptr;
  if (distances) GG_TRY(ws(g, WS_MS_OUT0, (size_t)V * nroots, &d_out));
  GG_CUDA(cudaMemsetAsync(lane_reached, 0, sizeof(u64) * LANES, s));
  msp_extract<<<grid_for(((size_t)V + 31) / 32, 1, g->num_sms, 16), 256, 0, s>>>(V, nroots, dist, d_out, lane_reached);
  L.launches += 1;
  GG_CUDA(cudaGetLastError());
  GG_TRY(timed_end(g, stats, L.launches));
  GG_TRY(tr.collect());
  if (distances) GG_CUDA(cudaMemcpy(distances, d_out, sizeof(float) * V * nroots, cudaMemcpyDeviceToHost));
  if (reached) GG_CUDA(cudaMemcpy(reached, lane_reached, sizeof(u64) * nroots, cudaMemcpyDeviceToHost));
  g->result[0] = d_out;
  g->result[1] = nullptr;
  return GG_OK;
}
