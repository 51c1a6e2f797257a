// Batched betweenness centrality: up to 64 roots (lanes) of Brandes'
// dependency computation in one pass over the graph per level, as
// toolkits/bc.cpp:24-196 does for one root.
//
// Layout (vertex-major, lane l of vertex v at v * 64 + l):
//   np   double  path counts; 1 / np is the reference's inv_num_paths
//   dep  double  dependencies
//   levels  per level, the compacted list of the vertices on it in some lane
//           with their lane masks (uint32 id + u64 mask): the memory trade of
//           the reference's compute_compact (bc.cpp:198-404, a level array
//           instead of one bitmap per level, bc.cpp:34-35).  12 B per
//           (vertex, level) pair that occurs in some lane, instead of 8 B per
//           vertex per level; two dense u64 mask arrays are rebuilt from the
//           lists for the level at hand and the next one.
//   visit u64    lanes that have reached the vertex
// Forward (bc.cpp:48-111), per level and for all lanes at once: the sparse /
// dense switch on the union frontier's out-degree sum (core/graph.hpp:1509);
// push = each frontier edge u -> v adds np[u][l] to np[v][l] for the lanes
// where u is on the frontier and v is unvisited; pull = each vertex sums the
// path counts of its in-neighbours on the frontier, lane by lane.  Path
// counts are integers, added exactly (below 2^53), so the order of the
// atomic adds does not matter.
// Backward (bc.cpp:112-176), deepest level first: dep[v][l] = (sum over the
// out-neighbours w on the next level of lane l of dep[w][l]) + 1 / np[v][l],
// each sum in out-list order (long lists: chunk partials combined in chunk
// order), then dep = (dep - inv) / inv (bc.cpp:177-183).  Unreached
// vertices end as NaN with inv = inf, as in the reference.
#include <vector>

#include "gg_common.cuh"
#include "gg_scan.cuh"

namespace gg {

namespace {

using u64 = unsigned long long;
constexpr int BCB_LANES = 64;

struct NonzeroU64 {
  const u64 *m;
  __device__ __forceinline__ uint32_t operator()(size_t i) const { return m[i] ? 1u : 0u; }
};

__device__ __forceinline__ u64 shfl_u64(u64 x, int src) {
  const unsigned lo = __shfl_sync(GG_FULL, (unsigned)x, src), hi = __shfl_sync(GG_FULL, (unsigned)(x >> 32), src);
  return ((u64)hi << 32) | lo;
}

__global__ void bcb_init(const uint32_t *roots, int n, u64 *visit, u64 *front, double *np) {
  const int l = threadIdx.x;
  if (l < n) {
    const uint32_t r = roots[l];
    atomicOr(visit + r, 1ull << l);
    atomicOr(front + r, 1ull << l);
    np[(size_t)r * BCB_LANES + l] = 1.0;
  }
}

// The level list of a dense mask array: (v, m[v]) for m[v] != 0, in vertex order.
__global__ void bcb_compact(const u64 *__restrict__ m, uint32_t V, const uint32_t *__restrict__ pos,
                            uint32_t *__restrict__ qv, u64 *__restrict__ qm) {
  for (size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (size_t)gridDim.x * blockDim.x) {
    const u64 x = m[v];
    if (x) {
      qv[pos[v]] = (uint32_t)v;
      qm[pos[v]] = x;
    }
  }
}

// dense[qv[i]] = qm[i], or 0 for every listed vertex when qm is null.
__global__ void bcb_scatter(const uint32_t *__restrict__ qv, const u64 *__restrict__ qm, uint32_t n, u64 *dense) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    dense[qv[i]] = qm ? qm[i] : 0ull;
}

// Out-degree sum of a level list (the switch's active_edges).
__global__ void bcb_list_degrees(const uint32_t *__restrict__ qv, uint32_t n, const uint32_t *__restrict__ out_deg,
                                 Counters *ctr) {
  Tally t;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    t.edges += out_deg[qv[i]];
    t.activated += 1;
  }
  t.flush(ctr);
}

// Sparse level: every out-edge of the queued frontier, edge-balanced (edge e
// belongs to queue entry upper_bound(prefix, e) - 1).
__global__ void __launch_bounds__(256)
    bcb_push(Dir d, const uint32_t *__restrict__ q, const u64 *__restrict__ prefix, uint32_t nq,
             const u64 *__restrict__ front, const u64 *__restrict__ visit, u64 *next, double *np) {
  const u64 total = prefix[nq];
  for (u64 e = (u64)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (u64)gridDim.x * blockDim.x) {
    uint32_t lo = 0, hi = nq;
    while (lo < hi) {
      const uint32_t mid = (lo + hi) >> 1;
      if (prefix[mid] <= e)
        lo = mid + 1;
      else
        hi = mid;
    }
    const uint32_t i = lo - 1, u = q[i];
    const uint32_t v = nbr_at(d, d.off[u] + (e - prefix[i]), GG_SITE);
    u64 m = front[u] & ~visit[v];
    if (!m) continue;
    atomicOr(next + v, m);
    while (m) {
      const int l = __ffsll((long long)m) - 1;
      m &= m - 1;
      atomicAdd(np + (size_t)v * BCB_LANES + l, np[(size_t)u * BCB_LANES + l]);
    }
  }
}

// One warp sums, lane by lane, the path counts of the in-neighbours in
// [b, e) that are on the frontier in the lanes of `need`: thread t keeps
// lanes t and t + 32.  Returns the lanes that got a contribution.
__device__ __forceinline__ u64 warp_gather_paths(const Dir &d, u64 b, u64 e, u64 need, const u64 *__restrict__ front,
                                                 const double *np, double *a0, double *a1) {
  const unsigned lane = lane_id();
  u64 got = 0;
  for (u64 base = b; base < e; base += 32) {
    const u64 k = base + lane;
    uint32_t u = 0;
    u64 f = 0;
    if (k < e) {
      u = nbr_at(d, k, GG_SITE);
      f = front[u] & need;
    }
    unsigned bal = __ballot_sync(GG_FULL, f != 0);
    while (bal) {
      const int j = __ffs(bal) - 1;
      bal &= bal - 1;
      const uint32_t uj = __shfl_sync(GG_FULL, u, j);
      const u64 fj = shfl_u64(f, j);
      got |= fj;
      if ((fj >> lane) & 1ull) *a0 += np[(size_t)uj * BCB_LANES + lane];
      if ((fj >> (lane + 32)) & 1ull) *a1 += np[(size_t)uj * BCB_LANES + lane + 32];
    }
  }
  return got;
}

// Dense level, in-lists up to d.light: a warp takes 32 consecutive vertices
// and serves, one at a time, those unvisited in some live lane.
__global__ void __launch_bounds__(256)
    bcb_pull_light(Dir d, uint32_t V, u64 alive, const u64 *__restrict__ front, const u64 *__restrict__ visit,
                   u64 *next, double *np) {
  const size_t nwarps = (size_t)gridDim.x * 8;
  const unsigned lane = lane_id();
  for (size_t g = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; g * 32 < V; g += nwarps) {
    const uint32_t v = (uint32_t)(g * 32 + lane);
    u64 need = 0;
    if (v < V) {
      const u64 deg = d.off[v + 1] - d.off[v];
      if (deg > 0 && deg <= d.light) need = ~visit[v] & alive;
    }
    unsigned todo = __ballot_sync(GG_FULL, need != 0);
    while (todo) {
      const int j = __ffs(todo) - 1;
      todo &= todo - 1;
      const uint32_t vj = (uint32_t)(g * 32 + j);
      const u64 nj = shfl_u64(need, j);
      double a0 = 0.0, a1 = 0.0;
      const u64 got = warp_gather_paths(d, d.off[vj], d.off[vj + 1], nj, front, np, &a0, &a1);
      if ((got >> lane) & 1ull) np[(size_t)vj * BCB_LANES + lane] = a0;
      if ((got >> (lane + 32)) & 1ull) np[(size_t)vj * BCB_LANES + lane + 32] = a1;
      if (lane == 0 && got) next[vj] = got;
    }
  }
}

// Dense level, longer in-lists: one warp per chunk, added atomically (exact).
__global__ void __launch_bounds__(256)
    bcb_pull_chunks(Dir d, u64 alive, const u64 *__restrict__ front, const u64 *__restrict__ visit, u64 *next,
                    double *np) {
  const size_t nwarps = (size_t)gridDim.x * 8;
  const unsigned lane = lane_id();
  for (size_t c = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < d.nbigchunks; c += nwarps) {
    uint32_t v;
    unsigned long long lo, b, e;
    big_range(d, (uint32_t)c, d.chunk, &v, &lo, &b, &e);
    const u64 need = ~visit[v] & alive;
    if (!need) continue;
    double a0 = 0.0, a1 = 0.0;
    const u64 got = warp_gather_paths(d, b, e, need, front, np, &a0, &a1);
    if ((got >> lane) & 1ull) atomicAdd(np + (size_t)v * BCB_LANES + lane, a0);
    if ((got >> (lane + 32)) & 1ull) atomicAdd(np + (size_t)v * BCB_LANES + lane + 32, a1);
    if (lane == 0 && got) atomicOr(next + v, got);
  }
}

// visit |= next; the lanes still advancing and the vertices reached.
__global__ void bcb_advance(u64 *visit, const u64 *__restrict__ next, uint32_t V, u64 *alive_out, Counters *ctr) {
  Tally t;
  u64 alive = 0;
  for (size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (size_t)gridDim.x * blockDim.x) {
    const u64 n = next[v];
    if (n) {
      visit[v] |= n;
      alive |= n;
      t.activated += 1;
    }
  }
  for (int o = 16; o > 0; o >>= 1) alive |= __shfl_xor_sync(GG_FULL, alive, o);
  if (lane_id() == 0 && alive) atomicOr(alive_out, alive);
  t.flush(ctr);
}

// One warp sums, lane by lane over the lanes of m, the dependencies of the
// out-neighbours in [b, e) that sit on the next level (nxt) in that lane.
__device__ __forceinline__ void warp_gather_dep(const Dir &d, u64 b, u64 e, u64 m, const u64 *__restrict__ nxt,
                                                const double *__restrict__ dep, double *s0, double *s1) {
  const unsigned lane = lane_id();
  for (u64 base = b; base < e; base += 32) {
    const u64 k = base + lane;
    uint32_t w = 0;
    u64 f = 0;
    if (k < e) {
      w = nbr_at(d, k, GG_SITE);
      f = nxt[w] & m;
    }
    unsigned bal = __ballot_sync(GG_FULL, f != 0);
    while (bal) {
      const int j = __ffs(bal) - 1;
      bal &= bal - 1;
      const uint32_t wj = __shfl_sync(GG_FULL, w, j);
      const u64 fj = shfl_u64(f, j);
      if ((fj >> lane) & 1ull) *s0 += dep[(size_t)wj * BCB_LANES + lane];
      if ((fj >> (lane + 32)) & 1ull) *s1 += dep[(size_t)wj * BCB_LANES + lane + 32];
    }
  }
}

// Backward level L, out-lists up to d.light (and empty ones): dep = sum + inv
// for every lane in which the vertex sits on level L.
__global__ void __launch_bounds__(256)
    bcb_back_light(Dir d, uint32_t V, const u64 *__restrict__ cur, const u64 *__restrict__ nxt, double *dep,
                   const double *__restrict__ np) {
  const size_t nwarps = (size_t)gridDim.x * 8;
  const unsigned lane = lane_id();
  for (size_t g = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; g * 32 < V; g += nwarps) {
    const uint32_t v = (uint32_t)(g * 32 + lane);
    u64 m = 0;
    if (v < V && d.off[v + 1] - d.off[v] <= d.light) m = cur[v];
    unsigned todo = __ballot_sync(GG_FULL, m != 0);
    while (todo) {
      const int j = __ffs(todo) - 1;
      todo &= todo - 1;
      const uint32_t vj = (uint32_t)(g * 32 + j);
      const u64 mj = shfl_u64(m, j);
      double s0 = 0.0, s1 = 0.0;
      if (nxt) warp_gather_dep(d, d.off[vj], d.off[vj + 1], mj, nxt, dep, &s0, &s1);
      const size_t o = (size_t)vj * BCB_LANES;
      if ((mj >> lane) & 1ull) dep[o + lane] = s0 + 1.0 / np[o + lane];
      if ((mj >> (lane + 32)) & 1ull) dep[o + lane + 32] = s1 + 1.0 / np[o + lane + 32];
    }
  }
}

// Backward level L, longer out-lists: per chunk partial sums (64 per chunk),
// then one warp per vertex adds them up in chunk order.
__global__ void __launch_bounds__(256)
    bcb_back_chunks(Dir d, const u64 *__restrict__ cur, const u64 *__restrict__ nxt, const double *__restrict__ dep,
                    double *partial) {
  const size_t nwarps = (size_t)gridDim.x * 8;
  const unsigned lane = lane_id();
  for (size_t c = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < d.nbigchunks; c += nwarps) {
    uint32_t v;
    unsigned long long lo, b, e;
    big_range(d, (uint32_t)c, d.chunk, &v, &lo, &b, &e);
    const u64 m = cur[v];
    if (!m) continue;
    double s0 = 0.0, s1 = 0.0;
    warp_gather_dep(d, b, e, m, nxt, dep, &s0, &s1);
    partial[c * BCB_LANES + lane] = s0;
    partial[c * BCB_LANES + lane + 32] = s1;
  }
}
__global__ void __launch_bounds__(256)
    bcb_back_finish(Dir d, const u64 *__restrict__ cur, const double *__restrict__ partial, double *dep,
                    const double *__restrict__ np) {
  const size_t nwarps = (size_t)gridDim.x * 8;
  const unsigned lane = lane_id();
  for (size_t i = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < d.nbig; i += nwarps) {
    const uint32_t v = d.big[i];
    const u64 m = cur[v];
    if (!m) continue;
    double s0 = 0.0, s1 = 0.0;
    for (uint32_t c = d.big_chunk[i]; c < d.big_chunk[i + 1]; c++) {
      s0 += partial[(size_t)c * BCB_LANES + lane];
      s1 += partial[(size_t)c * BCB_LANES + lane + 32];
    }
    const size_t o = (size_t)v * BCB_LANES;
    if ((m >> lane) & 1ull) dep[o + lane] = s0 + 1.0 / np[o + lane];
    if ((m >> (lane + 32)) & 1ull) dep[o + lane + 32] = s1 + 1.0 / np[o + lane + 32];
  }
}

// dep = (dep - inv) / inv, then both arrays lane-major for the n lanes in
// use (a 64 x 32 tile through shared memory); reached vertices per lane.
__global__ void __launch_bounds__(256)
    bcb_finish(const double *__restrict__ dep, const double *__restrict__ np, const u64 *__restrict__ visit,
               uint32_t V, int n, double *out_dep, double *out_inv, unsigned long long *reached) {
  __shared__ double s_dep[BCB_LANES][33];
  __shared__ double s_inv[BCB_LANES][33];
  __shared__ unsigned long long s_cnt[BCB_LANES];
  if (threadIdx.x < BCB_LANES) s_cnt[threadIdx.x] = 0;
  __syncthreads();
  for (size_t v0 = (size_t)blockIdx.x * 32; v0 < V; v0 += (size_t)gridDim.x * 32) {
    for (int i = threadIdx.x; i < 32 * BCB_LANES; i += blockDim.x) {
      const int vv = i / BCB_LANES, l = i % BCB_LANES;
      const size_t v = v0 + vv;
      double x = 0.0, inv = 0.0;
      if (v < V) {
        inv = 1.0 / np[v * BCB_LANES + l];
        x = (dep[v * BCB_LANES + l] - inv) / inv;
      }
      s_dep[l][vv] = x;
      s_inv[l][vv] = inv;
    }
    if (threadIdx.x < 32) {
      const size_t v = v0 + threadIdx.x;
      const u64 m = v < V ? visit[v] : 0ull;
      for (int l = 0; l < BCB_LANES; l++) {
        const unsigned c = __popc(__ballot_sync(GG_FULL, (m >> l) & 1ull));
        if (threadIdx.x == 0) s_cnt[l] += c;
      }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 32 * n; i += blockDim.x) {
      const int l = i / 32, vv = i % 32;
      const size_t v = v0 + vv;
      if (v < V) {
        if (out_dep) out_dep[(size_t)l * V + v] = s_dep[l][vv];
        if (out_inv) out_inv[(size_t)l * V + v] = s_inv[l][vv];
      }
    }
    __syncthreads();
  }
  if (threadIdx.x < (unsigned)n && s_cnt[threadIdx.x]) atomicAdd(reached + threadIdx.x, s_cnt[threadIdx.x]);
}

struct DevBuf {
  void *p = nullptr;
  DevBuf() = default;
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  DevBuf(DevBuf &&o) noexcept : p(o.p) { o.p = nullptr; }
  ~DevBuf() {
    if (p) cudaFree(p);
  }
};

}  // namespace

static int bc_batched_run(gg_graph *g, const uint32_t *roots, int n, double *dep_host, double *inv_host,
                          uint64_t *reached_host, gg_run_stats *st) {
  if (!g || !roots || n < 1 || n > BCB_LANES) {
    set_error("batched BC takes 1..64 roots");
    return GG_ERR_INVALID;
  }
  const uint32_t V = g->V;
  for (int i = 0; i < n; i++)
    if (roots[i] >= V) {
      set_error("root %u >= vertices %u", roots[i], V);
      return GG_ERR_INVALID;
    }
  GG_CUDA(cudaSetDevice(g->device));
  cudaStream_t s = g->stream;
  const size_t lanes_bytes = sizeof(double) * (size_t)V * BCB_LANES;
  DevBuf np_b, dep_b, visit_b, alive_b, roots_b, part_b, out_b, qpos_b, prefix_b, scan_b, scan64_b, ctr_b;
  GG_CUDA(cudaMalloc(&np_b.p, lanes_bytes));
  GG_CUDA(cudaMalloc(&dep_b.p, lanes_bytes));
  GG_CUDA(cudaMalloc(&visit_b.p, sizeof(u64) * V));
  GG_CUDA(cudaMalloc(&alive_b.p, sizeof(u64)));
  GG_CUDA(cudaMalloc(&roots_b.p, sizeof(uint32_t) * BCB_LANES));
  GG_CUDA(cudaMalloc(&ctr_b.p, sizeof(Counters)));
  GG_CUDA(cudaMalloc(&qpos_b.p, sizeof(uint32_t) * ((size_t)V + 1)));
  GG_CUDA(cudaMalloc(&prefix_b.p, sizeof(u64) * ((size_t)V + 1)));
  GG_CUDA(cudaMalloc(&scan_b.p, sizeof(uint32_t) * scan_scratch_elems((size_t)V + 1)));
  GG_CUDA(cudaMalloc(&scan64_b.p, sizeof(u64) * scan_scratch_elems((size_t)V + 1)));
  const uint32_t nbig = g->out.nbigchunks;
  GG_CUDA(cudaMalloc(&part_b.p, sizeof(double) * BCB_LANES * (nbig ? nbig : 1)));
  double *np = (double *)np_b.p, *dep = (double *)dep_b.p, *part = (double *)part_b.p;
  u64 *visit = (u64 *)visit_b.p, *alive_d = (u64 *)alive_b.p;
  Counters *ctr = (Counters *)ctr_b.p;
  uint32_t *qpos = (uint32_t *)qpos_b.p;
  u64 *prefix = (u64 *)prefix_b.p;
  // level lists (vertex ids, lane masks, count) and the two dense mask arrays
  struct Level {
    DevBuf v, m;
    uint32_t n = 0;
  };
  std::vector<Level> levels;
  DevBuf dense_b[2];
  for (DevBuf &b : dense_b) GG_CUDA(cudaMalloc(&b.p, sizeof(u64) * V));
  u64 *dense[2] = {(u64 *)dense_b[0].p, (u64 *)dense_b[1].p};
  auto new_level = [&](uint32_t count) -> int {
    levels.emplace_back();
    Level &l = levels.back();
    l.n = count;
    GG_CUDA(cudaMalloc(&l.v.p, sizeof(uint32_t) * (count ? count : 1)));
    GG_CUDA(cudaMalloc(&l.m.p, sizeof(u64) * (count ? count : 1)));
    return GG_OK;
  };
  auto lv = [&](int L) { return (const uint32_t *)levels[L].v.p; };
  auto lm = [&](int L) { return (const u64 *)levels[L].m.p; };
  Trace tr(st, g, "gg_bc_batched");
  int launches = 0;
  // level 0: the distinct roots and their lanes
  std::vector<uint32_t> r0;
  std::vector<u64> m0;
  for (int i = 0; i < n; i++) {
    size_t j = 0;
    while (j < r0.size() && r0[j] != roots[i]) j++;
    if (j == r0.size()) {
      r0.push_back(roots[i]);
      m0.push_back(0);
    }
    m0[j] |= 1ull << i;
  }
  GG_TRY(new_level((uint32_t)r0.size()));
  GG_CUDA(cudaMemcpyAsync(levels[0].v.p, r0.data(), sizeof(uint32_t) * r0.size(), cudaMemcpyHostToDevice, s));
  GG_CUDA(cudaMemcpyAsync(levels[0].m.p, m0.data(), sizeof(u64) * m0.size(), cudaMemcpyHostToDevice, s));
  GG_CUDA(cudaMemcpyAsync(roots_b.p, roots, sizeof(uint32_t) * n, cudaMemcpyHostToDevice, s));
  GG_TRY(timed_begin(g));
  GG_CUDA(cudaMemsetAsync(np, 0, lanes_bytes, s));
  GG_CUDA(cudaMemsetAsync(dep, 0, lanes_bytes, s));
  GG_CUDA(cudaMemsetAsync(visit, 0, sizeof(u64) * V, s));
  GG_CUDA(cudaMemsetAsync(dense[0], 0, sizeof(u64) * V, s));
  GG_CUDA(cudaMemsetAsync(dense[1], 0, sizeof(u64) * V, s));
  int cur = 0;
  u64 *front = dense[cur];
  bcb_init<<<1, BCB_LANES, 0, s>>>((const uint32_t *)roots_b.p, n, visit, front, np);
  launches += 1;
  const u64 all = n == 64 ? ~0ull : ((1ull << n) - 1);
  u64 alive = all;
  const unsigned vg = grid_for(V, 256, g->num_sms, 8);
  // ---- forward
  for (int L = 0;; L++) {
    Counters hc;
    const uint32_t nL = levels[L].n;
    GG_CUDA(cudaMemsetAsync(ctr, 0, sizeof(Counters), s));
    bcb_list_degrees<<<grid_for(nL ? nL : 1, 256, g->num_sms, 8), 256, 0, s>>>(lv(L), nL, g->out.deg, ctr);
    GG_CUDA(cudaMemcpyAsync(&hc, ctr, sizeof(Counters), cudaMemcpyDeviceToHost, s));
    GG_CUDA(cudaStreamSynchronize(s));
    launches += 1;
    const u64 ae = hc.edges;
    const bool sparse = ae < g->E / 20;
    tr.add(sparse ? 0 : 1, ae, 0);
    u64 *next = dense[cur ^ 1];
    if (sparse) {
      if (ae) {
        // the level list is the frontier queue
        GG_CUDA((exclusive_scan<unsigned long long, QueueDegreeIn>(QueueDegreeIn{lv(L), g->out.deg}, nL, prefix,
                                                                    (u64 *)scan64_b.p, s, &launches)));
        bcb_push<<<grid_for(ae, 256, g->num_sms, 16), 256, 0, s>>>(g->out, lv(L), prefix, nL, front, visit, next,
                                                                   np);
        launches += 1;
      }
    } else {
      bcb_pull_light<<<grid_for((size_t)V, 256, g->num_sms, 8), 256, 0, s>>>(g->in, V, alive, front, visit, next,
                                                                               np);
      launches += 1;
      if (g->in.nbigchunks) {
        bcb_pull_chunks<<<grid_for((size_t)g->in.nbigchunks * 32, 256, g->num_sms, 8), 256, 0, s>>>(
            g->in, alive, front, visit, next, np);
        launches += 1;
      }
    }
    GG_CUDA(cudaGetLastError());
    GG_CUDA(cudaMemsetAsync(ctr, 0, sizeof(Counters), s));
    GG_CUDA(cudaMemsetAsync(alive_d, 0, sizeof(u64), s));
    bcb_advance<<<vg, 256, 0, s>>>(visit, next, V, alive_d, ctr);
    launches += 1;
    GG_CUDA(cudaMemcpyAsync(&hc, ctr, sizeof(Counters), cudaMemcpyDeviceToHost, s));
    GG_CUDA(cudaMemcpyAsync(&alive, alive_d, sizeof(u64), cudaMemcpyDeviceToHost, s));
    GG_CUDA(cudaStreamSynchronize(s));
    tr.set_activated(hc.activated);
    // the next level's list, then this level's dense masks cleared for reuse
    if (hc.activated) {
      GG_TRY(new_level(hc.activated));
      GG_CUDA((exclusive_scan<uint32_t, NonzeroU64>(NonzeroU64{next}, V, qpos, (uint32_t *)scan_b.p, s,
                                                    &launches)));
      bcb_compact<<<vg, 256, 0, s>>>(next, V, qpos, (uint32_t *)levels[L + 1].v.p, (u64 *)levels[L + 1].m.p);
      launches += 1;
    }
    bcb_scatter<<<grid_for(nL ? nL : 1, 256, g->num_sms, 8), 256, 0, s>>>(lv(L), nullptr, nL, front);
    launches += 1;
    GG_CUDA(cudaGetLastError());
    cur ^= 1;
    front = next;
    if (!alive) break;
  }
  // both dense arrays are zero here: the last `next` had no lane, the other was cleared
  const int D = (int)levels.size();
  // ---- backward, deepest level first; cur / nxt are the dense masks of
  // levels L and L + 1, rebuilt from the lists
  const Dir &od = g->out;
  for (int L = D - 1; L >= 0; L--) {
    u64 *curm = dense[L & 1];
    u64 *nxtm = dense[(L + 1) & 1];
    const uint32_t nL = levels[L].n;
    bcb_scatter<<<grid_for(nL ? nL : 1, 256, g->num_sms, 8), 256, 0, s>>>(lv(L), lm(L), nL, curm);
    launches += 1;
    const u64 *nxt = L + 1 < D ? nxtm : nullptr;
    tr.add(1, 0, 0);
    bcb_back_light<<<grid_for((size_t)V, 256, g->num_sms, 8), 256, 0, s>>>(od, V, curm, nxt, dep, np);
    launches += 1;
    if (od.nbig) {
      if (nxt) {
        bcb_back_chunks<<<grid_for((size_t)od.nbigchunks * 32, 256, g->num_sms, 8), 256, 0, s>>>(od, curm, nxt, dep,
                                                                                                 part);
      } else {
        GG_CUDA(cudaMemsetAsync(part, 0, sizeof(double) * BCB_LANES * od.nbigchunks, s));
      }
      bcb_back_finish<<<grid_for((size_t)od.nbig * 32, 256, g->num_sms, 8), 256, 0, s>>>(od, curm, part, dep, np);
      launches += 2;
    }
    if (L + 1 < D) {
      // level L + 1's masks are no longer needed: clear them for level L - 1
      bcb_scatter<<<grid_for(levels[L + 1].n, 256, g->num_sms, 8), 256, 0, s>>>(lv(L + 1), nullptr, levels[L + 1].n,
                                                                                nxtm);
      launches += 1;
    }
    GG_CUDA(cudaGetLastError());
  }
  // ---- finish
  double *out_dep = nullptr, *out_inv = nullptr;
  if (dep_host || inv_host) {
    GG_CUDA(cudaMalloc(&out_b.p, sizeof(double) * 2 * (size_t)n * V));
    out_dep = (double *)out_b.p;
    out_inv = out_dep + (size_t)n * V;
  }
  DevBuf reached_b;
  GG_CUDA(cudaMalloc(&reached_b.p, sizeof(u64) * BCB_LANES));
  u64 *reached_d = (u64 *)reached_b.p;
  GG_CUDA(cudaMemsetAsync(reached_d, 0, sizeof(u64) * BCB_LANES, s));
  bcb_finish<<<grid_for(((size_t)V + 31) / 32 * 256, 256, g->num_sms, 8), 256, 0, s>>>(dep, np, visit, V, n, out_dep,
                                                                                        out_inv, reached_d);
  launches += 1;
  GG_CUDA(cudaGetLastError());
  GG_TRY(timed_end(g, st, launches));
  if (dep_host) GG_CUDA(cudaMemcpy(dep_host, out_dep, sizeof(double) * (size_t)n * V, cudaMemcpyDeviceToHost));
  if (inv_host) GG_CUDA(cudaMemcpy(inv_host, out_inv, sizeof(double) * (size_t)n * V, cudaMemcpyDeviceToHost));
  if (reached_host) {
    u64 r[BCB_LANES];
    GG_CUDA(cudaMemcpy(r, reached_d, sizeof(u64) * BCB_LANES, cudaMemcpyDeviceToHost));
    for (int i = 0; i < n; i++) reached_host[i] = r[i];
  }
  return GG_OK;
}

}  // namespace gg

extern "C" int gg_bc_batched(gg_graph *g, const uint32_t *roots, int nroots, double *dependencies,
                             double *inv_num_paths, uint64_t *reached, gg_run_stats *stats) {
  return gg::bc_batched_run(g, roots, nroots, dependencies, inv_num_paths, reached, stats);
}
