// BFS (toolkits/bfs.cpp) and PageRank (toolkits/pagerank.cpp) on the
// device engine, plus the process_vertices reduction of the switch.
#include <string.h>

#include "gg_engine.cuh"

namespace gg {

// ------------------------------------------------------------------ BFS
// Sparse slot (bfs.cpp:49-59): claim unvisited dst with a CAS on its parent.
struct BfsPush {
  uint32_t *parent;
  uint32_t V;
  // visited bits are set right after a vertex's parent: most already-reached
  // targets are turned away by this L2-resident bitmap, not by a random read
  // of the parent array; parent (then the CAS) stays the authority
  const uint32_t *visited;
  __device__ __forceinline__ bool push(uint32_t src, uint32_t, uint32_t dst, float) const {
    if (visited && bm_test(visited, dst)) return false;
    if (*(volatile uint32_t *)(parent + dst) != V) return false;
    return atomicCAS(parent + dst, V, src) == V;
  }
};

__global__ void bfs_root(uint32_t *parent, uint32_t root, uint32_t *visited, uint32_t *active, uint32_t *q,
                         const uint32_t *out_deg, Counters *ctr) {
  parent[root] = root;
  visited[root >> 5] |= 1u << (root & 31);
  active[root >> 5] |= 1u << (root & 31);
  q[0] = root;
  ctr->edges = out_deg[root];
  ctr->maxdeg = out_deg[root];
  ctr->activated = 1;
  ctr->qlen = 1;
}

// parent_slot: the workspace array the parent tree is written to (the
// pipelined calls alternate between two).
static int bfs_run(gg_graph *g, uint32_t root, uint32_t *parent_host, gg_run_stats *st, WsSlot parent_slot = WS_S0) {
  if (root >= g->V) {
    set_error("root %u >= vertices %u", root, g->V);
    return GG_ERR_INVALID;
  }
  GG_CUDA(cudaSetDevice(g->device));
  const uint32_t V = g->V;
  const size_t words = bitmap_words32(V);
  uint32_t *parent, *visited, *bm[2], *q[2];
  GG_TRY(ws(g, parent_slot, V, &parent));
  GG_TRY(ws(g, WS_BM0, words, &visited));
  GG_TRY(ws(g, WS_BM1, words, &bm[0]));
  GG_TRY(ws(g, WS_BM2, words, &bm[1]));
  GG_TRY(ws(g, WS_Q0, (size_t)V + 1, &q[0]));
  GG_TRY(ws(g, WS_Q1, (size_t)V + 1, &q[1]));
  Launch L(g);
  Trace tr(st, g, "gg_bfs");
  cudaStream_t s = g->stream;
  Counters *ctr = g->ws.ctr;
  GG_TRY(timed_begin(g));
  GG_CUDA(cudaMemsetAsync(visited, 0, words * 4, s));
  GG_CUDA(cudaMemsetAsync(bm[0], 0, words * 4, s));
  GG_TRY(counters_reset(g));
  fill_kernel<uint32_t><<<grid_for(V, 256, g->num_sms), 256, 0, s>>>(parent, V, V);
  bfs_root<<<1, 1, 0, s>>>(parent, root, visited, bm[0], q[0], g->out.deg, ctr);
  L.launches += 2;
  GG_CUDA(cudaGetLastError());
  Counters c;
  GG_TRY(counters_read(g, &c));
  unsigned long long ae = c.edges;
  uint32_t n_act = c.activated, nq = c.qlen, md = c.maxdeg;
  bool qvalid = true;  // q[cur] holds the active vertices with out-degree > 0
  int cur = 0;
  while (n_act > 0) {
    // the reference's mode (core/graph.hpp:1503-1509), recorded in the trace;
    // the kernel that runs follows g->bfs_pull_div (any in-neighbour on the
    // frontier is a valid parent, so the levels do not depend on it)
    const bool sparse = ae < g->E / 20;
    const bool push = ae < g->E / g->bfs_pull_div;
    if (sparse && push && qvalid && Launch::small_ok(nq, ae, md)) {
      // consecutive small sparse calls run on the device without host round trips
      GG_TRY((L.small_run<BfsPush, true, uint32_t>(g->out, BfsPush{parent, V, visited}, q, &cur, &nq, &ae, &md, &n_act, visited,
                                                   nullptr, nullptr, nullptr, tr, nullptr)));
      if (n_act > 0) {  // the next call is dense or large: its active set is q[cur]
        GG_CUDA(cudaMemsetAsync(bm[cur], 0, words * 4, s));
        if (nq) bitmap_from_queue<<<grid_for(nq, 256, g->num_sms), 256, 0, s>>>(q[cur], nq, bm[cur]);
        L.launches += 1;
      }
      continue;
    }
    tr.add(sparse ? 0 : 1, ae, 0);
    int nx = cur ^ 1;
    if (push && ae > 0 && !qvalid) GG_TRY(L.queue_from_bitmap(bm[cur], g->out.nz, q[cur], &nq));
    GG_CUDA(cudaMemsetAsync(bm[nx], 0, words * 4, s));
    GG_TRY(counters_reset(g));
    ActOut a;
    a.active_out = bm[nx];
    a.visited = visited;
    a.q_out = push ? q[nx] : nullptr;
    a.qlen = &ctr->qlen;
    a.out_deg = g->out.deg;
    a.queue_nonzero_only = true;
    if (push) {
      if (ae > 0) {
        unsigned long long *P;
        GG_TRY(L.scan_queue_degrees(q[cur], nq, g->out.deg, &P));
        GG_TRY(tr.kbegin());
        push_lb<BfsPush><<<L.push_grid(ae), PUSH_THREADS, 0, s>>>(q[cur], P, nq, ae, g->out, BfsPush{parent, V, visited},
                                                                    a, ctr);
        GG_TRY(tr.kend());
        L.launches += 1;
      }
    } else {
      GG_TRY(tr.kbegin());
      GG_TRY(L.bfs_pull(g->in, bm[cur], parent, a, ctr));
      GG_TRY(tr.kend());
    }
    GG_CUDA(cudaGetLastError());
    GG_TRY(counters_read(g, &c));
    n_act = c.activated;
    nq = c.qlen;
    md = c.maxdeg;
    qvalid = push;
    ae = c.edges;
    tr.set_activated(c.activated);
    cur = nx;
  }
  GG_TRY(timed_end(g, st, L.launches));
  GG_TRY(tr.collect());
  if (parent_host) GG_CUDA(cudaMemcpy(parent_host, parent, sizeof(uint32_t) * V, cudaMemcpyDeviceToHost));
  g->result[0] = parent;
  g->result[1] = nullptr;
  return GG_OK;
}

// ------------------------------------------------------------------ PageRank
// toolkits/pagerank.cpp:26-129.  Active = all vertices, so every
// process_edges call is dense (active_edges = edges >= edges/20); the pull
// gathers curr over the CSC and the process_vertices update that follows it
// (pagerank.cpp:77-97) is fused into the same kernel's epilogue.
template <typename T>
struct PrPull {
  using Acc = T;
  const T *curr;
  T *next;
  const uint32_t *out_deg;
  int last;
  uint32_t hot = 0xffffffffu;  // sources below this number are gathered through L1
  __device__ __forceinline__ bool want(uint32_t) const { return true; }
  __device__ __forceinline__ T identity(uint32_t) const { return T(0); }
  __device__ __forceinline__ T identity_coop() const { return T(0); }
  __device__ __forceinline__ T gather(const Dir &, unsigned long long, uint32_t u) const {
    return ld_gather(curr, u, hot);
  }
  __device__ __forceinline__ T combine(T a, T b) const { return a + b; }
  __device__ __forceinline__ T warp_combine(T x) const { return warp_sum(x); }
  __device__ __forceinline__ bool finish(uint32_t v, T sum, uint32_t, Tally &t) const;
};

template <>
__device__ __forceinline__ bool PrPull<double>::finish(uint32_t v, double sum, uint32_t, Tally &t) const {
  const double d = 0.85;
  double nv = __dadd_rn(1.0 - d, __dmul_rn(d, sum));
  if (!last) {
    uint32_t od = out_deg[v];
    if (od > 0) {
      nv = __ddiv_rn(nv, (double)od);
      t.delta += __dmul_rn(fabs(__dadd_rn(nv, -curr[v])), (double)od);
    } else {
      t.delta += fabs(__dadd_rn(nv, -curr[v]));
    }
  }
  next[v] = nv;
  return false;
}

template <>
__device__ __forceinline__ bool PrPull<float>::finish(uint32_t v, float sum, uint32_t, Tally &t) const {
  const float d = 0.85f;
  float nv = __fadd_rn(1.0f - d, __fmul_rn(d, sum));
  if (!last) {
    uint32_t od = out_deg[v];
    if (od > 0) {
      nv = __fdiv_rn(nv, (float)od);
      t.delta += (double)fabsf(__fadd_rn(nv, -curr[v])) * (double)od;
    } else {
      t.delta += (double)fabsf(__fadd_rn(nv, -curr[v]));
    }
  }
  next[v] = nv;
  return false;
}

template <typename T>
__global__ void pr_init(T *curr, const uint32_t *out_deg, uint32_t V) {
  for (size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (size_t)gridDim.x * blockDim.x) {
    uint32_t od = out_deg[v];
    curr[v] = od > 0 ? T(1) / (T)od : T(1);
  }
}

// Ranks computed in the hot-source numbering back to vertex order.
template <typename T>
__global__ void pr_unrank(const T *__restrict__ by_rank, const uint32_t *__restrict__ rank_of, uint32_t V,
                          T *__restrict__ out) {
  for (size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (size_t)gridDim.x * blockDim.x)
    out[v] = by_rank[rank_of[v]];
}

// pagerank.cpp:35-97.  With the hot-source layout (the default) the
// iterations run in that numbering: pr_od is the out-degree there, every
// vertex's arithmetic is unchanged, and only the order in which an in-list
// is summed differs from the plain adjacency (by source number).
template <typename T>
static int pr_run(gg_graph *g, int iterations, T *ranks_host, double *deltas_host, gg_run_stats *st) {
  if (iterations < 0) {
    set_error("iterations must be >= 0");
    return GG_ERR_INVALID;
  }
  GG_CUDA(cudaSetDevice(g->device));
  if (g->pr_layout) GG_TRY(pr_layout_build(g));
  const bool ranked = g->pr_layout && g->pr_ready;
  const Dir &din = ranked ? g->pr : g->in;
  const uint32_t *od = ranked ? g->pr_od : g->out.deg;
  const uint32_t V = g->V;
  T *buf[2], *out = nullptr;
  Counters *per_iter;
  if (ranked) GG_TRY(ws(g, WS_S0, (size_t)V, &out));
  GG_TRY(ws(g, WS_S2, (size_t)V, &buf[0]));
  GG_TRY(ws(g, WS_S3, (size_t)V, &buf[1]));
  GG_TRY(ws(g, WS_HUBSUM, (size_t)(iterations > 0 ? iterations : 1), &per_iter));
  Launch L(g);
  Trace tr(st, g, "gg_pagerank");
  cudaStream_t s = g->stream;
  const uint32_t hot = ranked ? (uint32_t)(g->l1_hot_bytes / sizeof(T)) : 0xffffffffu;
  T *part = nullptr;
  if (din.nbig) GG_TRY(ws(g, WS_PARTIAL, din.nbigchunks, &part));
  // The run is device work only, so it is captured once as a CUDA graph and
  // replayed while its arguments are unchanged: no launch gaps between the
  // iterations' kernels.
  PrGraphKey key;
  memset(&key, 0, sizeof(key));
  key.din = din;
  key.od = od;
  key.buf0 = buf[0];
  key.buf1 = buf[1];
  key.out = out;
  key.per_iter = per_iter;
  key.partial = part;
  key.V = V;
  key.iterations = iterations;
  key.tsize = (int32_t)sizeof(T);
  key.ranked = ranked;
  key.timing = tr.timing_requested();
  key.hot = hot;
  key.split = g->pull_light_blocks;
  key.side = g->side;
  const int slot = sizeof(T) == 4 ? 0 : 1;  // one cached graph per precision
  cudaGraphExec_t &exec = g->pr_exec[slot];
  const bool replay = exec && memcmp(&key, &g->pr_key[slot], sizeof(key)) == 0;
  int cur = 0;
  // bookkeeping (trace, launch count) always; launches only while capturing
  auto enqueue = [&](bool launch) -> int {
    if (launch) {
      GG_CUDA(cudaMemsetAsync(per_iter, 0, sizeof(Counters) * (iterations > 0 ? iterations : 1), s));
      pr_init<T><<<grid_for(V, 256, g->num_sms), 256, 0, s>>>(buf[0], od, V);
    }
    L.launches += 1;
    cur = 0;
    // active = all: active_edges = sum of out_degree = adjacency entries
    unsigned long long ae = g->nadj;
    for (int i = 0; i < iterations; i++) {
      tr.add(ae < g->E / 20 ? 0 : 1, ae, V);
      PrPull<T> op{buf[cur], buf[cur ^ 1], od, i == iterations - 1, hot};
      GG_TRY(tr.kbegin());
      if (launch)
        GG_TRY(L.pull(din, op, ActOut(), per_iter + i));
      else
        L.launches += Launch::pull_launches(din);
      GG_TRY(tr.kend());
      cur ^= 1;
    }
    if (ranked) {
      if (launch) pr_unrank<T><<<grid_for(V, 256, g->num_sms), 256, 0, s>>>(buf[cur], g->pr_rank_of, V, out);
      L.launches += 1;
    }
    if (launch) GG_CUDA(cudaGetLastError());
    return GG_OK;
  };
  if (!replay) {
    if (exec) GG_CUDA(cudaGraphExecDestroy(exec));
    exec = nullptr;
    GG_TRY(tr.reserve_events(2 * (size_t)iterations));
    GG_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    tr.capturing = true;
    const int rc = enqueue(true);
    tr.capturing = false;
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamEndCapture(s, &graph);
    if (rc == GG_OK && e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    if (rc != GG_OK) return rc;
    GG_CUDA(e);
    g->pr_key[slot] = key;
  } else {
    tr.replay = true;
    GG_TRY(enqueue(false));
  }
  GG_TRY(timed_begin(g));
  GG_CUDA(cudaGraphLaunch(exec, s));
  const T *result = ranked ? out : buf[cur];
  GG_TRY(timed_end(g, st, L.launches));
  GG_TRY(tr.collect());
  if (deltas_host && iterations > 0) {
    Counters *hc = new Counters[iterations];
    cudaError_t e = cudaMemcpy(hc, per_iter, sizeof(Counters) * iterations, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) {
      deltas_host[0] = 1.0;  // process_vertices returns 1 per vertex; divided by |V|
      for (int i = 1; i < iterations; i++) deltas_host[i] = hc[i - 1].delta / V;
    }
    delete[] hc;
    GG_CUDA(e);
  }
  if (ranks_host) GG_CUDA(cudaMemcpy(ranks_host, result, sizeof(T) * V, cudaMemcpyDeviceToHost));
  g->result[0] = result;
  g->result[1] = nullptr;
  return GG_OK;
}

// ------------------------------------------------------------------ process_vertices
__global__ void active_edges_kernel(const uint32_t *__restrict__ bm, size_t words, const uint32_t *__restrict__ deg,
                                    uint32_t V, Counters *ctr) {
  Tally t;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < words; i += (size_t)gridDim.x * blockDim.x) {
    uint32_t w = bm[i];
    while (w) {
      uint32_t b = __ffs(w) - 1;
      w &= w - 1;
      size_t v = i * 32 + b;
      if (v < V) t.edges += deg[v];
    }
  }
  t.flush(ctr);
}

}  // namespace gg

using namespace gg;

extern "C" {

int gg_bfs(gg_graph *g, uint32_t root, uint32_t *parent, gg_run_stats *stats) {
  if (!g) {
    set_error("null graph");
    return GG_ERR_INVALID;
  }
  return bfs_run(g, root, parent, stats);
}

int gg_graph_set_pr_layout(gg_graph *g, int hot_sources) {
  if (!g) {
    set_error("null graph");
    return GG_ERR_INVALID;
  }
  g->pr_layout = hot_sources ? 1 : 0;
  if (!g->pr_layout) pr_layout_free(g);
  return GG_OK;
}

int gg_graph_set_l1_hot(gg_graph *g, uint32_t l1_bytes) {
  if (!g) {
    set_error("null graph");
    return GG_ERR_INVALID;
  }
  g->l1_hot_bytes = l1_bytes;
  return GG_OK;
}

int gg_graph_set_dense_push(gg_graph *g, uint32_t divisor) {
  if (!g) {
    set_error("null graph");
    return GG_ERR_INVALID;
  }
  g->dense_push_div = divisor;
  return GG_OK;
}

int gg_graph_set_bfs_pull(gg_graph *g, uint32_t divisor) {
  if (!g || divisor == 0) {
    set_error("need a graph and a divisor > 0");
    return GG_ERR_INVALID;
  }
  g->bfs_pull_div = divisor;
  return GG_OK;
}

int gg_graph_set_pull_split(gg_graph *g, uint32_t light_blocks) {
  if (!g || light_blocks > 7) {
    set_error("need a graph and 0..7 light blocks per SM");
    return GG_ERR_INVALID;
  }
  g->pull_light_blocks = light_blocks;
  return GG_OK;
}

int gg_bfs_many(gg_graph *g, const uint32_t *roots, int n, uint32_t *const *parents, gg_run_stats *stats) {
  if (!g || !roots || n < 0 || (n && !parents)) {
    set_error("null argument");
    return GG_ERR_INVALID;
  }
  for (int i = 0; i < n; i++)
    if (roots[i] >= g->V) {
      set_error("root %u >= vertices %u", roots[i], g->V);
      return GG_ERR_INVALID;
    }
  GG_CUDA(cudaSetDevice(g->device));
  if (stats) {
    stats->calls = 0;
    stats->active_edges_total = 0;
    stats->device_ms = 0;
    stats->kernel_launches = 0;
  }
  const WsSlot slot[2] = {WS_S0, WS_PIPE};
  cudaStream_t cs = nullptr;
  cudaEvent_t done[2] = {nullptr, nullptr}, copied[2] = {nullptr, nullptr};
  int status = GG_OK;
  cudaError_t e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
  for (int b = 0; b < 2 && e == cudaSuccess; b++) {
    e = cudaEventCreateWithFlags(&done[b], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&copied[b], cudaEventDisableTiming);
  }
  if (e != cudaSuccess) status = cuda_status(e, "pipeline set-up");
  for (int i = 0; i < n && status == GG_OK; i++) {
    const int b = i & 1;
    // the buffer's previous result must be on the host before it is reused
    if (i >= 2) e = cudaStreamWaitEvent(g->stream, copied[b], 0);
    if (e != cudaSuccess) {
      status = cuda_status(e, "pipeline wait");
      break;
    }
    gg_run_stats one;
    memset(&one, 0, sizeof(one));
    status = bfs_run(g, roots[i], nullptr, &one, slot[b]);
    if (status != GG_OK) break;
    if (stats) {
      stats->calls += one.calls;
      stats->active_edges_total += one.active_edges_total;
      stats->device_ms += one.device_ms;
      stats->kernel_launches += one.kernel_launches;
    }
    uint32_t *dev = nullptr;
    status = ws(g, slot[b], g->V, &dev);
    if (status != GG_OK) break;
    e = cudaEventRecord(done[b], g->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(cs, done[b], 0);
    if (e == cudaSuccess && parents[i])
      e = cudaMemcpyAsync(parents[i], dev, sizeof(uint32_t) * g->V, cudaMemcpyDeviceToHost, cs);
    if (e == cudaSuccess) e = cudaEventRecord(copied[b], cs);
    if (e != cudaSuccess) status = cuda_status(e, "pipeline copy");
  }
  if (cs) {
    const cudaError_t e2 = cudaStreamSynchronize(cs);
    if (status == GG_OK && e2 != cudaSuccess) status = cuda_status(e2, "pipeline copy");
    cudaStreamDestroy(cs);
  }
  for (int b = 0; b < 2; b++) {
    if (done[b]) cudaEventDestroy(done[b]);
    if (copied[b]) cudaEventDestroy(copied[b]);
  }
  return status;
}

int gg_pagerank(gg_graph *g, int iterations, double *ranks, double *deltas, gg_run_stats *stats) {
  if (!g) {
    set_error("null graph");
    return GG_ERR_INVALID;
  }
  return pr_run<double>(g, iterations, ranks, deltas, stats);
}

int gg_pagerank_f32(gg_graph *g, int iterations, float *ranks, double *deltas, gg_run_stats *stats) {
  if (!g) {
    set_error("null graph");
    return GG_ERR_INVALID;
  }
  return pr_run<float>(g, iterations, ranks, deltas, stats);
}

int gg_active_edges(gg_graph *g, const uint64_t *active_bitmap, uint64_t *active_edges) {
  if (!g || !active_bitmap || !active_edges) {
    set_error("null argument");
    return GG_ERR_INVALID;
  }
  GG_CUDA(cudaSetDevice(g->device));
  Trace range(nullptr, g, "process_vertices");
  size_t words = bitmap_words32(g->V);
  uint32_t *bm;
  GG_TRY(ws(g, WS_BM3, words, &bm));
  GG_CUDA(cudaMemcpyAsync(bm, active_bitmap, words * 4, cudaMemcpyHostToDevice, g->stream));
  GG_TRY(counters_reset(g));
  active_edges_kernel<<<grid_for(words, 256, g->num_sms), 256, 0, g->stream>>>(bm, words, g->out.deg, g->V,
                                                                              g->ws.ctr);
  GG_CUDA(cudaGetLastError());
  Counters c;
  GG_TRY(counters_read(g, &c));
  *active_edges = c.edges;
  return GG_OK;
}

}  // extern "C"
