// CC (toolkits/cc.cpp), SSSP (toolkits/sssp.cpp) and BC (toolkits/bc.cpp,
// compute) on the device engine.
#include <vector>

#include "gg_engine.cuh"

namespace gg {

// ------------------------------------------------------------------ CC
// Sparse slot (cc.cpp:48-59): msg = label of the source at the start of the
// call (snapshot); a lower msg lowers label[dst] and activates dst.
struct CcPush {
  uint32_t *label;
  const uint32_t *msg;
  __device__ __forceinline__ bool push(uint32_t, uint32_t i, uint32_t dst, float) const {
    uint32_t m = msg[i];
    if (m < *(volatile uint32_t *)(label + dst)) {
      atomicMin(label + dst, m);
      return true;
    }
    return false;
  }
};

// Dense signal + slot (cc.cpp:60-79): msg = min(dst, labels of all
// in-neighbours); read from cur, written to nxt.
struct CcPull {
  using Acc = uint32_t;
  const uint32_t *cur;
  uint32_t *nxt;
  const uint32_t *ids = nullptr;  // hot-source layout: vertex id of each rank (the message starts at dst's id)
  uint32_t hot = 0xffffffffu;     // sources below this number are gathered through L1
  __device__ __forceinline__ bool want(uint32_t) const { return true; }
  __device__ __forceinline__ uint32_t identity(uint32_t v) const { return ids ? ids[v] : v; }
  __device__ __forceinline__ uint32_t identity_coop() const { return 0xffffffffu; }
  __device__ __forceinline__ uint32_t gather(const Dir &, unsigned long long, uint32_t u) const {
    return ld_gather(cur, u, hot);
  }
  __device__ __forceinline__ uint32_t combine(uint32_t a, uint32_t b) const { return b < a ? b : a; }
  __device__ __forceinline__ uint32_t warp_combine(uint32_t x) const { return warp_min(x); }
  __device__ __forceinline__ bool finish(uint32_t v, uint32_t m, uint32_t, Tally &) const {
    uint32_t c = cur[v];
    if (m < c) {
      nxt[v] = m;
      return true;
    }
    nxt[v] = c;
    return false;
  }
};

// ------------------------------------------------------------------ SSSP
// Lowers *p to v if v is smaller; true if this call lowered it (write_min,
// core/atomic.hpp:35-42).  Non-negative floats order like their int bits;
// negative floats order like the reverse of their unsigned bits, and any
// stored value of the other sign compares correctly in both forms.
__device__ __forceinline__ bool atomic_min_float(float *p, float v) {
  if (!(v < 0.0f)) {
    int old = atomicMin((int *)p, __float_as_int(v));
    return __int_as_float(old) > v;
  }
  unsigned old = atomicMax((unsigned *)p, __float_as_uint(v));
  return __uint_as_float(old) > v;
}

struct SsspPush {
  float *dist;
  const float *msg;
  __device__ __forceinline__ bool push(uint32_t, uint32_t i, uint32_t dst, float w) const {
    float relax = __fadd_rn(msg[i], w);
    if (relax < *(volatile float *)(dist + dst)) return atomic_min_float(dist + dst, relax);
    return false;
  }
};

// sssp.cpp:60-80: the dense signal takes the min over ALL in-edges (its
// active check is commented out, sssp.cpp:64-70); INF = 1e9.
struct SsspPull {
  using Acc = float;
  const float *cur;
  float *nxt;
  uint32_t hot = 0xffffffffu;  // sources below this number are gathered through L1
  __device__ __forceinline__ bool want(uint32_t) const { return true; }
  __device__ __forceinline__ float identity(uint32_t) const { return 1e9f; }
  __device__ __forceinline__ float identity_coop() const { return 1e9f; }
  __device__ __forceinline__ float gather(const Dir &d, unsigned long long k, uint32_t u) const {
    return __fadd_rn(ld_gather(cur, u, hot), d.w[k]);
  }
  // the same candidate with the weight read by the kernel
  __device__ __forceinline__ float gather_w(uint32_t u, float w) const { return __fadd_rn(ld_gather(cur, u, hot), w); }
  __device__ __forceinline__ float combine(float a, float b) const { return b < a ? b : a; }
  __device__ __forceinline__ float warp_combine(float x) const { return warp_min(x); }
  __device__ __forceinline__ bool finish(uint32_t v, float m, uint32_t, Tally &) const {
    float c = cur[v];
    if (m < c) {
      nxt[v] = m;
      return true;
    }
    nxt[v] = c;
    return false;
  }
};

// Runs the CC / SSSP frontier loop: both toolkits loop while the slots
// activate something, with a message snapshot for push calls and two state
// buffers for pull calls.
template <typename T, class PushOp, class PullOp>
static int relax_loop(gg_graph *g, const Dir &dout, const Dir &din, const PullOp &pull, T *state0, T *state1,
                      uint32_t *q0, uint32_t *q1, uint32_t *bm0, uint32_t *bm1, uint32_t n_act, uint32_t nq, uint32_t md,
                      bool qvalid, unsigned long long ae, Trace &tr, Launch &L, T **result) {
  const uint32_t V = g->V;
  const size_t words = bitmap_words32(V);
  cudaStream_t s = g->stream;
  Counters *ctr = g->ws.ctr;
  T *cur = state0, *nxt = state1;
  uint32_t *q[2] = {q0, q1};
  uint32_t *bm[2] = {bm0, bm1};
  T *msg;
  uint32_t *stamp;
  GG_TRY(ws(g, WS_MSG, (size_t)V + 1, &msg));
  GG_TRY(ws(g, WS_STAMP, V, &stamp));
  GG_CUDA(cudaMemsetAsync(stamp, 0, sizeof(uint32_t) * V, s));
  int c_i = 0;
  while (n_act > 0) {
    bool sparse = ae < g->E / 20;
    if (sparse && qvalid && Launch::small_ok(nq, ae, md)) {
      // consecutive small sparse calls run on the device without host round trips
      GG_TRY((L.small_run<PushOp, false, T>(dout, PushOp{cur, msg}, q, &c_i, &nq, &ae, &md, &n_act, nullptr, nullptr,
                                            cur, msg, tr, stamp)));
      continue;
    }
    tr.add(sparse ? 0 : 1, ae, 0);
    // A dense call may run as a push over the frontier: a source that is
    // not active was relaxed against its current value in the call after it
    // last changed, so it cannot lower any out-neighbour now, and the
    // minimum over the active sources' candidates is the dense call's
    // minimum over all in-edges -- the same values and the same activated
    // set (the snapshot keeps every signal before every slot).
    const bool push = sparse || (g->dense_push_div && ae < g->nadj / g->dense_push_div);
    int nx = c_i ^ 1;
    if (push && ae > 0 && !qvalid) GG_TRY(L.queue_from_bitmap(bm[c_i], dout.nz, q[c_i], &nq));
    GG_CUDA(cudaMemsetAsync(bm[nx], 0, words * 4, s));
    GG_TRY(counters_reset(g));
    ActOut a;
    a.active_out = bm[nx];
    a.q_out = push ? q[nx] : nullptr;
    a.qlen = &ctr->qlen;
    a.out_deg = dout.deg;
    a.queue_nonzero_only = true;
    if (push) {
      if (ae > 0) {
        gather_by_queue<T><<<grid_for(nq, 256, g->num_sms), 256, 0, s>>>(q[c_i], nq, cur, msg);
        unsigned long long *P;
        GG_TRY(L.scan_queue_degrees(q[c_i], nq, dout.deg, &P));
        GG_TRY(tr.kbegin());
        push_lb<PushOp><<<L.push_grid(ae), PUSH_THREADS, 0, s>>>(q[c_i], P, nq, ae, dout, PushOp{cur, msg}, a,
                                                                   ctr);
        GG_TRY(tr.kend());
        L.launches += 2;
      }
    } else {
      GG_TRY(tr.kbegin());
      PullOp op = pull;
      op.cur = cur;
      op.nxt = nxt;
      GG_TRY(L.pull(din, op, a, ctr));
      GG_TRY(tr.kend());
      T *t = cur;
      cur = nxt;
      nxt = t;
    }
    GG_CUDA(cudaGetLastError());
    Counters c;
    GG_TRY(counters_read(g, &c));
    n_act = c.activated;
    nq = c.qlen;
    md = c.maxdeg;
    qvalid = push;
    ae = c.edges;
    tr.set_activated(c.activated);
    c_i = nx;
  }
  *result = cur;
  return GG_OK;
}

// out[v] = by_rank[rank_of[v]]
template <typename T>
__global__ void unrank(const T *__restrict__ by_rank, const uint32_t *__restrict__ rank_of, uint32_t V,
                       T *__restrict__ out) {
  for (size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (size_t)gridDim.x * blockDim.x)
    out[v] = by_rank[rank_of[v]];
}

static int cc_run(gg_graph *g, uint32_t *label_host, gg_run_stats *st) {
  GG_CUDA(cudaSetDevice(g->device));
  const uint32_t V = g->V;
  const size_t words = bitmap_words32(V);
  uint32_t *lab[2], *bm[2], *q[2];
  GG_TRY(ws(g, WS_S0, V, &lab[0]));
  GG_TRY(ws(g, WS_S1, V, &lab[1]));
  GG_TRY(ws(g, WS_BM1, words, &bm[0]));
  GG_TRY(ws(g, WS_BM2, words, &bm[1]));
  GG_TRY(ws(g, WS_Q0, (size_t)V + 1, &q[0]));
  GG_TRY(ws(g, WS_Q1, (size_t)V + 1, &q[1]));
  // On a symmetric graph the hot-source layout (vertices renumbered by
  // descending degree, built once and shared with PageRank) packs the most
  // gathered labels into few cache lines.  Labels stay vertex ids, so the
  // minimum is the reference's; they map back to vertex order at the end.
  if (g->symmetric && g->pr_layout) GG_TRY(pr_layout_build(g));
  const bool ranked = g->symmetric && g->pr_layout && g->pr_ready;
  const Dir &dout = ranked ? g->pr : g->out;
  const Dir &din = ranked ? g->pr : g->in;
  uint32_t *out = nullptr;
  if (ranked) GG_TRY(ws(g, WS_S2, V, &out));
  Launch L(g);
  Trace tr(st, g, "gg_cc");
  cudaStream_t s = g->stream;
  GG_TRY(timed_begin(g));
  // label[v] = v over active_in = all (cc.cpp:31-37)
  if (ranked)
    GG_CUDA(cudaMemcpyAsync(lab[0], g->pr_id_of_rank, sizeof(uint32_t) * V, cudaMemcpyDeviceToDevice, s));
  else
    iota_u32<<<grid_for(V, 256, g->num_sms), 256, 0, s>>>(lab[0], V);
  bitmap_fill<<<grid_for(words, 256, g->num_sms), 256, 0, s>>>(bm[0], words, V);
  L.launches += ranked ? 1 : 2;
  GG_CUDA(cudaGetLastError());
  uint32_t *res = nullptr;
  CcPull pull{};
  pull.ids = ranked ? g->pr_id_of_rank : nullptr;
  pull.hot = ranked ? g->l1_hot_bytes / 4 : 0xffffffffu;
  GG_TRY((relax_loop<uint32_t, CcPush, CcPull>(g, dout, din, pull, lab[0], lab[1], q[0], q[1], bm[0], bm[1], V, 0,
                                               0xffffffffu, false, g->nadj, tr, L, &res)));
  if (ranked) {
    unrank<uint32_t><<<grid_for(V, 256, g->num_sms), 256, 0, s>>>(res, g->pr_rank_of, V, out);
    L.launches += 1;
    GG_CUDA(cudaGetLastError());
    res = out;
  }
  GG_TRY(timed_end(g, st, L.launches));
  GG_TRY(tr.collect());
  if (label_host) GG_CUDA(cudaMemcpy(label_host, res, sizeof(uint32_t) * V, cudaMemcpyDeviceToHost));
  g->result[0] = res;
  g->result[1] = nullptr;
  return GG_OK;
}

__global__ void sssp_root(float *dist, uint32_t root, uint32_t *active, uint32_t *q, const uint32_t *out_deg,
                          Counters *ctr) {
  dist[root] = 0.0f;
  active[root >> 5] |= 1u << (root & 31);
  q[0] = root;
  ctr->edges = out_deg[root];
  ctr->maxdeg = out_deg[root];
}

static int sssp_run(gg_graph *g, uint32_t root, float *dist_host, gg_run_stats *st) {
  if (!g->weighted) {
    set_error("sssp needs a weighted graph");
    return GG_ERR_UNWEIGHTED;
  }
  if (root >= g->V) {
    set_error("root %u >= vertices %u", root, g->V);
    return GG_ERR_INVALID;
  }
  GG_CUDA(cudaSetDevice(g->device));
  const uint32_t V = g->V;
  const size_t words = bitmap_words32(V);
  float *dist[2];
  uint32_t *bm[2], *q[2];
  GG_TRY(ws(g, WS_S0, V, &dist[0]));
  GG_TRY(ws(g, WS_S1, V, &dist[1]));
  GG_TRY(ws(g, WS_BM1, words, &bm[0]));
  GG_TRY(ws(g, WS_BM2, words, &bm[1]));
  GG_TRY(ws(g, WS_Q0, (size_t)V + 1, &q[0]));
  GG_TRY(ws(g, WS_Q1, (size_t)V + 1, &q[1]));
  // Hot-source layout (as PageRank's and CC's): both directions renumbered
  // by descending out-degree, weights carried along.  Every candidate
  // distance d[u] + w is the same sum, and a minimum does not depend on
  // order, so the distances are bit-identical; they map back to vertex order
  // at the end.
  if (g->pr_layout) {
    GG_TRY(pr_layout_build(g));
    if (!g->symmetric) GG_TRY(hot_out_build(g));
  }
  const bool ranked = g->pr_layout && g->pr_ready && (g->symmetric || g->pr_out_ready);
  const Dir &dout = ranked ? (g->symmetric ? g->pr : g->pr_out) : g->out;
  const Dir &din = ranked ? g->pr : g->in;
  uint32_t start = root;
  float *out = nullptr;
  if (ranked) {
    GG_CUDA(cudaMemcpy(&start, g->pr_rank_of + root, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    GG_TRY(ws(g, WS_S2, V, &out));
  }
  Launch L(g);
  Trace tr(st, g, "gg_sssp");
  cudaStream_t s = g->stream;
  GG_TRY(timed_begin(g));
  GG_CUDA(cudaMemsetAsync(bm[0], 0, words * 4, s));
  GG_TRY(counters_reset(g));
  fill_kernel<float><<<grid_for(V, 256, g->num_sms), 256, 0, s>>>(dist[0], V, 1e9f);
  sssp_root<<<1, 1, 0, s>>>(dist[0], start, bm[0], q[0], dout.deg, g->ws.ctr);
  L.launches += 2;
  GG_CUDA(cudaGetLastError());
  Counters c;
  GG_TRY(counters_read(g, &c));
  float *res = nullptr;
  SsspPull pull{};
  pull.hot = ranked ? g->l1_hot_bytes / 4 : 0xffffffffu;
  GG_TRY((relax_loop<float, SsspPush, SsspPull>(g, dout, din, pull, dist[0], dist[1], q[0], q[1], bm[0], bm[1], 1,
                                                1, c.maxdeg, true, c.edges, tr, L, &res)));
  if (ranked) {
    unrank<float><<<grid_for(V, 256, g->num_sms), 256, 0, s>>>(res, g->pr_rank_of, V, out);
    L.launches += 1;
    GG_CUDA(cudaGetLastError());
    res = out;
  }
  GG_TRY(timed_end(g, st, L.launches));
  GG_TRY(tr.collect());
  if (dist_host) GG_CUDA(cudaMemcpy(dist_host, res, sizeof(float) * V, cudaMemcpyDeviceToHost));
  g->result[0] = res;
  g->result[1] = nullptr;
  return GG_OK;
}

// ------------------------------------------------------------------ BC
// Forward sparse slot (bc.cpp:58-69): unvisited dst gains the source's path
// count; the first contribution (old value 0) activates dst.
struct BcFwdPush {
  double *np;
  const uint32_t *visited;
  __device__ __forceinline__ bool push(uint32_t src, uint32_t, uint32_t dst, float) const {
    if (bm_test(visited, dst)) return false;
    return atomicAdd(np + dst, np[src]) == 0.0;
  }
};

// Forward dense (bc.cpp:70-89): an unvisited vertex sums the path counts of
// its active in-neighbours.
struct BcFwdPull {
  using Acc = double;
  double *np;
  const uint32_t *active_in;
  const uint32_t *visited;
  __device__ __forceinline__ bool want(uint32_t v) const { return !bm_test(visited, v); }
  __device__ __forceinline__ double identity(uint32_t) const { return 0.0; }
  __device__ __forceinline__ double identity_coop() const { return 0.0; }
  __device__ __forceinline__ double gather(const Dir &, unsigned long long, uint32_t s) const {
    return bm_test_ldg(active_in, s) ? np[s] : 0.0;
  }
  __device__ __forceinline__ double combine(double a, double b) const { return a + b; }
  __device__ __forceinline__ double warp_combine(double x) const { return warp_sum(x); }
  __device__ __forceinline__ bool finish(uint32_t v, double sum, uint32_t, Tally &) const {
    if (sum > 0.0) {
      np[v] += sum;
      return true;
    }
    return false;
  }
};

// Backward sparse slot (bc.cpp:130-138) on the transposed graph.
struct BcBwdPush {
  double *dep;
  const uint32_t *visited;
  __device__ __forceinline__ bool push(uint32_t src, uint32_t, uint32_t dst, float) const {
    if (!bm_test(visited, dst)) atomicAdd(dep + dst, dep[src]);
    return false;
  }
};

// Backward dense (bc.cpp:139-155): unvisited vertices sum the dependencies
// of their in-neighbours (on the transposed graph) in the current level.
struct BcBwdPull {
  using Acc = double;
  double *dep;
  const uint32_t *level;
  const uint32_t *visited;
  __device__ __forceinline__ bool want(uint32_t v) const { return !bm_test(visited, v); }
  __device__ __forceinline__ double identity(uint32_t) const { return 0.0; }
  __device__ __forceinline__ double identity_coop() const { return 0.0; }
  __device__ __forceinline__ double gather(const Dir &, unsigned long long, uint32_t s) const {
    return bm_test_ldg(level, s) ? dep[s] : 0.0;
  }
  __device__ __forceinline__ double combine(double a, double b) const { return a + b; }
  __device__ __forceinline__ double warp_combine(double x) const { return warp_sum(x); }
  __device__ __forceinline__ bool finish(uint32_t v, double sum, uint32_t deg, Tally &) const {
    if (deg > 0) dep[v] += sum;
    return false;
  }
};

__global__ void bc_root(double *np, uint32_t root, uint32_t *visited, uint32_t *active, uint32_t *qlev,
                        const uint32_t *out_deg, const uint32_t *in_deg, Counters *ctr) {
  np[root] = 1.0;
  visited[root >> 5] |= 1u << (root & 31);
  active[root >> 5] |= 1u << (root & 31);
  qlev[0] = root;
  ctr->edges = out_deg[root];
  ctr->in_edges = in_deg[root];
}

// inv_num_paths = 1 / num_paths, dependencies = 0 (bc.cpp:103-111).
__global__ void bc_invert(double *np, double *dep, uint32_t V) {
  for (size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (size_t)gridDim.x * blockDim.x) {
    np[v] = 1.0 / np[v];
    dep[v] = 0.0;
  }
}

// process_vertices over one level: visited |= level, dep += inv (bc.cpp:113-120,157-164).
__global__ void bc_level_apply(const uint32_t *q, uint32_t n, uint32_t *visited, double *dep, const double *inv) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    uint32_t v = q[i];
    atomicOr(visited + (v >> 5), 1u << (v & 31));
    dep[v] += inv[v];
  }
}

// dependencies = (dep - inv) / inv (bc.cpp:170-176).
__global__ void bc_final(double *dep, const double *inv, uint32_t V) {
  for (size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (size_t)gridDim.x * blockDim.x)
    dep[v] = (dep[v] - inv[v]) / inv[v];
}

static int bc_run(gg_graph *g, uint32_t root, double *dep_host, double *inv_host, gg_run_stats *st) {
  if (root >= g->V) {
    set_error("root %u >= vertices %u", root, g->V);
    return GG_ERR_INVALID;
  }
  GG_CUDA(cudaSetDevice(g->device));
  const uint32_t V = g->V;
  const size_t words = bitmap_words32(V);
  double *np, *dep;
  uint32_t *visited, *bm[2], *lvbm, *qlev;
  GG_TRY(ws(g, WS_S2, V, &np));
  GG_TRY(ws(g, WS_S3, V, &dep));
  GG_TRY(ws(g, WS_BM0, words, &visited));
  GG_TRY(ws(g, WS_BM1, words, &bm[0]));
  GG_TRY(ws(g, WS_BM2, words, &bm[1]));
  GG_TRY(ws(g, WS_BM3, words, &lvbm));
  GG_TRY(ws(g, WS_QLEV, (size_t)V + 2, &qlev));
  // Hot-source layout (as SSSP's): both directions renumbered; path counts
  // are exact and dependencies change only in summation order.
  if (g->pr_layout) {
    GG_TRY(pr_layout_build(g));
    if (!g->symmetric) GG_TRY(hot_out_build(g));
  }
  const bool ranked = g->pr_layout && g->pr_ready && (g->symmetric || g->pr_out_ready);
  const Dir &dout = ranked ? (g->symmetric ? g->pr : g->pr_out) : g->out;
  const Dir &din = ranked ? g->pr : g->in;
  uint32_t start = root;
  double *dep_out = dep, *np_out = np;
  if (ranked) {
    GG_CUDA(cudaMemcpy(&start, g->pr_rank_of + root, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    GG_TRY(ws(g, WS_S0, V, &dep_out));
    GG_TRY(ws(g, WS_S1, V, &np_out));
  }
  Launch L(g);
  Trace tr(st, g, "gg_bc");
  cudaStream_t s = g->stream;
  Counters *ctr = g->ws.ctr;
  GG_TRY(timed_begin(g));
  GG_CUDA(cudaMemsetAsync(visited, 0, words * 4, s));
  GG_CUDA(cudaMemsetAsync(bm[0], 0, words * 4, s));
  GG_TRY(counters_reset(g));
  fill_kernel<double><<<grid_for(V, 256, g->num_sms), 256, 0, s>>>(np, V, 0.0);
  bc_root<<<1, 1, 0, s>>>(np, start, visited, bm[0], qlev, dout.deg, din.deg, ctr);
  L.launches += 2;
  GG_CUDA(cudaGetLastError());
  Counters c;
  GG_TRY(counters_read(g, &c));
  // level L occupies qlev[lev_off[L], lev_off[L+1]); lev_out/in = degree sums
  std::vector<uint64_t> lev_off{0, 1}, lev_out{c.edges}, lev_in{c.in_edges};
  int cur = 0;
  uint32_t n = 1;
  while (n > 0) {
    size_t L_ = lev_off.size() - 2;
    unsigned long long ae = lev_out[L_];
    bool sparse = ae < g->E / 20;
    tr.add(sparse ? 0 : 1, ae, 0);
    int nx = cur ^ 1;
    GG_CUDA(cudaMemsetAsync(bm[nx], 0, words * 4, s));
    GG_TRY(counters_reset(g));
    ActOut a;
    a.active_out = bm[nx];
    a.q_out = qlev + lev_off.back();
    a.qlen = &ctr->qlen;
    a.out_deg = dout.deg;
    a.in_deg = din.deg;
    const uint32_t *qin = qlev + lev_off[L_];
    a.q_out = sparse ? qlev + lev_off.back() : nullptr;
    if (sparse) {
      if (ae > 0) {
        unsigned long long *P;
        GG_TRY(L.scan_queue_degrees(qin, n, dout.deg, &P));
        GG_TRY(tr.kbegin());
        push_lb<BcFwdPush><<<L.push_grid(ae), PUSH_THREADS, 0, s>>>(qin, P, n, ae, dout, BcFwdPush{np, visited},
                                                                      a, ctr);
        GG_TRY(tr.kend());
        L.launches += 1;
      }
    } else {
      GG_TRY(tr.kbegin());
      GG_TRY(L.pull(din, BcFwdPull{np, bm[cur], visited}, a, ctr));
      GG_TRY(tr.kend());
    }
    GG_CUDA(cudaGetLastError());
    GG_TRY(counters_read(g, &c));
    tr.set_activated(c.activated);
    n = c.activated;
    if (!sparse && n > 0) {
      uint32_t nl = 0;
      GG_TRY(L.queue_from_bitmap(bm[nx], nullptr, qlev + lev_off.back(), &nl));
    }
    // visited |= active_out (bc.cpp:91-98)
    bitmap_or<<<grid_for(words, 256, g->num_sms), 256, 0, s>>>(visited, bm[nx], words);
    L.launches += 1;
    lev_off.push_back(lev_off.back() + n);
    lev_out.push_back(c.edges);
    lev_in.push_back(c.in_edges);
    cur = nx;
  }
  // levels 0..top; level `top` is the empty set the last forward call produced
  const int top = (int)lev_off.size() - 2;
  bc_invert<<<grid_for(V, 256, g->num_sms), 256, 0, s>>>(np, dep, V);
  GG_CUDA(cudaMemsetAsync(visited, 0, words * 4, s));
  L.launches += 1;
  // backward on the transposed graph: push over the CSC, pull over the CSR
  const Dir &tout = din, &tin = dout;
  for (int lev = top; lev >= 1; lev--) {
    uint32_t ln = (uint32_t)(lev_off[lev + 1] - lev_off[lev]);
    const uint32_t *ql = qlev + lev_off[lev];
    unsigned long long ae = lev_in[lev];
    bool sparse = ae < g->E / 20;
    tr.add(sparse ? 0 : 1, ae, 0);
    if (sparse) {
      if (ae > 0) {
        unsigned long long *P;
        GG_TRY(L.scan_queue_degrees(ql, ln, tout.deg, &P));
        GG_TRY(tr.kbegin());
        push_lb<BcBwdPush><<<L.push_grid(ae), PUSH_THREADS, 0, s>>>(ql, P, ln, ae, tout, BcBwdPush{dep, visited},
                                                                      ActOut(), ctr);
        GG_TRY(tr.kend());
        L.launches += 1;
      }
    } else {
      GG_CUDA(cudaMemsetAsync(lvbm, 0, words * 4, s));
      if (ln) bitmap_from_queue<<<grid_for(ln, 256, g->num_sms), 256, 0, s>>>(ql, ln, lvbm);
      GG_TRY(tr.kbegin());
      GG_TRY(L.pull(tin, BcBwdPull{dep, lvbm, visited}, ActOut(), ctr));
      GG_TRY(tr.kend());
      L.launches += 1;
    }
    uint32_t pn = (uint32_t)(lev_off[lev] - lev_off[lev - 1]);
    if (pn)
      bc_level_apply<<<grid_for(pn, 256, g->num_sms), 256, 0, s>>>(qlev + lev_off[lev - 1], pn, visited, dep, np);
    L.launches += 1;
    GG_CUDA(cudaGetLastError());
  }
  bc_final<<<grid_for(V, 256, g->num_sms), 256, 0, s>>>(dep, np, V);
  L.launches += 1;
  if (ranked) {
    unrank<double><<<grid_for(V, 256, g->num_sms), 256, 0, s>>>(dep, g->pr_rank_of, V, dep_out);
    unrank<double><<<grid_for(V, 256, g->num_sms), 256, 0, s>>>(np, g->pr_rank_of, V, np_out);
    L.launches += 2;
  }
  GG_CUDA(cudaGetLastError());
  GG_TRY(timed_end(g, st, L.launches));
  GG_TRY(tr.collect());
  if (dep_host) GG_CUDA(cudaMemcpy(dep_host, dep_out, sizeof(double) * V, cudaMemcpyDeviceToHost));
  if (inv_host) GG_CUDA(cudaMemcpy(inv_host, np_out, sizeof(double) * V, cudaMemcpyDeviceToHost));
  g->result[0] = dep_out;
  g->result[1] = np_out;
  return GG_OK;
}

}  // namespace gg

using namespace gg;

extern "C" {

int gg_cc(gg_graph *g, uint32_t *label, gg_run_stats *stats) {
  if (!g) {
    set_error("null graph");
    return GG_ERR_INVALID;
  }
  return cc_run(g, label, stats);
}

int gg_sssp(gg_graph *g, uint32_t root, float *distance, gg_run_stats *stats) {
  if (!g) {
    set_error("null graph");
    return GG_ERR_INVALID;
  }
  return sssp_run(g, root, distance, stats);
}

int gg_bc(gg_graph *g, uint32_t root, double *dependencies, double *inv_num_paths, gg_run_stats *stats) {
  if (!g) {
    set_error("null graph");
    return GG_ERR_INVALID;
  }
  return bc_run(g, root, dependencies, inv_num_paths, stats);
}

}  // extern "C"
