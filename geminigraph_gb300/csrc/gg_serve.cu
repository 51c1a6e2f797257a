// Serving loop: resident graphs, BFS/SSSP queries with continuous batching.
//
// No counterpart in the reference (its toolkits run one root per process).
// Each (graph, kind) has a lane pool (gg_lanes.cuh) driven by its own worker
// thread on its own CUDA stream, so pools of different graphs or kinds run
// concurrently on the device.  A worker admits waiting queries into free
// lanes between iterations, runs one iteration of all its lanes, and retires
// the lanes whose frontier emptied, reporting each query's reached count and
// result checksum (gg_result_checksum).  An idle pool may hold its first
// queries for a batch window so that more start together (gg_server_set_window).
// A pool is opened only when its
// buffers fit in the server's HBM budget and in the device's free memory;
// otherwise its queries wait until an idle pool closes and frees memory.
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

#include "gg_gen.h"
#include "gg_lanes.cuh"

namespace gg {

// Reached count and gg_result_checksum (kind 1) of one distance array.
__global__ void solo_digest(const float *__restrict__ dist, uint32_t V, unsigned long long *out) {
  unsigned long long c = 0, h = 0;
  for (size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (size_t)gridDim.x * blockDim.x) {
    const float d = dist[v];
    if (d < 1e9f) {
      c += 1;
      h += gg_mix64((unsigned long long)v * 0x9E3779B97F4A7C15ull + __float_as_uint(d));
    }
  }
  c = warp_sum(c);
  h = warp_sum(h);
  if (lane_id() == 0) {
    atomicAdd(out, c);
    atomicAdd(out + 1, h);
  }
}

static double now_ms() {
  using namespace std::chrono;
  return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

struct Query {
  uint64_t ticket;
  int graph, kind;
  uint32_t root;
  double t_submit;
};

struct PoolSlot {
  LanePool *pool = nullptr;
  size_t bytes = 0;
  unsigned long long *solo_out = nullptr;  // device: reached, checksum of a solo run
  std::deque<Query> pending;
  Query lane_q[POOL_LANES];
  std::thread worker;
  bool started = false;
};

}  // namespace gg

using namespace gg;

struct gg_server {
  int device = 0;
  uint64_t budget = 0, used = 0;
  uint64_t reserve = 2ull << 30;  // device memory left free for the graphs' own calls
  double idle_close_ms = 200.0;
  // batch window per kind: an idle pool waits up to this long after its
  // oldest waiting query for more queries to start with it (0: start at once)
  double window_ms[2] = {0.0, 0.0};
  // an idle SSSP pool with fewer waiting queries than this runs them one at
  // a time through the single-root SSSP (0: always batch)
  int sssp_solo_below = 16;
  std::vector<gg_graph *> graphs;
  std::map<std::pair<int, int>, PoolSlot *> pools;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<gg_query_result> done;
  uint64_t next_ticket = 1;
  bool stop = false;
  int error = GG_OK;
  // statistics
  uint64_t completed = 0, pools_opened = 0, pools_closed = 0, admission_waits = 0, solo_runs = 0;
  int busy_pools = 0, max_busy_pools = 0, max_lanes_in_use = 0, lanes_in_use = 0;
};

// One query through the single-root SSSP (gg_sssp) on the graph's own
// stream; its distances are digested on the device.  Only this pool's worker
// calls single-root code on the graph while the server runs.
static int solo_sssp(gg_server *S, gg_graph *g, PoolSlot *slot, const Query &q) {
  if (!slot->solo_out) GG_CUDA(cudaMalloc(&slot->solo_out, 2 * sizeof(unsigned long long)));
  gg_run_stats st;
  memset(&st, 0, sizeof(st));
  GG_TRY(gg_sssp(g, q.root, nullptr, &st));
  GG_CUDA(cudaMemsetAsync(slot->solo_out, 0, 2 * sizeof(unsigned long long), g->stream));
  solo_digest<<<grid_for(g->V, 256, g->num_sms, 8), 256, 0, g->stream>>>((const float *)g->result[0], g->V,
                                                                         slot->solo_out);
  unsigned long long h[2];
  GG_CUDA(cudaMemcpyAsync(h, slot->solo_out, sizeof(h), cudaMemcpyDeviceToHost, g->stream));
  GG_CUDA(cudaStreamSynchronize(g->stream));
  gg_query_result r;
  r.ticket = q.ticket;
  r.graph = q.graph;
  r.kind = q.kind;
  r.root = q.root;
  r.status = GG_OK;
  r.reached = h[0];
  r.checksum = h[1];
  r.active_edges = 0;
  r.latency_ms = now_ms() - q.t_submit;
  std::lock_guard<std::mutex> lk(S->mu);
  S->done.push_back(r);
  S->completed += 1;
  S->solo_runs += 1;
  S->cv_done.notify_all();
  return GG_OK;
}

static void worker_loop(gg_server *S, std::pair<int, int> key, PoolSlot *slot) {
  cudaSetDevice(S->device);
  gg_graph *g = S->graphs[key.first];
  const LanePool::Kind kind = (LanePool::Kind)key.second;
  double idle_since = now_ms();
  bool counted_busy = false;
  for (;;) {
    std::vector<Query> take;
    {
      std::unique_lock<std::mutex> lk(S->mu);
      for (;;) {
        if (S->stop) break;
        const bool has_work = !slot->pending.empty() || (slot->pool && slot->pool->active());
        if (has_work) break;
        // idle: close the pool after a while so its memory can serve others
        if (slot->pool && slot->pool->is_open() && now_ms() - idle_since > S->idle_close_ms) {
          slot->pool->close();
          S->used -= slot->bytes;
          S->pools_closed += 1;
          S->cv_work.notify_all();
        }
        if (counted_busy) {
          S->busy_pools -= 1;
          counted_busy = false;
        }
        S->cv_work.wait_for(lk, std::chrono::milliseconds(20));
      }
      if (S->stop) break;
      if (!counted_busy) {
        S->busy_pools += 1;
        counted_busy = true;
        if (S->busy_pools > S->max_busy_pools) S->max_busy_pools = S->busy_pools;
      }
      // solo: too few SSSP queries for a batch to beat single-root runs
      if (kind == LanePool::SSSP && !slot->pool->active() && !slot->pending.empty() &&
          (int)slot->pending.size() < S->sssp_solo_below) {
        const Query q = slot->pending.front();
        slot->pending.pop_front();
        lk.unlock();
        int st = solo_sssp(S, g, slot, q);
        lk.lock();
        if (st != GG_OK) {
          S->error = st;
          S->stop = true;
          S->cv_done.notify_all();
          break;
        }
        idle_since = now_ms();
        continue;
      }
      // admission: the pool's buffers must fit the budget and the free memory
      if (!slot->pool->is_open()) {
        size_t free_b = 0, total_b = 0;
        cudaMemGetInfo(&free_b, &total_b);
        if (S->used + slot->bytes > S->budget || free_b < slot->bytes + S->reserve) {
          S->admission_waits += 1;
          S->cv_work.wait_for(lk, std::chrono::milliseconds(5));
          continue;
        }
        S->used += slot->bytes;
        lk.unlock();
        int st = slot->pool->open();
        lk.lock();
        if (st != GG_OK) {
          S->used -= slot->bytes;
          S->admission_waits += 1;
          continue;
        }
        S->pools_opened += 1;
      }
      const unsigned long long free_lanes = ~slot->pool->used();
      int nfree = __builtin_popcountll(free_lanes);
      // batch window: an idle pool that cannot fill its lanes yet waits for
      // more queries, until the oldest has waited window_ms
      const double win = S->window_ms[key.second];
      if (win > 0.0 && !slot->pool->active() && !slot->pending.empty() && (int)slot->pending.size() < nfree) {
        const double left = slot->pending.front().t_submit + win - now_ms();
        if (left > 0.0) {
          S->cv_work.wait_for(lk, std::chrono::microseconds((long long)(left * 1000.0) + 1));
          continue;
        }
      }
      while (nfree > 0 && !slot->pending.empty()) {
        take.push_back(slot->pending.front());
        slot->pending.pop_front();
        nfree--;
      }
    }
    LanePool *p = slot->pool;
    if (!take.empty()) {
      uint32_t roots[POOL_LANES];
      int lanes[POOL_LANES];
      unsigned long long free_lanes = ~p->used();
      for (size_t i = 0; i < take.size(); i++) {
        const int l = __builtin_ctzll(free_lanes);
        free_lanes &= free_lanes - 1;
        lanes[i] = l;
        roots[i] = take[i].root;
        slot->lane_q[l] = take[i];
      }
      if (p->admit(roots, lanes, (int)take.size()) != GG_OK) {
        std::lock_guard<std::mutex> lk(S->mu);
        S->error = GG_ERR_CUDA;
        S->stop = true;
        S->cv_done.notify_all();
        break;
      }
      std::lock_guard<std::mutex> lk(S->mu);
      S->lanes_in_use += (int)take.size();
      if (S->lanes_in_use > S->max_lanes_in_use) S->max_lanes_in_use = S->lanes_in_use;
    }
    int st = p->step();
    const unsigned long long fin = p->done();
    unsigned long long reached[POOL_LANES], checksum[POOL_LANES], edges[POOL_LANES];
    if (st == GG_OK && fin) st = p->digest(fin, reached, checksum, edges);
    if (st != GG_OK) {
      std::lock_guard<std::mutex> lk(S->mu);
      S->error = st;
      S->stop = true;
      S->cv_done.notify_all();
      break;
    }
    if (fin) {
      p->retire(fin);
      const double t = now_ms();
      std::lock_guard<std::mutex> lk(S->mu);
      for (int l = 0; l < POOL_LANES; l++) {
        if (!((fin >> l) & 1ull)) continue;
        const Query &q = slot->lane_q[l];
        gg_query_result r;
        r.ticket = q.ticket;
        r.graph = q.graph;
        r.kind = q.kind;
        r.root = q.root;
        r.status = GG_OK;
        r.reached = reached[l];
        r.checksum = checksum[l];
        r.active_edges = kind == LanePool::BFS ? edges[l] : 0;
        r.latency_ms = t - q.t_submit;
        S->done.push_back(r);
        S->completed += 1;
        S->lanes_in_use -= 1;
      }
      S->cv_done.notify_all();
    }
    if (!p->active()) idle_since = now_ms();
  }
  std::lock_guard<std::mutex> lk(S->mu);
  if (counted_busy) S->busy_pools -= 1;
}

extern "C" {

int gg_server_create(int device, uint64_t hbm_budget, gg_server **out) {
  if (!out) {
    set_error("null argument");
    return GG_ERR_INVALID;
  }
  GG_CUDA(cudaSetDevice(device));
  size_t free_b = 0, total_b = 0;
  GG_CUDA(cudaMemGetInfo(&free_b, &total_b));
  gg_server *S = new gg_server();
  S->device = device;
  S->budget = hbm_budget ? hbm_budget : (free_b > S->reserve ? free_b - S->reserve : 0);
  *out = S;
  return GG_OK;
}

int gg_server_set_solo(gg_server *S, int below) {
  if (!S || below < 0 || below > POOL_LANES) {
    set_error("need a server and 0..64 queries");
    return GG_ERR_INVALID;
  }
  std::lock_guard<std::mutex> lk(S->mu);
  S->sssp_solo_below = below;
  return GG_OK;
}

int gg_server_set_window(gg_server *S, int kind, double window_ms) {
  if (!S || (kind != 0 && kind != 1) || !(window_ms >= 0.0)) {
    set_error("need a server, kind 0 (BFS) or 1 (SSSP) and a window >= 0");
    return GG_ERR_INVALID;
  }
  std::lock_guard<std::mutex> lk(S->mu);
  S->window_ms[kind] = window_ms;
  return GG_OK;
}

int gg_server_add_graph(gg_server *S, gg_graph *g, int *graph_id) {
  if (!S || !g || !graph_id) {
    set_error("null argument");
    return GG_ERR_INVALID;
  }
  if (g->device != S->device) {
    set_error("graph is on device %d, server on %d", g->device, S->device);
    return GG_ERR_INVALID;
  }
  std::lock_guard<std::mutex> lk(S->mu);
  S->graphs.push_back(g);
  *graph_id = (int)S->graphs.size() - 1;
  return GG_OK;
}

int gg_server_submit(gg_server *S, int graph_id, int kind, uint32_t root, uint64_t *ticket) {
  if (!S) {
    set_error("null server");
    return GG_ERR_INVALID;
  }
  std::lock_guard<std::mutex> lk(S->mu);
  if (S->error != GG_OK) {
    set_error("server stopped after an error");
    return S->error;
  }
  if (graph_id < 0 || graph_id >= (int)S->graphs.size() || (kind != 0 && kind != 1)) {
    set_error("bad graph id or kind");
    return GG_ERR_INVALID;
  }
  gg_graph *g = S->graphs[graph_id];
  if (root >= g->V) {
    set_error("root %u >= vertices %u", root, g->V);
    return GG_ERR_INVALID;
  }
  if (kind == 1 && !g->weighted) {
    set_error("sssp needs a weighted graph");
    return GG_ERR_UNWEIGHTED;
  }
  const std::pair<int, int> key(graph_id, kind);
  PoolSlot *&slot = S->pools[key];
  if (!slot) {
    slot = new PoolSlot();
    slot->pool = new LanePool(g, (LanePool::Kind)kind, false);
    slot->bytes = LanePool::bytes_needed(g, (LanePool::Kind)kind, false);
    if (slot->bytes > S->budget) {
      set_error("a %s pool on graph %d needs %llu bytes, over the server's budget", kind ? "SSSP" : "BFS",
                graph_id, (unsigned long long)slot->bytes);
      delete slot->pool;
      delete slot;
      S->pools.erase(key);
      return GG_ERR_NOMEM;
    }
  }
  Query q;
  q.ticket = S->next_ticket++;
  q.graph = graph_id;
  q.kind = kind;
  q.root = root;
  q.t_submit = now_ms();
  slot->pending.push_back(q);
  if (!slot->started) {
    slot->started = true;
    slot->worker = std::thread(worker_loop, S, key, slot);
  }
  if (ticket) *ticket = q.ticket;
  S->cv_work.notify_all();
  return GG_OK;
}

int gg_server_wait(gg_server *S, gg_query_result *out, int max_results, int timeout_ms, int *n) {
  if (!S || !out || !n || max_results < 1) {
    set_error("null argument");
    return GG_ERR_INVALID;
  }
  std::unique_lock<std::mutex> lk(S->mu);
  if (S->done.empty() && S->error == GG_OK)
    S->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms < 0 ? 0 : timeout_ms),
                        [&] { return !S->done.empty() || S->error != GG_OK; });
  int k = 0;
  while (k < max_results && !S->done.empty()) {
    out[k++] = S->done.front();
    S->done.pop_front();
  }
  *n = k;
  if (S->error != GG_OK) {
    set_error("server stopped after an error");
    return S->error;
  }
  return GG_OK;
}

int gg_server_stats_get(gg_server *S, gg_server_stats *st) {
  if (!S || !st) {
    set_error("null argument");
    return GG_ERR_INVALID;
  }
  std::lock_guard<std::mutex> lk(S->mu);
  st->completed = S->completed;
  st->pending = 0;
  st->pools_open = 0;
  for (auto &kv : S->pools) {
    st->pending += kv.second->pending.size();
    if (kv.second->pool && kv.second->pool->is_open()) st->pools_open += 1;
  }
  st->pools_opened = S->pools_opened;
  st->pools_closed = S->pools_closed;
  st->admission_waits = S->admission_waits;
  st->bytes_in_use = S->used;
  st->budget = S->budget;
  st->max_busy_pools = S->max_busy_pools;
  st->max_lanes_in_use = S->max_lanes_in_use;
  st->solo_runs = S->solo_runs;
  return GG_OK;
}

int gg_server_free(gg_server *S) {
  if (!S) return GG_OK;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stop = true;
  }
  S->cv_work.notify_all();
  for (auto &kv : S->pools)
    if (kv.second->started) kv.second->worker.join();
  for (auto &kv : S->pools) {
    if (kv.second->solo_out) cudaFree(kv.second->solo_out);
    delete kv.second->pool;
    delete kv.second;
  }
  delete S;
  return GG_OK;
}

uint64_t gg_pool_bytes(const gg_graph *g, int kind) {
  if (!g || (kind != 0 && kind != 1)) return 0;
  return LanePool::bytes_needed(g, (LanePool::Kind)kind, false);
}

int gg_levels_from_parents(const uint32_t *parent, uint32_t vertices, uint32_t root, int32_t *levels) {
  if (!parent || !levels || root >= vertices) {
    set_error("bad argument");
    return GG_ERR_INVALID;
  }
  for (uint32_t v = 0; v < vertices; v++) levels[v] = -2;  // -2: not yet known
  levels[root] = 0;
  std::vector<uint32_t> path;
  for (uint32_t v = 0; v < vertices; v++) {
    if (levels[v] != -2) continue;
    path.clear();
    uint32_t u = v;
    while (levels[u] == -2) {
      if (parent[u] >= vertices) {
        levels[u] = -1;
        break;
      }
      if (path.size() > vertices) {
        set_error("parent array has a cycle");
        return GG_ERR_INVALID;
      }
      path.push_back(u);
      u = parent[u];
    }
    int32_t base = levels[u];
    for (size_t i = path.size(); i-- > 0;) {
      const uint32_t w = path[i];
      if (levels[w] != -2) {
        base = levels[w];
        continue;
      }
      levels[w] = base < 0 ? -1 : base + 1;
      base = levels[w];
    }
  }
  return GG_OK;
}

}  // extern "C"
