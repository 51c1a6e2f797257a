// Lane pools: up to 64 independent traversals ("lanes") of one graph that
// advance together, one iteration at a time, on their own CUDA stream.  New
// roots are admitted into free lanes between iterations and finished lanes
// are retired between iterations, so a pool serves a stream of queries with
// continuous batching (the serving loop) as well as one batch of roots
// (gg_bfs_batched / gg_sssp_batched).
#ifndef GG_LANES_CUH
#define GG_LANES_CUH

#include <stddef.h>

#include "gg_common.cuh"

namespace gg {

constexpr int POOL_LANES = 64;

struct LaneCounters {
  unsigned long long alive;  // OR of the lanes that activated something this iteration
  unsigned long long edges;  // sum of out_degree over the vertices touched this iteration
  unsigned int touched;
  unsigned int qlen;
  unsigned int lpos;         // level-list entries appended this iteration (pull steps)
  unsigned int pad;
};

// Level lists (batched BFS without parents): one 16-byte entry per vertex
// and iteration in which the vertex gained lanes -- x vertex, y iteration,
// z / w the low / high half of the lane mask gained.  A lane's level at v is
// the entry's iteration less the lane's start; the lists hold every lane's
// levels in place of the 256-byte per-vertex level rows.
typedef uint4 LevelEntry;
// Bucketed SSSP filter results, after the LaneCounters in the same buffer.
struct BucketCounters {
  unsigned long long expand;  // lanes with a vertex below its threshold
  unsigned int minp[64];      // per lane, the least waiting distance (float bits)
};
constexpr size_t BUCKET_OFFSET = 64;

// Device-driven steps: the pool's traversal state in device memory, so that
// one CUDA-graph launch runs many steps.  A loop node repeats one step's
// subgraph; its first kernel picks push or pull from the counters of the last
// step and switches the branches on, its last kernel advances this state and
// ends the loop when no lane is left (or after `cap` steps, when the host
// reads the per-step rows and launches again).
constexpr int MS_ROWS = 1024;
enum MsRowBits { MS_ROW_DENSE = 1, MS_ROW_BUILD = 2, MS_ROW_CLEAR = 4, MS_ROW_PUSH = 8, MS_ROW_PUSH_THREAD = 16 };
struct MsState {
  unsigned long long *front, *next;  // lane masks of this step's frontier / of the lanes it reaches
  uint32_t *qa, *qb;                 // queue of the frontier / of the vertices this step reaches
  unsigned long long active;         // lanes still traversing
  unsigned long long ae;             // out-edges of the union frontier
  uint32_t nq, iter, qvalid, next_clear;
  uint32_t steps, cap, mode, pad;    // mode: MsRowBits of the running step
  // one row per step: mode bits, union frontier out-edges, vertices reached
  unsigned long long row_ae[MS_ROWS];
  uint32_t row_mode[MS_ROWS];
  uint32_t row_reached[MS_ROWS];
};
constexpr size_t MS_HEADER = offsetof(MsState, row_ae);

class LanePool {
 public:
  enum Kind { BFS = 0, SSSP = 1 };
  LanePool(gg_graph *g, Kind kind, bool parents) : g_(g), kind_(kind), parents_(parents) {}
  ~LanePool() { close(); }
  // Device bytes open() allocates for this graph and kind.
  static size_t bytes_needed(const gg_graph *g, Kind kind, bool parents);
  int open();  // allocates the pool's buffers and stream
  void close();
  bool is_open() const { return open_; }
  Kind kind() const { return kind_; }
  gg_graph *graph() const { return g_; }
  cudaStream_t stream() const { return s_; }

  unsigned long long used() const { return used_; }      // lanes holding a query
  unsigned long long active() const { return active_; }  // lanes still traversing
  unsigned long long done() const { return used_ & ~active_; }
  // Puts roots[i] into lane lanes[i] (free lanes); takes effect for the next step().
  int admit(const uint32_t *roots, const int *lanes, int n);
  // One iteration of every active lane; lanes whose frontier empties become done.
  int step();
  // Steps until no lane is active.  Device-driven (one CUDA-graph launch per
  // MS_ROWS steps, no host wait between steps) when the graph asks for it
  // (gg_graph_set_batched_graph) and no per-step kernel time is asked for.
  int run(bool per_step_timing);
  // Per-lane results of the lanes in mask (arrays indexed by lane):
  // reached vertices, a checksum of the lane's result array (see
  // gg_result_checksum in the header), and the single-root TEPS numerator (BFS).
  int digest(unsigned long long mask, unsigned long long *reached, unsigned long long *checksum,
             unsigned long long *edges);
  // Lane-major result arrays of the lanes in mask, in ascending lane order,
  // into device buffers (BFS: levels, parents; SSSP: distances in levels_f).
  int extract(unsigned long long mask, int32_t *levels, uint32_t *parents, float *dist);
  void retire(unsigned long long mask) { used_ &= ~mask; }
  // Level lists instead of level rows for the traversals admitted while the
  // pool is empty (BFS without parents; takes effect at that admission).
  void set_level_lists(bool on) { want_lists_ = on; }
  int calls() const { return calls_; }
  bool parents() const { return parents_; }
  void set_trace(struct Trace *tr) { tr_ = tr; }
  int launches = 0;

 private:
  int read_counters(LaneCounters *h);
  int run_device_steps();
  int list_room(size_t more);
  int lists_to_rows();
  int build_step_graph();
  void destroy_step_graph();
  bool step_graph_current() const;
  int build_queue();
  // the kernels of one step's parts; G: launched into the step graph, their
  // arguments read from st_ on the device; n counts the launches
  template <bool G> int queue_kernels(int *n);
  template <bool G> int pull_kernels(int *n);
  template <bool G> int push_kernels(bool per_thread, int *n);
  template <bool G> int push_tail(int *n);
  int bfs_step();
  int sssp_step();
  int sssp_bucket_step();
  gg_graph *g_;
  Kind kind_;
  bool parents_;
  bool open_ = false;
  cudaStream_t s_ = nullptr;
  // device buffers
  unsigned long long *visit_ = nullptr, *front_ = nullptr, *next_ = nullptr;
  uint32_t *lvl_ = nullptr, *par_ = nullptr;
  float *dist_ = nullptr;
  // bucketed SSSP (graph->sssp_delta > 0, no negative weights): lanes lowered
  // but not yet expanded, and each lane's distance threshold
  unsigned long long *pend_ = nullptr;
  float *thr_dev_ = nullptr;
  float thr_[64] = {};
  float delta_ = 0.0f;
  bool bucket_ = false;
  uint32_t *q_[2] = {nullptr, nullptr};
  unsigned long long *prefix_ = nullptr, *scan64_ = nullptr;
  uint32_t *qpos_ = nullptr, *scan32_ = nullptr;
  uint32_t *roots_dev_ = nullptr, *start_dev_ = nullptr;
  int *lanes_dev_ = nullptr;
  LaneCounters *mc_ = nullptr, *mc_host_ = nullptr;
  unsigned long long *out_dev_ = nullptr, *out_host_ = nullptr;  // 3 x 64 digest values
  // BFS without parents: per lane, vertices reached and their out-degree sum,
  // kept up to date by the level pass of every step (2 x 64)
  unsigned long long *lane_sum_ = nullptr;
  // host state
  unsigned long long used_ = 0, active_ = 0;
  unsigned long long ae_ = 0;
  uint32_t nq_ = 0;
  bool qvalid_ = false, next_clear_ = false;
  int cur_ = 0;
  uint32_t iter_ = 0;
  uint32_t start_[POOL_LANES] = {};
  int calls_ = 0;
  struct Trace *tr_ = nullptr;
  // level lists: entries in use, capacity, on for the traversals now running
  LevelEntry *list_ = nullptr;
  size_t list_n_ = 0, list_cap_ = 0;
  bool list_mode_ = false, want_lists_ = false;
  // device-driven steps
  MsState *st_ = nullptr, *st_host_ = nullptr;
  cudaGraph_t step_graph_ = nullptr;
  cudaGraphExec_t step_exec_ = nullptr;
  Dir key_in_, key_out_;  // the adjacency (and bins) the step graph was built for
  uint32_t key_div_ = 0, key_tl_ = 0;
  // kernel launches of each part of a step (control, pull, queue build,
  // clear, push, thread push, push epilogue)
  int n_ctl_ = 0, n_dense_ = 0, n_build_ = 0, n_clear_ = 0, n_push_ = 0, n_push_t_ = 0, n_tail_ = 0;
};

}  // namespace gg

#endif
