// Lane pools: up to 64 independent traversals ("lanes") of one graph that
// advance together, one iteration at a time, on their own CUDA stream.  New
// roots are admitted into free lanes between iterations and finished lanes
// are retired between iterations, so a pool serves a stream of queries with
// continuous batching (the serving loop) as well as one batch of roots
// (gg_bfs_batched / gg_sssp_batched).
#ifndef GG_LANES_CUH
#define GG_LANES_CUH

#include "gg_common.cuh"

namespace gg {

constexpr int POOL_LANES = 64;

struct LaneCounters {
  unsigned long long alive;  // OR of the lanes that activated something this iteration
  unsigned long long edges;  // sum of out_degree over the vertices touched this iteration
  unsigned int touched;
  unsigned int qlen;
};
// Bucketed SSSP filter results, after the LaneCounters in the same buffer.
struct BucketCounters {
  unsigned long long expand;  // lanes with a vertex below its threshold
  unsigned int minp[64];      // per lane, the least waiting distance (float bits)
};
constexpr size_t BUCKET_OFFSET = 64;

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
  // Per-lane results of the lanes in mask (arrays indexed by lane):
  // reached vertices, a checksum of the lane's result array (see
  // gg_result_checksum in the header), and the single-root TEPS numerator (BFS).
  int digest(unsigned long long mask, unsigned long long *reached, unsigned long long *checksum,
             unsigned long long *edges);
  // Lane-major result arrays of the lanes in mask, in ascending lane order,
  // into device buffers (BFS: levels, parents; SSSP: distances in levels_f).
  int extract(unsigned long long mask, int32_t *levels, uint32_t *parents, float *dist);
  void retire(unsigned long long mask) { used_ &= ~mask; }
  int calls() const { return calls_; }
  bool parents() const { return parents_; }
  void set_trace(struct Trace *tr) { tr_ = tr; }
  int launches = 0;

 private:
  int read_counters(LaneCounters *h);
  int build_queue();
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
};

}  // namespace gg

#endif
