/*
 * gemini_gb300.h -- C ABI of the GB300-native Gemini edge-processing engine.
 *
 * One graph lives on one GPU.  Every call is synchronous with respect to the
 * host: when it returns, results requested into host memory are there.
 * Status codes replace the reference's assert()/exit(-1); nothing in the
 * library aborts the process.
 *
 * Each entry point names the reference interface it replaces
 * (core/graph.hpp, toolkits/*.cpp of shugo256/GeminiGraph).  Vertex ids are
 * uint32 (VertexId, core/type.hpp:24), edge counts uint64 (EdgeId,
 * core/type.hpp:25).  Input records are the reference's binary edge list
 * (EdgeUnit, core/type.hpp:27-41): packed {uint32 src, uint32 dst} (8 B) or
 * {uint32 src, uint32 dst, float weight} (12 B); a trailing partial record
 * is ignored, as core/graph.hpp:782 does.
 *
 * Thread safety: calls on different graphs may run from different host
 * threads; calls on one graph must be serialised by the caller.
 */
#ifndef GEMINI_GB300_H
#define GEMINI_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define GG_OK 0
#define GG_ERR_INVALID 1      /* bad argument (null pointer, root >= vertices, ...) */
#define GG_ERR_IO 2           /* file missing or unreadable */
#define GG_ERR_RANGE 3        /* an edge names a vertex id >= vertices */
#define GG_ERR_CUDA 4         /* CUDA runtime error (no device, launch failure) */
#define GG_ERR_NOMEM 5        /* device or pinned host allocation failed */
#define GG_ERR_UNWEIGHTED 6   /* the operation needs edge weights */
#define GG_ERR_TOO_LARGE 7    /* adjacency entries per direction >= 2^32 */
#define GG_ERR_LIMIT 8        /* a fixed capacity of the call was exceeded */
#define GG_ERR_CHECK 9        /* a device bounds check failed (libgemini_gb300_check.so only) */

typedef struct gg_graph gg_graph;

/* Mirrors the public fields of Graph<EdgeData> (core/graph.hpp:94-111). */
typedef struct {
  uint32_t vertices;         /* |V| */
  uint64_t edges;            /* file records: `edges` of the sparse/dense switch */
  uint64_t adj_entries;      /* adjacency entries per direction (2*edges if symmetric) */
  int32_t weighted;          /* 1: float edge data (EdgeData = float) */
  int32_t symmetric;         /* 1: loaded by load_undirected_from_directed */
  int32_t transposed;        /* 1: after an odd number of gg_graph_transpose calls */
  int32_t device;            /* CUDA device ordinal */
  uint64_t device_bytes;     /* device memory held by the graph and its workspace */
  uint64_t host_bytes;       /* pinned host memory holding the adjacency (adjacency_host) */
} gg_graph_info;

/* Per-call record of a traversal: one row per process_edges call. */
typedef struct {
  int32_t trace_capacity;    /* in: rows the arrays below can take (0 = no trace) */
  int32_t calls;             /* out: process_edges calls made */
  int32_t *mode;             /* in/out: per call, 0 = sparse (push), 1 = dense (pull) */
  uint64_t *active_edges;    /* in/out: per call, the switch value (graph.hpp:1503-1508) */
  uint64_t *activated;       /* in/out: per call, vertices the slots activated */
  double *call_ms;           /* in/out (may be NULL): per call, device time of the call's
                                edge kernel (push or pull), CUDA events on the graph's stream */
  uint64_t active_edges_total; /* out: sum of active_edges over all calls (TEPS numerator) */
  double device_ms;          /* out: device time of the traversal (CUDA events) */
  int32_t kernel_launches;   /* out: kernels this call launched */
} gg_run_stats;

/* Last error message of the calling thread ("" when none). */
const char *gg_last_error(void);

/* core/graph.hpp:253-307 (dump_vertex_array / restore_vertex_array) with one
 * partition: the file holds the vertices x elem_size bytes of the array,
 * vertex 0 first.  array may be host or device memory.  Restoring from a
 * file of another length returns GG_ERR_INVALID (the reference asserts). */
int gg_dump_vertex_array(const void *array, uint64_t elem_size, uint32_t vertices, const char *path);
int gg_restore_vertex_array(void *array, uint64_t elem_size, uint32_t vertices, const char *path);

/* Pinned (page-locked) host memory for inputs and results: the
 * alloc_vertex_array of the host side (core/graph.hpp:229-237). */
int gg_host_alloc(uint64_t bytes, void **out);
int gg_host_free(void *p);

/* ---- graph store ---- */

/* Graph::load_directed (core/graph.hpp:772) when symmetric == 0,
 * Graph::load_undirected_from_directed (core/graph.hpp:350) when 1.
 * Reads the edge-list file, builds CSR (out) and CSC (in) on the device. */
int gg_graph_load(const char *path, uint32_t vertices, int weighted, int symmetric,
                  int device, gg_graph **out);

/* As gg_graph_load, from records already in host memory. */
int gg_graph_from_records(const void *records, uint64_t bytes, uint32_t vertices,
                          int weighted, int symmetric, int device, gg_graph **out);

/* As gg_graph_load, from records already in device memory (not modified). */
int gg_graph_from_device_records(const void *d_records, uint64_t bytes, uint32_t vertices,
                                 int weighted, int symmetric, int device, gg_graph **out);

/* Options of the graph build (core/graph.hpp:805-821 streams the edge file in
 * CHUNKSIZE pieces so that the whole list is never resident at once; this is
 * the device-memory form of that bound).  The in-core build holds the records
 * and two sort buffers on the device (about 3x the adjacency).  When that
 * working set exceeds the budget, the partitioned build leaves the records in
 * host memory (pinned, or registered for the duration of the call; the
 * kernels read them over NVLink-C2C) and builds each direction in ranges of
 * its major ids, holding one range's sort buffers at a time.  Both builds
 * give identical adjacency (same neighbour and weight order).
 * adjacency_host = 1 keeps the neighbour and weight arrays in mapped pinned
 * host memory, read by every kernel over NVLink-C2C, for graphs larger than
 * free device memory; PageRank then pulls the plain incoming adjacency (its
 * renumbered device copy is off unless gg_graph_set_pr_layout asks for it). */
typedef struct {
  uint64_t build_budget;     /* in: device bytes the build may hold beyond the graph;
                                0 = free device memory less the graph and a reserve */
  int32_t adjacency_host;    /* in: 1 = neighbour / weight arrays in host memory */
  int32_t force_partitions;  /* in: 1..256 = partitioned build, ranges of at most
                                ceil(entries / force_partitions) entries (a longer
                                list is a range of its own); 0 = by budget */
  uint32_t partitions;       /* out: ranges per direction (1 = in-core build) */
  uint32_t record_passes;    /* out: passes over the records, all directions (partitioned:
                                degrees, range counts, one per group of ranges) */
  double build_ms;           /* out: wall time of the call */
} gg_build_options;

/* gg_graph_load / gg_graph_from_records with build options (opt may be NULL:
 * automatic budget, adjacency in device memory).  The plain calls choose the
 * build the same way. */
int gg_graph_load_ex(const char *path, uint32_t vertices, int weighted, int symmetric, int device,
                     gg_build_options *opt, gg_graph **out);
int gg_graph_from_records_ex(const void *records, uint64_t bytes, uint32_t vertices, int weighted,
                             int symmetric, int device, gg_build_options *opt, gg_graph **out);

/* Builds a graph from a seeded R-MAT (a=.57 b=.19 c=.19 d=.05) or grid edge list
 * generated on the device; identical to loading the file gg_generate_* writes.
 * kind 0 = R-MAT (p1 = scale, p2 = edge factor), 1 = grid (p1 = side, p2 unused). */
int gg_graph_generate(int kind, uint32_t p1, uint32_t p2, uint64_t seed, int weighted,
                      int symmetric, int device, gg_graph **out);

/* gg_graph_generate with build options (the records are generated in device
 * memory; opt may be NULL). */
int gg_graph_generate_ex(int kind, uint32_t p1, uint32_t p2, uint64_t seed, int weighted, int symmetric,
                         int device, gg_build_options *opt, gg_graph **out);

/* Host generator of the same records (records = edge count * 8 or 12 bytes). */
uint64_t gg_generate_count(int kind, uint32_t p1, uint32_t p2);
int gg_generate_records(int kind, uint32_t p1, uint32_t p2, uint64_t seed, int weighted,
                        void *records, int threads);

/* ~Graph: frees all device memory of the graph. */
int gg_graph_free(gg_graph *g);

int gg_graph_info_get(const gg_graph *g, gg_graph_info *info);

/* Graph::transpose (core/graph.hpp:760): swaps the two directions. */
int gg_graph_transpose(gg_graph *g);

/* Copies one direction to host memory (incoming != 0: CSC).  Any pointer may be
 * NULL.  offsets: vertices+1 entries; neighbours/weights: adj_entries entries;
 * degree: vertices entries (out_degree / in_degree, core/graph.hpp:110-111). */
int gg_graph_adjacency(const gg_graph *g, int incoming, uint64_t *offsets, uint32_t *neighbours,
                       float *weights, uint32_t *degree);

/* Device view of one direction of the graph, for kernels compiled outside
 * the library (the process_edges / process_vertices templates of
 * gemini/engine.cuh).  Plain device pointers owned by the graph, valid until
 * gg_graph_free; incoming = 1 gives the CSC (in-lists), 0 the CSR, as
 * swapped by gg_graph_transpose.  Replaces the reference's direct access to
 * the partition's adjacency (outgoing_adj_*, incoming_adj_*,
 * core/graph.hpp:121-140). */
typedef struct {
  const uint64_t *offsets;     /* vertices + 1 */
  const uint32_t *neighbours;  /* entries */
  const float *weights;        /* entries; NULL when unweighted */
  const uint32_t *degree;      /* vertices */
  uint32_t vertices;
  uint64_t entries;
  uint64_t edges;              /* edge records: the |E| of the sparse/dense switch */
  int32_t device;
} gg_device_adj;
int gg_graph_device_view(const gg_graph *g, int incoming, gg_device_adj *out);

/* ---- toolkits (the compute() of toolkits/*.cpp, on one GPU) ----
 * Output pointers are host memory; NULL leaves the result on the device
 * (see gg_result_device_ptr).  stats may be NULL. */

/* toolkits/bfs.cpp:22-109: parent array; parent[v] == vertices if unreached. */
int gg_bfs(gg_graph *g, uint32_t root, uint32_t *parent, gg_run_stats *stats);

/* toolkits/pagerank.cpp:26-129: double ranks after `iterations` iterations;
 * deltas (may be NULL) receives the `iterations` values printed as delta(i). */
/* n single-root BFS runs (each exactly gg_bfs) back to back, the parent tree
 * of run i copied to parents[i] (host memory, V entries; NULL skips it) on a
 * second stream while run i + 1 computes, from two alternating device
 * buffers.  With page-locked host memory (gg_host_alloc) the copies hide
 * behind the next run: the runs' own small readbacks go through the SMs
 * into mapped memory, so they never queue behind a result copy.
 * stats: calls, active_edges_total, device_ms and kernel_launches summed over
 * the runs (no per-call rows).  No reference counterpart: the reference's
 * bfs main() runs compute() six times in a row (toolkits/bfs.cpp:111-139). */
int gg_bfs_many(gg_graph *g, const uint32_t *roots, int n, uint32_t *const *parents, gg_run_stats *stats);
int gg_pagerank(gg_graph *g, int iterations, double *ranks, double *deltas, gg_run_stats *stats);

/* As gg_pagerank in float arithmetic (float ranks, float sums). */
int gg_pagerank_f32(gg_graph *g, int iterations, float *ranks, double *deltas, gg_run_stats *stats);

/* toolkits/cc.cpp:22-88 on a symmetric graph: min-label of every vertex. */
int gg_cc(gg_graph *g, uint32_t *label, gg_run_stats *stats);

/* toolkits/sssp.cpp:24-90 on a weighted graph: float distances, 1e9 if unreached. */
int gg_sssp(gg_graph *g, uint32_t root, float *distance, gg_run_stats *stats);

/* toolkits/bc.cpp:24-196 (compute): dependencies and inv_num_paths (1/path count;
 * inf for unreached vertices, whose dependency is NaN as in the reference). */
int gg_bc(gg_graph *g, uint32_t root, double *dependencies, double *inv_num_paths,
          gg_run_stats *stats);

/* ---- batched multi-source traversals (no counterpart in the reference) ----
 * Up to 64 roots ("lanes") in one traversal; lane i's result equals gg_bfs /
 * gg_sssp run alone on roots[i].  Results are lane-major host arrays
 * (nroots * vertices entries, lane i at offset i * vertices); any may be NULL. */

/* BFS: levels[i*V + v] = hop count from roots[i] (-1 if unreached); parents[i*V + v]
 * = a BFS-tree parent (vertices if unreached); reached[i] = vertices reached;
 * lane_edges[i] = the sum of active_edges a single-root run of roots[i] counts. */
int gg_bfs_batched(gg_graph *g, const uint32_t *roots, int nroots, int32_t *levels, uint32_t *parents,
                   uint64_t *reached, uint64_t *lane_edges, gg_run_stats *stats);

/* SSSP on a weighted graph: distances[i*V + v] (1e9 if unreached), bit-identical
 * to gg_sssp(g, roots[i]); reached[i] = vertices with distance < 1e9. */
int gg_sssp_batched(gg_graph *g, const uint32_t *roots, int nroots, float *distances, uint64_t *reached,
                    gg_run_stats *stats);

/* Sparse/dense switch of the batched BFS steps: a step pulls when the union
 * frontier's out-edges reach edges / divisor (0 = 20, the reference's rule,
 * core/graph.hpp:1509).  Levels and reached counts do not depend on it. */
int gg_graph_set_batched_switch(gg_graph *g, uint32_t divisor);

/* Batched SSSP relaxation order (no reference counterpart): delta > 0
 * expands each lane's lowered vertices in rising distance buckets of this
 * width; 0 (the default) runs plain Bellman-Ford rounds, which on R-MAT
 * graphs is faster (scale 24, 64 roots: 640 ms against 800-1100 ms for widths
 * 0.4-0.02: all lanes share every round's adjacency scan, while buckets
 * desynchronise the lanes).  Graphs with a negative weight always run rounds.
 * Distances do not depend on it.  Takes effect when a lane pool of the graph
 * next starts from empty. */
int gg_graph_set_sssp_delta(gg_graph *g, float delta);

/* Batched SSSP (gg_sssp_batched and the serving pools; no reference
 * counterpart): a step with at most `lanes` traversals in flight relaxes each
 * edge in one thread, looping over the source's lanes, instead of one warp
 * per edge covering all 64 lanes.  0 always uses the warp form.  Distances
 * do not depend on it.  Default 16 (measured: with 16 lanes the thread form
 * is faster at R-MAT 20-26, with 64 the warp form). */
int gg_graph_set_batched_thread_lanes(gg_graph *g, uint32_t lanes);

/* Batched BFS and SSSP without buckets (gg_bfs_batched, gg_sssp_batched; no
 * reference counterpart): on, the steps of a batch run device-driven -- one
 * CUDA-graph launch whose loop node repeats a step, the step's push or pull
 * picked on the device by the same rule, so the host waits once per batch
 * (per 1024 steps) instead of once per step.  Off (default): one host wait
 * per step.  Results and per-step traces do not depend on it.  Measured on
 * GB300 the host-driven steps are the faster: 64-root batches of R-MAT 24 BFS
 * 6.79 against 6.86 ms, SSSP 618 against 636 ms, 1024 x 1024 grid BFS 108.5
 * against 110.4 ms, 8192 x 8192 grid BFS 3.49 against 3.92 s (the step
 * graph's kernels take their lengths from device memory, so its scans and
 * pushes launch over the largest grid).  A call that asks for per-call
 * kernel times (gg_run_stats.call_ms) always runs its steps from the host. */
int gg_graph_set_batched_graph(gg_graph *g, int on);

/* gg_bfs_batched without parents (no reference counterpart): on (default)
 * the lanes' levels are kept as level lists -- one 16-byte entry (vertex,
 * step, lanes gained) per vertex and step that reached it, appended by the
 * step's kernels -- and the per-lane levels, reached counts and TEPS
 * numerators are read from them; off: as 256-byte rows of 64 levels per
 * vertex, written as lanes reach it.  A list past 16 entries per vertex
 * moves into the rows and the batch goes on with rows.  Results do not
 * depend on it. */
int gg_graph_set_batched_lists(gg_graph *g, int on);

/* Batched betweenness centrality (no reference counterpart; per lane the
 * computation of toolkits/bc.cpp:24-196): up to 64 roots in one pass per
 * level.  dependencies and inv_num_paths (either may be NULL) receive
 * nroots x vertices doubles, lane-major (root i at [i * vertices]): the
 * reference's printed dependencies and 1 / num_paths, NaN / inf where the
 * root does not reach; reached[i] = vertices root i reaches.  Device memory:
 * 2 x 64 x 8 bytes per vertex plus 8 bytes per vertex per BFS level.
 * Dependencies equal the single-root gg_bc's within summation rounding. */
int gg_bc_batched(gg_graph *g, const uint32_t *roots, int nroots, double *dependencies, double *inv_num_paths,
                  uint64_t *reached, gg_run_stats *stats);

/* Checksum of one traversal result, as the serving loop reports it: the sum
 * (mod 2^64) over reached vertices v of mix64(v * 0x9E3779B97F4A7C15 + x), where
 * x is the hop count (kind 0: int32 levels, -1 = unreached) or the float bits
 * of the distance (kind 1: float distances, >= 1e9 = unreached) and mix64 is
 * the SplitMix64 finaliser. */
uint64_t gg_result_checksum(const void *values, uint32_t vertices, int kind);

/* Hop count of every vertex in a BFS parent array (-1 if unreached); host code. */
int gg_levels_from_parents(const uint32_t *parent, uint32_t vertices, uint32_t root, int32_t *levels);

/* ---- serving loop (no counterpart in the reference) ----
 * Resident graphs answer BFS (kind 0) and SSSP (kind 1) queries with
 * continuous batching: every (graph, kind) has a pool of 64 lanes on its own
 * stream and worker thread; queries join free lanes between iterations and
 * leave when their traversal ends, so queries of different graphs and kinds
 * overlap on the device.  A pool is opened only if its buffers fit the budget
 * and the device's free memory; its queries wait otherwise.  Each result
 * carries the query's reached count and gg_result_checksum of its result
 * array, identical to a single-root gg_bfs / gg_sssp run of the same root. */
typedef struct gg_server gg_server;

typedef struct {
  uint64_t ticket;
  int32_t graph;
  int32_t kind;
  uint32_t root;
  int32_t status;
  uint64_t reached;
  uint64_t checksum;
  uint64_t active_edges;     /* BFS: the single-root TEPS numerator */
  double latency_ms;         /* submit to completion, host clock */
} gg_query_result;

typedef struct {
  uint64_t completed, pending, pools_open, pools_opened, pools_closed, admission_waits;
  uint64_t bytes_in_use, budget;
  int32_t max_busy_pools;    /* most pools running at once */
  int32_t max_lanes_in_use;  /* most queries on the device at once */
  uint64_t solo_runs;        /* SSSP queries run alone (gg_server_set_solo) */
} gg_server_stats;

/* Device bytes one pool of kind (0 BFS, 1 SSSP) on g holds while open. */
uint64_t gg_pool_bytes(const gg_graph *g, int kind);
/* hbm_budget: device bytes the pools may hold (0 = free memory less 2 GiB). */
int gg_server_create(int device, uint64_t hbm_budget, gg_server **out);
/* The graph must outlive the server; calls on it must not overlap serving. */
/* Batch window of the pools of one kind (0 BFS, 1 SSSP): a pool with no
 * traversal running and fewer waiting queries than free lanes holds them up
 * to window_ms after the oldest one arrived, so that more queries start in
 * the same steps.  0 (the default) starts them at once.  Results do not
 * depend on it; latency does. */
int gg_server_set_window(gg_server *s, int kind, double window_ms);
/* An SSSP pool with no traversal running and fewer than `below` waiting
 * queries runs them one at a time through the single-root SSSP (gg_sssp, on
 * the graph's own stream) instead of starting a batch: a batched SSSP step
 * costs nearly as much with a few lanes as with 64, so small batches are
 * slower than single-root runs (R-MAT 26: 257 ms for one lane against 75 ms
 * alone; batches pass single-root runs near 20 lanes).  0 always batches.
 * Default 16.  While a server runs, only it may call single-root toolkits on
 * its graphs. */
int gg_server_set_solo(gg_server *s, int below);
int gg_server_add_graph(gg_server *s, gg_graph *g, int *graph_id);
int gg_server_submit(gg_server *s, int graph_id, int kind, uint32_t root, uint64_t *ticket);
/* Up to max_results completed queries; waits up to timeout_ms for the first. */
int gg_server_wait(gg_server *s, gg_query_result *out, int max_results, int timeout_ms, int *n);
int gg_server_stats_get(gg_server *s, gg_server_stats *stats);
int gg_server_free(gg_server *s);

/* Device address of the last result of a toolkit kept on the device:
 * which = 0 primary output (parent / ranks / label / distance / dependencies),
 * 1 secondary (inv_num_paths).  Valid until the next toolkit call on g. */
const void *gg_result_device_ptr(const gg_graph *g, int which);

/* ---- autotuner (no counterpart in the reference; Graph::tune_chunks,
 * core/graph.hpp:1341-1404, balances threads by edge counts at load) ----
 * The pull kernels split vertices into light lists (<= light_deg entries, one
 * lane each) and longer lists cut into pull_chunk-edge warp work items, whose
 * lanes load 16-byte windows of the list (pull_vector bit 0 set) or every
 * 32nd entry (clear); pull_vector bit 1 makes the reduction pulls' light
 * lanes read their lists by aligned 32-byte windows (two 16-byte loads per
 * eight entries) instead of one entry per load.  gg_graph_set_bins sets all
 * three (light_deg 1..2048; pull_chunk 128, 256 or 512; pull_vector 0..3).  gg_autotune times the
 * 36 candidates (light_deg 16 to 512) on the graph itself with CUDA events, on the workloads the
 * objective mask names (GG_TUNE_PAGERANK: four float PageRank iterations;
 * GG_TUNE_BFS: one BFS; GG_TUNE_BATCHED: one 64-root gg_bfs_batched, and
 * gg_sssp_batched on a weighted graph; GG_TUNE_SSSP / GG_TUNE_CC / GG_TUNE_BC:
 * one SSSP / CC / BC run; GG_TUNE_PAGERANK64: four double PageRank
 * iterations), keeps the fastest, then times on top of it, for objectives
 * with reduction pulls (all but BFS and batched), the light windows at the
 * chosen bound and, where they win, at twice it, the PageRank L1 policy
 * (PageRank objectives) and the pull split, and records the result in
 * <cache_dir>/bins_v5.txt (cache_dir NULL: $GG_TUNE_CACHE, else
 * ~/.cache/geminigraph_gb300) under a fingerprint of the graph and the
 * objective; a later call on the same graph reads the cache instead of
 * searching.  Traversal results (BFS, CC, SSSP) do not depend on the bins;
 * PageRank and BC sums may differ in the last bits. */
typedef struct {
  uint32_t light_deg;
  uint32_t pull_chunk;
  uint32_t pull_vector;
  double best_ms;        /* timing workload with the chosen bins */
  double default_ms;     /* the same with the defaults (32, 256, 1) */
  int32_t candidates;    /* candidates timed (0 when read from the cache) */
  int32_t from_cache;
  uint32_t l1_hot_bytes; /* the pulls' L1 policy kept (gg_graph_set_l1_hot; PageRank
                            objective: every gather cached, or the hottest 160 KiB) */
  uint32_t pull_split;   /* the pulls' light kernel blocks per SM beside the chunk kernel
                            (gg_graph_set_pull_split; objectives with reduction pulls:
                            0, or 4 where it is faster) */
  uint32_t bfs_pull;     /* gg_bfs's pull divisor in effect (gg_graph_set_bfs_pull; not
                            tuned: an earlier pull wins on some roots and loses on others) */
} gg_tune_result;

int gg_graph_set_bins(gg_graph *g, uint32_t light_deg, uint32_t pull_chunk, uint32_t pull_vector);

#define GG_TUNE_PAGERANK 1u
#define GG_TUNE_BFS 2u
#define GG_TUNE_BATCHED 4u
#define GG_TUNE_SSSP 8u    /* one SSSP from the vertex of largest out-degree (weighted graphs) */
#define GG_TUNE_CC 16u     /* one CC (symmetric graphs) */
#define GG_TUNE_PAGERANK64 32u /* four double PageRank iterations */
#define GG_TUNE_BC 64u     /* one BC from the vertex of largest out-degree */
int gg_autotune(gg_graph *g, uint32_t objective, const char *cache_dir, gg_tune_result *out);

/* PageRank's adjacency layout (no reference counterpart; the reference pulls
 * its CSC as loaded).  hot_sources = 1 (the default): on its first call
 * gg_pagerank / gg_pagerank_f32 build, and keep with the graph, a copy of the
 * incoming adjacency with vertices renumbered by descending out-degree and
 * each in-list sorted by the new numbers; the iterations run there and the
 * ranks are mapped back to vertex order.  Sums then run in that order, so
 * ranks differ from the plain layout's in the last bits only.  hot_sources =
 * 0 frees the copy and pulls the plain incoming adjacency.  The copy is
 * dropped by gg_graph_transpose and counted in device_bytes.  gg_cc on a
 * symmetric graph uses the same copy, and gg_sssp and gg_bc use it together
 * with the outgoing adjacency in the same numbering (built on their first
 * call on a directed graph), weights carried along: labels and distances are
 * identical either way, BC dependencies equal up to summation order. */
int gg_graph_set_pr_layout(gg_graph *g, int hot_sources);

/* Cache policy of the reduction pulls on that layout (no reference
 * counterpart: the reference's gathers go through the CPU caches).  The
 * gathered state of the first l1_bytes worth of sources -- the most gathered
 * ones -- is cached in each SM's L1, and every other gather is read past L1 so
 * that it does not evict them.  0 reads every gather past L1; a value at least
 * the whole state array caches every gather (the plain layout always does).
 * Results do not depend on it.  Default: every gather cached (measured
 * fastest on R-MAT 24 and 26, where the other gathers reuse L1 lines too). */
int gg_graph_set_l1_hot(gg_graph *g, uint32_t l1_bytes);

/* Kernel choice for the dense calls of gg_cc and gg_sssp (no reference
 * counterpart; the reference's dense mode pulls every in-list,
 * core/graph.hpp:1664-1855).  A call that the reference's switch makes dense
 * runs as a push over the frontier when its active out-edges are below
 * adjacency entries / divisor; 0 always pulls.  A source that is not active
 * cannot lower a neighbour's label or distance, so both forms give the same
 * values, the same activated set and the same per-call trace (which records
 * the reference's mode).  Default 4 (measured on R-MAT 25 SSSP: 131 -> 145
 * GTEPS; CC on R-MAT 26 unchanged). */
int gg_graph_set_dense_push(gg_graph *g, uint32_t divisor);

/* Kernel choice of gg_bfs / gg_bfs_many (the reference's dense mode is the
 * pull, core/graph.hpp:1503-1509): a call runs the pull kernels when its
 * active out-edges are at least edges / divisor and the push kernels
 * otherwise (default 20, the reference's own switch).  Any in-neighbour on
 * the frontier is a valid parent, so levels, the tree's validity and the
 * per-call trace (which records the reference's mode) do not depend on it. */
int gg_graph_set_bfs_pull(gg_graph *g, uint32_t divisor);

/* Reduction pulls (PageRank, CC, SSSP, BC backward) whose light-list and
 * chunk kernels run side by side on two streams (no reference counterpart):
 * light_blocks in 1..7 launches the light kernel over light_blocks blocks per
 * SM and the chunk kernel over the other 8 - light_blocks, so both are
 * resident on every SM from the start; 0 (default) launches each over the
 * whole GPU, so the chunk kernel's blocks start as the light kernel's retire.
 * Results do not depend on it. */
int gg_graph_set_pull_split(gg_graph *g, uint32_t light_blocks);

/* ---- engine primitives ---- */

/* Graph::process_vertices (core/graph.hpp:1406-1469) for the reduction
 * process_edges makes first: sum of out_degree over the set bits of a host
 * bitmap in the reference's layout (core/bitmap.hpp: 64-bit words,
 * vertices/64 + 1 of them). */
int gg_active_edges(gg_graph *g, const uint64_t *active_bitmap, uint64_t *active_edges);

/* No counterpart in the reference.  gg_active_edges for callers that cannot
 * let a library allocate device memory: a serving process that reserves all of
 * HBM for its own pool at start-up, or a latency-critical caller that cannot
 * take the device synchronisation of cudaMalloc/cudaFree.  All pointers are
 * device memory the caller provides: d_bitmap (vertices/64+1 64-bit words, the
 * reference's bitmap layout), d_degree (vertices out-degrees), d_active_edges
 * (one uint64 that receives the sum).  stream is a cudaStream_t, or NULL for
 * the default stream; the call returns once that stream has finished.  It
 * runs on the calling thread's current device.
 * It allocates nothing: its only scratch is a fixed 32 KiB device array inside
 * the library (one partial sum per 65,536 vertices), so it accepts at most
 * GG_NOALLOC_MAX_VERTICES vertices and returns GG_ERR_LIMIT beyond.  The first
 * call on a device looks up that array's device address (cudaGetSymbolAddress)
 * and keeps it for the life of the process: make that first call before any
 * stream capture, and do not reset the device (cudaDeviceReset) after it.
 * All calls share the array,
 * which keeps the last call's partial sums; calls that overlap on the GPU race. */
#define GG_NOALLOC_MAX_VERTICES 268435456u
int gg_active_edges_noalloc(const uint64_t *d_bitmap, const uint32_t *d_degree, uint32_t vertices,
                            uint64_t *d_active_edges, void *stream);

/* The sparse/dense switch of process_edges (core/graph.hpp:1509). */
int gg_is_sparse(uint64_t active_edges, uint64_t edges);

#ifdef __cplusplus
}
#endif

#endif
