// Host C++ face of the GB300 engine with the reference's Graph<EdgeData> names
// (core/graph.hpp:91-1869), core types (core/type.hpp:22-68) and bitmaps
// (core/bitmap.hpp:20-61).  Compiled by any C++11 compiler; all device work
// goes through the C ABI in gemini_gb300.h (libgemini_gb300.so), so no CUDA
// type appears here.
//
// Differences from the reference, by design:
//  * one partition on one GPU: partition_id is 0, partitions is 1, and
//    gather_vertex_array is a no-op;
//  * the five toolkits run on the GPU inside the library (bfs(), pagerank(),
//    cc(), sssp(), bc() below); a std::function lambda cannot run on the
//    device, so user-written process_edges / process_vertices loops use the
//    device-lambda engine of gemini/engine.cuh (compiled with nvcc) on the
//    same Graph;
//  * errors throw gemini::Error instead of assert()/exit(-1).
#ifndef GEMINI_GB300_GRAPH_HPP
#define GEMINI_GB300_GRAPH_HPP

#include <stdint.h>
#include <string.h>

#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "gemini_gb300.h"

struct Empty {};
typedef uint32_t VertexId;
typedef uint64_t EdgeId;

#if defined(__CUDACC__)
#define GEMINI_HD __host__ __device__
#else
#define GEMINI_HD
#endif

// One adjacency entry and one vertex's adjacency list in the reference's
// layout (core/type.hpp:44-68): neighbour id, then the edge data, packed; an
// unweighted entry is the bare 4-byte id.  The list form of
// gemini::Engine::process_edges (gemini/engine.cuh) hands callbacks these.
template <typename EdgeData>
struct AdjUnit {
  VertexId neighbour;
  EdgeData edge_data;
} __attribute__((packed));

template <>
struct AdjUnit<Empty> {
  union {
    VertexId neighbour;
    Empty edge_data;
  };
} __attribute__((packed));

template <typename EdgeData>
struct VertexAdjList {
  AdjUnit<EdgeData> *begin;
  AdjUnit<EdgeData> *end;
  GEMINI_HD VertexAdjList() : begin(nullptr), end(nullptr) {}
  GEMINI_HD VertexAdjList(AdjUnit<EdgeData> *b, AdjUnit<EdgeData> *e) : begin(b), end(e) {}
};

#define WORD_OFFSET(i) ((i) >> 6)
#define BIT_OFFSET(i) ((i) & 0x3f)

// core/bitmap.hpp: 64-bit words, bit i%64 of word i/64, size/64+1 words.
class Bitmap {
 public:
  size_t size;
  unsigned long *data;
  Bitmap() : size(0), data(nullptr) {}
  explicit Bitmap(size_t n) : size(n), data(new unsigned long[WORD_OFFSET(n) + 1]) { clear(); }
  ~Bitmap() { delete[] data; }
  Bitmap(const Bitmap &) = delete;
  Bitmap &operator=(const Bitmap &) = delete;
  void clear() { memset(data, 0, sizeof(unsigned long) * (WORD_OFFSET(size) + 1)); }
  void fill() {
    const size_t words = WORD_OFFSET(size);
    for (size_t i = 0; i < words; i++) data[i] = ~0ul;
    data[words] = 0;
    for (size_t i = words << 6; i < size; i++) data[words] |= 1ul << BIT_OFFSET(i);
  }
  unsigned long get_bit(size_t i) const { return data[WORD_OFFSET(i)] & (1ul << BIT_OFFSET(i)); }
  void set_bit(size_t i) { __atomic_fetch_or(data + WORD_OFFSET(i), 1ul << BIT_OFFSET(i), __ATOMIC_RELAXED); }
};
typedef Bitmap VertexSubset;

namespace gemini {

class Error : public std::runtime_error {
 public:
  Error(int code, const std::string &what) : std::runtime_error(what), code(code) {}
  int code;
};

inline void check(int rc, const char *what) {
  if (rc != GG_OK) throw Error(rc, std::string(what) + ": " + gg_last_error());
}

}  // namespace gemini

template <typename EdgeData = Empty>
class Graph {
 public:
  int partition_id = 0;
  int partitions = 1;
  bool symmetric = false;
  VertexId vertices = 0;
  EdgeId edges = 0;
  VertexId *out_degree = nullptr;  // host copies, filled by the loaders
  VertexId *in_degree = nullptr;

  explicit Graph(int device = 0) : device_(device) {
    static_assert(std::is_same<EdgeData, Empty>::value || std::is_same<EdgeData, float>::value,
                  "edge data is Empty or float (the reference toolkits' two cases)");
  }
  ~Graph() {
    if (g_) gg_graph_free(g_);
    delete[] out_degree;
    if (in_degree != out_degree) delete[] in_degree;
  }
  Graph(const Graph &) = delete;
  Graph &operator=(const Graph &) = delete;

  // core/graph.hpp:772.  opt (may be null): device-memory budget of the build,
  // partitioned build, adjacency in host memory (gg_build_options).
  void load_directed(std::string path, VertexId n, gg_build_options *opt = nullptr) { load(path, n, false, opt); }
  // core/graph.hpp:350
  void load_undirected_from_directed(std::string path, VertexId n, gg_build_options *opt = nullptr) {
    load(path, n, true, opt);
  }

  // core/graph.hpp:760
  void transpose() {
    gemini::check(gg_graph_transpose(g_), "transpose");
    std::swap(out_degree, in_degree);
  }

  // core/graph.hpp:229-251: vertex arrays live in pinned host memory.
  template <typename T>
  T *alloc_vertex_array() {
    void *p = nullptr;
    gemini::check(gg_host_alloc(sizeof(T) * vertices, &p), "alloc_vertex_array");
    return (T *)p;
  }
  template <typename T>
  void dealloc_vertex_array(T *array) {
    gg_host_free(array);
  }
  template <typename T>
  void fill_vertex_array(T *array, T value) {
    for (VertexId v = 0; v < vertices; v++) array[v] = value;
  }
  // core/graph.hpp:253-307: the array's bytes in a file (host or device array)
  template <typename T>
  void dump_vertex_array(T *array, std::string path) {
    gemini::check(gg_dump_vertex_array(array, sizeof(T), vertices, path.c_str()), "dump_vertex_array");
  }
  template <typename T>
  void restore_vertex_array(T *array, std::string path) {
    gemini::check(gg_restore_vertex_array(array, sizeof(T), vertices, path.c_str()), "restore_vertex_array");
  }
  // core/graph.hpp:327
  VertexSubset *alloc_vertex_subset() { return new VertexSubset(vertices); }
  // core/graph.hpp:311: one partition holds every vertex already.
  template <typename T>
  void gather_vertex_array(T *, int) {}

  // The process_vertices reduction process_edges starts with
  // (core/graph.hpp:1503-1508), and its switch (:1509).
  EdgeId active_edges(VertexSubset *active) {
    uint64_t ae = 0;
    gemini::check(gg_active_edges(g_, (const uint64_t *)active->data, &ae), "active_edges");
    return ae;
  }
  bool sparse(EdgeId active_edges_value) const { return gg_is_sparse(active_edges_value, edges) != 0; }

  // The toolkits' compute() loops, on the GPU (toolkits/*.cpp).
  void bfs(VertexId root, VertexId *parent, gg_run_stats *st = nullptr) {
    gemini::check(gg_bfs(g_, root, parent, st), "bfs");
  }
  void pagerank(int iterations, double *ranks, double *deltas = nullptr, gg_run_stats *st = nullptr) {
    gemini::check(gg_pagerank(g_, iterations, ranks, deltas, st), "pagerank");
  }
  void cc(VertexId *label, gg_run_stats *st = nullptr) { gemini::check(gg_cc(g_, label, st), "cc"); }
  void sssp(VertexId root, float *distance, gg_run_stats *st = nullptr) {
    gemini::check(gg_sssp(g_, root, distance, st), "sssp");
  }
  void bc(VertexId root, double *dependencies, double *inv_num_paths, gg_run_stats *st = nullptr) {
    gemini::check(gg_bc(g_, root, dependencies, inv_num_paths, st), "bc");
  }

  gg_graph *handle() const { return g_; }

 private:
  void load(const std::string &path, VertexId n, bool sym, gg_build_options *opt) {
    const int weighted = std::is_same<EdgeData, float>::value ? 1 : 0;
    gemini::check(gg_graph_load_ex(path.c_str(), n, weighted, sym ? 1 : 0, device_, opt, &g_), "load");
    gg_graph_info info;
    gemini::check(gg_graph_info_get(g_, &info), "info");
    vertices = info.vertices;
    edges = info.edges;
    symmetric = sym;
    out_degree = new VertexId[vertices];
    gemini::check(gg_graph_adjacency(g_, 0, nullptr, nullptr, nullptr, out_degree), "out_degree");
    if (sym) {
      in_degree = out_degree;
    } else {
      in_degree = new VertexId[vertices];
      gemini::check(gg_graph_adjacency(g_, 1, nullptr, nullptr, nullptr, in_degree), "in_degree");
    }
  }
  int device_;
  gg_graph *g_ = nullptr;
};

// Per-call trace buffers for gg_run_stats (the reference prints only the
// active counts, under its own loop).
struct TraceBuffers {
  std::vector<int32_t> mode;
  std::vector<uint64_t> active_edges, activated;
  gg_run_stats stats;
  explicit TraceBuffers(int capacity = 1 << 16) : mode(capacity), active_edges(capacity), activated(capacity) {
    memset(&stats, 0, sizeof(stats));
    stats.trace_capacity = capacity;
    stats.mode = mode.data();
    stats.active_edges = active_edges.data();
    stats.activated = activated.data();
  }
};

#endif
