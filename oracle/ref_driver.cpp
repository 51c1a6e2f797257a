// TEST INFRASTRUCTURE: drives one reference toolkit's own compute() over
// several arguments (roots, or iteration counts) on a graph loaded once by
// the reference's own loader, so that the CPU baseline times the reference
// code itself without reloading the graph per root.
//
// The toolkit source (toolkits/<app>.cpp of the reference, staged under
// oracle/_ref/src by build_ref.sh) is included with its main() renamed; the
// rest -- Graph, load_directed / load_undirected_from_directed,
// process_edges, compute() -- is the reference's, unmodified.  Each compute()
// prints its own exec_time line; this driver adds `load_time=` and, before
// each run, `run_arg=`.  The BFS driver also prints `teps_edges=` after each
// run: the sum of out_degree over the vertices the run reached, which equals
// the sum of active_edges over its process_edges calls (core/graph.hpp:
// 1503-1508; every reached vertex is active in exactly one call), read from
// the parent array as compute() frees it, outside its timed region.
//
// Build (build_ref.sh): g++ -O3 -fopenmp -march=native -DGG_APP_<APP>
//   -I oracle/shim -I oracle/_ref/src oracle/ref_driver.cpp
//
// Usage: ref_<app> <edge file> <vertices> <arg> [<arg> ...]
#include <stdio.h>
#include <stdlib.h>

#define main gemini_reference_toolkit_main
#if defined(GG_APP_BFS)
#include "toolkits/bfs.cpp"
typedef Graph<Empty> DriverGraph;
#elif defined(GG_APP_SSSP)
#include "toolkits/sssp.cpp"
typedef Graph<Weight> DriverGraph;
#elif defined(GG_APP_PAGERANK)
#include "toolkits/pagerank.cpp"
typedef Graph<Empty> DriverGraph;
#elif defined(GG_APP_CC)
#include "toolkits/cc.cpp"
typedef Graph<Empty> DriverGraph;
#elif defined(GG_APP_BC)
#include "toolkits/bc.cpp"
typedef Graph<Empty> DriverGraph;
#else
#error "define one of GG_APP_BFS, GG_APP_SSSP, GG_APP_PAGERANK, GG_APP_CC, GG_APP_BC"
#endif
#undef main

#if defined(GG_APP_BFS)
static DriverGraph *observed_graph = nullptr;
static bool observe_next_parent = false;
static unsigned long long teps_edges = 0;

// compute() frees exactly one vertex array, its parent array
// (toolkits/bfs.cpp:104), through dealloc_vertex_array -> numa_free.
static void count_reached_edges(const void *start, size_t size) {
  if (!observe_next_parent || size != sizeof(VertexId) * (size_t)observed_graph->vertices) return;
  const VertexId *parent = (const VertexId *)start;
  const VertexId V = observed_graph->vertices;
  const VertexId *deg = observed_graph->out_degree;
  unsigned long long sum = 0;
#pragma omp parallel for reduction(+ : sum) schedule(static)
  for (VertexId v = 0; v < V; v++)
    if (parent[v] < V) sum += deg[v];
  teps_edges = sum;
  observe_next_parent = false;
}
#endif

int main(int argc, char **argv) {
  MPI_Instance mpi(&argc, &argv);
  if (argc < 4) {
    fprintf(stderr, "usage: %s <edge file> <vertices> <arg> [<arg> ...]\n", argv[0]);
    return 2;
  }
  DriverGraph *graph = new DriverGraph();
  double t0 = get_time();
#if defined(GG_APP_CC)
  graph->load_undirected_from_directed(argv[1], std::atoi(argv[2]));
#else
  graph->load_directed(argv[1], std::atoi(argv[2]));
#endif
  printf("load_time=%lf(s)\n", get_time() - t0);
#if defined(GG_APP_BFS)
  observed_graph = graph;
  gg_shim_free_observer = count_reached_edges;
#endif
  for (int i = 3; i < argc; i++) {
    printf("run_arg=%s\n", argv[i]);
    fflush(stdout);
#if defined(GG_APP_CC)
    compute(graph);
#elif defined(GG_APP_PAGERANK)
    compute(graph, std::atoi(argv[i]));
#elif defined(GG_APP_BFS)
    observe_next_parent = true;
    compute(graph, (VertexId)std::atoi(argv[i]));
    printf("teps_edges=%llu\n", teps_edges);
#else
    compute(graph, (VertexId)std::atoi(argv[i]));
#endif
    fflush(stdout);
  }
  return 0;
}
