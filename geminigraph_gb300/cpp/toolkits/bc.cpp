// toolkits/bc.cpp command line (compute, COMPACT 0) on the GB300 engine:
// same argv, same output.
#include "common.hpp"

static void compute(Graph<Empty> *graph, VertexId root) {
  double exec_time = 0;
  exec_time -= get_time();
  double *dependencies = graph->alloc_vertex_array<double>();
  double *inv_num_paths = graph->alloc_vertex_array<double>();
  TraceBuffers tb;
  graph->bc(root, dependencies, inv_num_paths, &tb.stats);
  // forward calls run until one activates nothing; the rest are backward
  int forward = 0;
  while (forward < tb.stats.calls && tb.activated[forward] > 0) forward++;
  if (forward < tb.stats.calls) forward++;
  printf("forward\n");
  print_active(tb, forward, 1);
  printf("backward\n");
  exec_time += get_time();
  printf("exec_time=%lf(s)\n", exec_time);
  for (VertexId v = 0; v < 20 && v < graph->vertices; v++)
    printf("%lf %lf\n", dependencies[v], 1 / inv_num_paths[v]);
  graph->dealloc_vertex_array(dependencies);
  graph->dealloc_vertex_array(inv_num_paths);
}

int main(int argc, char **argv) {
  if (argc < 4) {
    printf("bc [file] [vertices] [root]\n");
    exit(-1);
  }
  return run_main([&] {
    Graph<Empty> *graph = new Graph<Empty>();
    VertexId root = std::atoi(argv[3]);
    graph->load_directed(argv[1], std::atoi(argv[2]));
    for (int run = 0; run < 6; run++) compute(graph, root);
    delete graph;
  });
}
