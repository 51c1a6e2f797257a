// toolkits/cc.cpp command line on the GB300 engine: same argv, same output.
// The counts a sparse call prints are distinct vertices (the reference's
// count races there, counting repeated activations of one vertex).
#include "common.hpp"

static void compute(Graph<Empty> *graph) {
  double exec_time = 0;
  exec_time -= get_time();
  VertexId *label = graph->alloc_vertex_array<VertexId>();
  TraceBuffers tb;
  graph->cc(label, &tb.stats);
  print_active(tb, tb.stats.calls, graph->vertices);
  exec_time += get_time();
  printf("exec_time=%lf(s)\n", exec_time);
  std::vector<VertexId> count(graph->vertices, 0);
  for (VertexId v = 0; v < graph->vertices; v++) count[label[v]] += 1;
  VertexId components = 0;
  for (VertexId v = 0; v < graph->vertices; v++)
    if (count[v] > 0) components += 1;
  printf("components = %u\n", components);
  graph->dealloc_vertex_array(label);
}

int main(int argc, char **argv) {
  if (argc < 3) {
    printf("cc [file] [vertices]\n");
    exit(-1);
  }
  return run_main([&] {
    Graph<Empty> *graph = new Graph<Empty>();
    graph->load_undirected_from_directed(argv[1], std::atoi(argv[2]));
    for (int run = 0; run < 6; run++) compute(graph);
    delete graph;
  });
}
