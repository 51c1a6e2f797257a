// toolkits/bfs.cpp command line on the GB300 engine: same argv, same output.
#include "common.hpp"

static void compute(Graph<Empty> *graph, VertexId root) {
  double exec_time = 0;
  exec_time -= get_time();
  VertexId *parent = graph->alloc_vertex_array<VertexId>();
  TraceBuffers tb;
  graph->bfs(root, parent, &tb.stats);
  print_active(tb, tb.stats.calls, 1);
  exec_time += get_time();
  printf("exec_time=%lf(s)\n", exec_time);
  VertexId found_vertices = 0;
  for (VertexId v = 0; v < graph->vertices; v++)
    if (parent[v] < graph->vertices) found_vertices += 1;
  printf("found_vertices = %u\n", found_vertices);
  graph->dealloc_vertex_array(parent);
}

int main(int argc, char **argv) {
  if (argc < 4) {
    printf("bfs [file] [vertices] [root]\n");
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
