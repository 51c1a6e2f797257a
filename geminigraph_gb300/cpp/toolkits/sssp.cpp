// toolkits/sssp.cpp command line on the GB300 engine: same argv, same output.
#include "common.hpp"

static void compute(Graph<float> *graph, VertexId root) {
  double exec_time = 0;
  exec_time -= get_time();
  float *distance = graph->alloc_vertex_array<float>();
  TraceBuffers tb;
  graph->sssp(root, distance, &tb.stats);
  print_active(tb, tb.stats.calls, 1);
  exec_time += get_time();
  printf("exec_time=%lf(s)\n", exec_time);
  VertexId max_v_i = root;
  for (VertexId v = 0; v < graph->vertices; v++)
    if (distance[v] < 1e9 && distance[v] > distance[max_v_i]) max_v_i = v;
  printf("distance[%u]=%f\n", max_v_i, distance[max_v_i]);
  graph->dealloc_vertex_array(distance);
}

int main(int argc, char **argv) {
  if (argc < 4) {
    printf("sssp [file] [vertices] [root]\n");
    exit(-1);
  }
  return run_main([&] {
    Graph<float> *graph = new Graph<float>();
    graph->load_directed(argv[1], std::atoi(argv[2]));
    VertexId root = std::atoi(argv[3]);
    for (int run = 0; run < 6; run++) compute(graph, root);
    delete graph;
  });
}
