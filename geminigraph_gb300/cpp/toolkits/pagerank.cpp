// toolkits/pagerank.cpp command line on the GB300 engine: same argv, same output.
#include "common.hpp"

static void compute(Graph<Empty> *graph, int iterations) {
  double exec_time = 0;
  exec_time -= get_time();
  double *curr = graph->alloc_vertex_array<double>();
  std::vector<double> deltas(iterations > 0 ? iterations : 1);
  graph->pagerank(iterations, curr, deltas.data());
  for (int i = 0; i < iterations; i++) printf("delta(%d)=%lf\n", i, deltas[i]);
  exec_time += get_time();
  printf("exec_time=%lf(s)\n", exec_time);
  double pr_sum = 0;
  for (VertexId v = 0; v < graph->vertices; v++) pr_sum += curr[v];
  printf("pr_sum=%lf\n", pr_sum);
  VertexId max_v_i = 0;
  for (VertexId v = 0; v < graph->vertices; v++)
    if (curr[v] > curr[max_v_i]) max_v_i = v;
  printf("pr[%u]=%lf\n", max_v_i, curr[max_v_i]);
  graph->dealloc_vertex_array(curr);
}

int main(int argc, char **argv) {
  if (argc < 4) {
    printf("pagerank [file] [vertices] [iterations]\n");
    exit(-1);
  }
  return run_main([&] {
    Graph<Empty> *graph = new Graph<Empty>();
    graph->load_directed(argv[1], std::atoi(argv[2]));
    int iterations = std::atoi(argv[3]);
    for (int run = 0; run < 6; run++) compute(graph, iterations);
    delete graph;
  });
}
