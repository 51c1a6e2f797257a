// TEST INFRASTRUCTURE: the reference's SSSP callbacks on this library's
// engine.  The four process_edges callbacks of the reference's SSSP toolkit
// (toolkits/sssp.cpp:46-80) are taken from the staged reference source by
// oracle/build_ref.sh into _ref/src/sssp_callbacks.inc with one mechanical
// change -- each lambda becomes a __device__ lambda capturing by value
// (`[&](` -> `[=] __device__ (`), as CUDA requires of device lambdas -- and
// compiled here against gemini/engine.cuh, whose list form of process_edges
// takes the reference's callback signatures (VertexAdjList, emit, write_min,
// VertexSubset::set_bit).  The loop around them restates compute()'s
// (toolkits/sssp.cpp:24-44, 81-85).
//
// Usage: ref_engine_sssp <weighted edge file> <vertices> <root> <out>
//   <out> receives the distances (float32); stdout one line per
//   process_edges call: "call <i> mode <0 sparse|1 dense> returned <R>".
#include <stdio.h>
#include <stdlib.h>

#include <utility>
#include <vector>

#include "gemini/engine.cuh"

typedef float Weight;
typedef gemini::DeviceSubset VertexSubset_;

int main(int argc, char **argv) {
  if (argc < 5) {
    fprintf(stderr, "usage: %s <weighted edge file> <vertices> <root> <out>\n", argv[0]);
    return 2;
  }
  try {
    Graph<Weight> host_graph;
    host_graph.load_directed(argv[1], (VertexId)strtoul(argv[2], nullptr, 10));
    const VertexId root = (VertexId)strtoul(argv[3], nullptr, 10);
    gemini::Engine<Weight> engine(host_graph);
    gemini::DeviceGraph<Weight> *graph = engine.device_graph();
    Weight *distance = engine.alloc_vertex_array<Weight>();
    VertexSubset_ *active_in = engine.alloc_vertex_subset();
    VertexSubset_ *active_out = engine.alloc_vertex_subset();
    active_in->clear();
    active_in->set_bit(root);
    engine.fill_vertex_array(distance, (Weight)1e9);
    const Weight zero = 0;
    gemini::cuda_check(cudaMemcpyAsync(distance + root, &zero, sizeof(Weight), cudaMemcpyHostToDevice,
                                       engine.stream()),
                       "root");
    VertexId active_vertices = 1;
    for (int i_i = 0; active_vertices > 0; i_i++) {
      active_out->clear();
      active_vertices = engine.process_edges<VertexId, Weight>(
#include "sssp_callbacks.inc"
          active_in);
      printf("call %d mode %d returned %u\n", i_i, engine.last_mode, active_vertices);
      std::swap(active_in, active_out);
    }
    std::vector<Weight> h(engine.vertices);
    engine.copy_to_host(h.data(), distance);
    FILE *f = fopen(argv[4], "wb");
    if (!f) {
      perror(argv[4]);
      return 2;
    }
    fwrite(h.data(), sizeof(Weight), h.size(), f);
    fclose(f);
    engine.dealloc_vertex_array(distance);
    delete active_in;
    delete active_out;
  } catch (const gemini::Error &e) {
    fprintf(stderr, "error %d: %s\n", e.code, e.what());
    return 1;
  }
  return 0;
}
