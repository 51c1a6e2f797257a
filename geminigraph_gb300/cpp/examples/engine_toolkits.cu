// The reference's five toolkits (toolkits/{bfs,cc,pagerank,sssp,bc}.cpp)
// written against the generic engine of gemini/engine.cuh: the same loops,
// subsets and signal/slot pairs, with the slots and signals as device lambdas
// taking one edge each.  Unlike the library's built-in gg_bfs etc., nothing
// here is specialised: every kernel is the engine's template instantiated
// for these lambdas.
//
//   engine_toolkits bfs      <file> <vertices> <root>        <out>   parent (u32)
//   engine_toolkits cc       <file> <vertices>               <out>   label (u32)
//   engine_toolkits pagerank <file> <vertices> <iterations>  <out>   ranks (f64)
//   engine_toolkits sssp     <file> <vertices> <root>        <out>   distance (f32), weighted file
//   engine_toolkits bc       <file> <vertices> <root>        <out>   dependencies, then 1/num_paths (f64)
//
// <out> receives the result array(s) raw; stdout gets one line per
// process_edges call: "call <i> mode <0 sparse|1 dense> returned <R>".
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include <utility>
#include <vector>

#include "gemini/engine.cuh"

using gemini::DeviceSubset;
using gemini::Msg;

template <typename T>
static void write_out(const char *path, const std::vector<T> &a, const char *mode = "wb") {
  FILE *f = fopen(path, mode);
  if (!f) {
    perror(path);
    exit(2);
  }
  fwrite(a.data(), sizeof(T), a.size(), f);
  fclose(f);
}

template <typename T, typename E>
static std::vector<T> to_host(gemini::Engine<E> &eng, const T *dev) {
  std::vector<T> h(eng.vertices);
  eng.copy_to_host(h.data(), dev);
  return h;
}

template <typename T, typename E>
static void put(gemini::Engine<E> &eng, T *dev, VertexId v, T value) {
  gemini::cuda_check(cudaMemcpyAsync(dev + v, &value, sizeof(T), cudaMemcpyHostToDevice, eng.stream()), "put");
  eng.sync();
}

static int call_no = 0;
template <typename R, typename E>
static void trace(gemini::Engine<E> &eng, R r) {
  printf("call %d mode %d returned %.17g\n", call_no++, eng.last_mode, (double)r);
}

// toolkits/bfs.cpp:22-109
static void bfs(Graph<Empty> &graph, VertexId root, const char *out) {
  gemini::Engine<Empty> eng(graph);
  const VertexId V = eng.vertices;
  VertexId *parent = eng.alloc_vertex_array<VertexId>();
  DeviceSubset *visited = eng.alloc_vertex_subset();
  DeviceSubset *active_in = eng.alloc_vertex_subset();
  DeviceSubset *active_out = eng.alloc_vertex_subset();
  visited->set_bit(root);
  active_in->set_bit(root);
  eng.fill_vertex_array(parent, V);
  put(eng, parent, root, root);
  VertexId active_vertices = 1;
  while (active_vertices > 0) {
    active_out->clear();
    const auto in = gemini::ref(active_in), nx = gemini::ref(active_out), vis = gemini::ref(visited);
    active_vertices = eng.process_edges<VertexId, VertexId>(
        gemini::sparse([] __device__(VertexId src) { return gemini::emit(src); },
                       [=] __device__(VertexId src, VertexId, VertexId dst, Empty) -> VertexId {
                         if (parent[dst] == V && atomicCAS(parent + dst, V, src) == V) {
                           nx.set_bit(dst);
                           return 1;
                         }
                         return 0;
                       }),
        gemini::dense([=] __device__(VertexId dst) { return !vis.get_bit(dst); },
                      [=] __device__(VertexId, VertexId src, Empty) {
                        return in.get_bit(src) ? gemini::emit(src) : gemini::no_msg<VertexId>();
                      },
                      [] __device__(Msg<VertexId> & acc, Msg<VertexId> x) {
                        if (!acc.emit && x.emit) acc = x;
                        return acc.emit != 0;
                      },
                      [=] __device__(VertexId dst, VertexId msg) -> VertexId {
                        if (atomicCAS(parent + dst, V, msg) == V) {
                          nx.set_bit(dst);
                          return 1;
                        }
                        return 0;
                      }),
        active_in, visited);
    trace(eng, active_vertices);
    active_vertices = eng.process_vertices<VertexId>(
        [=] __device__(VertexId v) -> VertexId {
          vis.set_bit(v);
          return 1;
        },
        active_out);
    std::swap(active_in, active_out);
  }
  write_out(out, to_host(eng, parent));
  eng.dealloc_vertex_array(parent);
  delete visited;
  delete active_in;
  delete active_out;
}

// toolkits/cc.cpp:22-109
static void cc(Graph<Empty> &graph, const char *out) {
  gemini::Engine<Empty> eng(graph);
  VertexId *label = eng.alloc_vertex_array<VertexId>();
  DeviceSubset *active_in = eng.alloc_vertex_subset();
  DeviceSubset *active_out = eng.alloc_vertex_subset();
  active_in->fill();
  VertexId active_vertices = eng.process_vertices<VertexId>(
      [=] __device__(VertexId v) -> VertexId {
        label[v] = v;
        return 1;
      },
      active_in);
  while (active_vertices > 0) {
    active_out->clear();
    const auto nx = gemini::ref(active_out);
    active_vertices = eng.process_edges<VertexId, VertexId>(
        gemini::sparse([=] __device__(VertexId src) { return gemini::emit(label[src]); },
                       [=] __device__(VertexId, VertexId msg, VertexId dst, Empty) -> VertexId {
                         if (msg < label[dst]) {
                           atomicMin(label + dst, msg);
                           nx.set_bit(dst);
                           return 1;
                         }
                         return 0;
                       }),
        gemini::dense([] __device__(VertexId) { return true; },
                      [=] __device__(VertexId, VertexId src, Empty) { return gemini::emit(label[src]); },
                      [] __device__(Msg<VertexId> & acc, Msg<VertexId> x) {
                        if (x.emit && (!acc.emit || x.value < acc.value)) acc = x;
                        return false;
                      },
                      [=] __device__(VertexId dst, VertexId msg) -> VertexId {
                        // the reference emits only min(label[src]) < dst
                        if (msg < dst && msg < label[dst]) {
                          atomicMin(label + dst, msg);
                          nx.set_bit(dst);
                          return 1;
                        }
                        return 0;
                      }),
        active_in);
    trace(eng, active_vertices);
    std::swap(active_in, active_out);
  }
  write_out(out, to_host(eng, label));
  eng.dealloc_vertex_array(label);
  delete active_in;
  delete active_out;
}

// toolkits/pagerank.cpp:26-129
static void pagerank(Graph<Empty> &graph, int iterations, const char *out) {
  gemini::Engine<Empty> eng(graph);
  const double d = 0.85;
  double *curr = eng.alloc_vertex_array<double>();
  double *next = eng.alloc_vertex_array<double>();
  DeviceSubset *active = eng.alloc_vertex_subset();
  active->fill();
  const uint32_t *od = eng.out_degree;
  double delta = eng.process_vertices<double>(
      [=] __device__(VertexId v) {
        curr[v] = 1.0;
        if (od[v] > 0) curr[v] /= od[v];
        return 1.0;
      },
      active);
  delta /= eng.vertices;
  std::vector<double> deltas;
  for (int i = 0; i < iterations; i++) {
    deltas.push_back(delta);
    eng.fill_vertex_array(next, 0.0);
    const int r = eng.process_edges<int, double>(
        gemini::sparse([=] __device__(VertexId src) { return gemini::emit(curr[src]); },
                       [=] __device__(VertexId, double msg, VertexId dst, Empty) {
                         atomicAdd(next + dst, msg);
                         return 0;
                       }),
        gemini::dense([] __device__(VertexId) { return true; },
                      [=] __device__(VertexId, VertexId src, Empty) { return gemini::emit(curr[src]); },
                      [] __device__(Msg<double> & acc, Msg<double> x) {
                        acc.value = acc.emit ? acc.value + x.value : x.value;
                        acc.emit = 1;
                        return false;
                      },
                      [=] __device__(VertexId dst, double msg) {
                        atomicAdd(next + dst, msg);
                        return 0;
                      }),
        active);
    trace(eng, r);
    const bool last = i == iterations - 1;
    delta = eng.process_vertices<double>(
        [=] __device__(VertexId v) {
          next[v] = 1 - d + d * next[v];
          if (last) return 0.0;
          if (od[v] > 0) {
            next[v] /= od[v];
            return fabs(next[v] - curr[v]) * od[v];
          }
          return fabs(next[v] - curr[v]);
        },
        active);
    delta /= eng.vertices;
    std::swap(curr, next);
  }
  write_out(out, to_host(eng, curr));
  write_out(std::string(out).append(".deltas").c_str(), deltas);
  eng.dealloc_vertex_array(curr);
  eng.dealloc_vertex_array(next);
  delete active;
}

// toolkits/sssp.cpp:24-105; distances compared as float bits
static void sssp(Graph<float> &graph, VertexId root, const char *out) {
  gemini::Engine<float> eng(graph);
  float *dist = eng.alloc_vertex_array<float>();
  DeviceSubset *active_in = eng.alloc_vertex_subset();
  DeviceSubset *active_out = eng.alloc_vertex_subset();
  active_in->set_bit(root);
  eng.fill_vertex_array(dist, 1e9f);
  put(eng, dist, root, 0.0f);
  VertexId active_vertices = 1;
  while (active_vertices > 0) {
    active_out->clear();
    const auto nx = gemini::ref(active_out);
    active_vertices = eng.process_edges<VertexId, float>(
        gemini::sparse([=] __device__(VertexId src) { return gemini::emit(dist[src]); },
                       [=] __device__(VertexId, float msg, VertexId dst, float w) -> VertexId {
                         const float relax = msg + w;
                         if (relax < dist[dst]) {
                           // non-negative floats order like their bit patterns
                           const int old = atomicMin(reinterpret_cast<int *>(dist + dst), __float_as_int(relax));
                           if (relax < __int_as_float(old)) {
                             nx.set_bit(dst);
                             return 1;
                           }
                         }
                         return 0;
                       }),
        gemini::dense([] __device__(VertexId) { return true; },
                      [=] __device__(VertexId, VertexId src, float w) { return gemini::emit(dist[src] + w); },
                      [] __device__(Msg<float> & acc, Msg<float> x) {
                        if (x.emit && (!acc.emit || x.value < acc.value)) acc = x;
                        return false;
                      },
                      [=] __device__(VertexId dst, float msg) -> VertexId {
                        if (msg < 1e9f && msg < dist[dst]) {
                          atomicMin(reinterpret_cast<int *>(dist + dst), __float_as_int(msg));
                          nx.set_bit(dst);
                          return 1;
                        }
                        return 0;
                      }),
        active_in);
    trace(eng, active_vertices);
    std::swap(active_in, active_out);
  }
  write_out(out, to_host(eng, dist));
  eng.dealloc_vertex_array(dist);
  delete active_in;
  delete active_out;
}

// toolkits/bc.cpp:24-196
static void bc(Graph<Empty> &graph, VertexId root, const char *out) {
  gemini::Engine<Empty> eng(graph);
  double *num_paths = eng.alloc_vertex_array<double>();
  double *dep = eng.alloc_vertex_array<double>();
  DeviceSubset *active_all = eng.alloc_vertex_subset();
  active_all->fill();
  DeviceSubset *visited = eng.alloc_vertex_subset();
  std::vector<DeviceSubset *> levels;
  DeviceSubset *active_in = eng.alloc_vertex_subset();
  visited->set_bit(root);
  active_in->set_bit(root);
  levels.push_back(active_in);
  eng.fill_vertex_array(num_paths, 0.0);
  put(eng, num_paths, root, 1.0);
  VertexId active_vertices = 1;
  while (active_vertices > 0) {
    DeviceSubset *active_out = eng.alloc_vertex_subset();
    const auto in = gemini::ref(active_in), nx = gemini::ref(active_out), vis = gemini::ref(visited);
    const VertexId r = eng.process_edges<VertexId, double>(
        gemini::sparse([=] __device__(VertexId src) { return gemini::emit(num_paths[src]); },
                       [=] __device__(VertexId, double msg, VertexId dst, Empty) -> VertexId {
                         if (!vis.get_bit(dst)) {
                           if (num_paths[dst] == 0) nx.set_bit(dst);
                           atomicAdd(num_paths + dst, msg);
                         }
                         return 0;
                       }),
        gemini::dense([=] __device__(VertexId dst) { return !vis.get_bit(dst); },
                      [=] __device__(VertexId, VertexId src, Empty) {
                        return in.get_bit(src) ? gemini::emit(num_paths[src]) : gemini::no_msg<double>();
                      },
                      [] __device__(Msg<double> & acc, Msg<double> x) {
                        if (x.emit) {
                          acc.value = acc.emit ? acc.value + x.value : x.value;
                          acc.emit = 1;
                        }
                        return false;
                      },
                      [=] __device__(VertexId dst, double msg) -> VertexId {
                        if (msg > 0 && !vis.get_bit(dst)) {
                          nx.set_bit(dst);
                          atomicAdd(num_paths + dst, msg);
                        }
                        return 0;
                      }),
        active_in, visited);
    trace(eng, r);
    active_vertices = eng.process_vertices<VertexId>(
        [=] __device__(VertexId v) -> VertexId {
          vis.set_bit(v);
          return 1;
        },
        active_out);
    levels.push_back(active_out);
    active_in = active_out;
  }
  double *inv = num_paths;
  eng.process_vertices<VertexId>(
      [=] __device__(VertexId v) -> VertexId {
        inv[v] = 1 / num_paths[v];
        dep[v] = 0;
        return 1;
      },
      active_all);
  visited->clear();
  {
    const auto vis = gemini::ref(visited);
    eng.process_vertices<VertexId>(
        [=] __device__(VertexId v) -> VertexId {
          vis.set_bit(v);
          dep[v] += inv[v];
          return 1;
        },
        levels.back());
  }
  eng.transpose();
  while (levels.size() > 1) {
    const auto lev = gemini::ref(levels.back()), vis = gemini::ref(visited);
    const VertexId r = eng.process_edges<VertexId, double>(
        gemini::sparse([=] __device__(VertexId src) { return gemini::emit(dep[src]); },
                       [=] __device__(VertexId, double msg, VertexId dst, Empty) -> VertexId {
                         if (!vis.get_bit(dst)) atomicAdd(dep + dst, msg);
                         return 0;
                       }),
        gemini::dense([=] __device__(VertexId dst) { return !vis.get_bit(dst); },
                      [=] __device__(VertexId, VertexId src, Empty) {
                        return gemini::emit(lev.get_bit(src) ? dep[src] : 0.0);
                      },
                      [] __device__(Msg<double> & acc, Msg<double> x) {
                        acc.value = acc.emit ? acc.value + x.value : x.value;
                        acc.emit = 1;
                        return false;
                      },
                      [=] __device__(VertexId dst, double msg) -> VertexId {
                        if (!vis.get_bit(dst)) atomicAdd(dep + dst, msg);
                        return 0;
                      }),
        levels.back(), visited);
    trace(eng, r);
    delete levels.back();
    levels.pop_back();
    const auto vis2 = gemini::ref(visited);
    eng.process_vertices<VertexId>(
        [=] __device__(VertexId v) -> VertexId {
          vis2.set_bit(v);
          dep[v] += inv[v];
          return 1;
        },
        levels.back());
  }
  eng.process_vertices<VertexId>(
      [=] __device__(VertexId v) -> VertexId {
        dep[v] = (dep[v] - inv[v]) / inv[v];
        return 1;
      },
      active_all);
  eng.transpose();
  std::vector<double> a = to_host(eng, dep), b = to_host(eng, inv);
  a.insert(a.end(), b.begin(), b.end());
  write_out(out, a);
  eng.dealloc_vertex_array(num_paths);
  eng.dealloc_vertex_array(dep);
  for (DeviceSubset *s : levels) delete s;
  delete visited;
  delete active_all;
}

int main(int argc, char **argv) {
  if (argc < 5) {
    fprintf(stderr, "usage: %s bfs|cc|pagerank|sssp|bc <file> <vertices> [root|iterations] <out>\n", argv[0]);
    return 1;
  }
  const std::string app = argv[1];
  const char *path = argv[2];
  const VertexId V = (VertexId)strtoul(argv[3], nullptr, 10);
  try {
    if (app == "cc") {
      Graph<Empty> g;
      g.load_undirected_from_directed(path, V);
      cc(g, argv[4]);
      return 0;
    }
    if (argc < 6) {
      fprintf(stderr, "%s needs a root or an iteration count\n", app.c_str());
      return 1;
    }
    const unsigned long x = strtoul(argv[4], nullptr, 10);
    if (app == "sssp") {
      Graph<float> g;
      g.load_directed(path, V);
      sssp(g, (VertexId)x, argv[5]);
    } else {
      Graph<Empty> g;
      g.load_directed(path, V);
      if (app == "bfs")
        bfs(g, (VertexId)x, argv[5]);
      else if (app == "pagerank")
        pagerank(g, (int)x, argv[5]);
      else if (app == "bc")
        bc(g, (VertexId)x, argv[5]);
      else {
        fprintf(stderr, "unknown toolkit %s\n", app.c_str());
        return 1;
      }
    }
  } catch (const std::exception &e) {
    fprintf(stderr, "%s\n", e.what());
    return 3;
  }
  return 0;
}
