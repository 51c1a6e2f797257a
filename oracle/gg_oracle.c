/*
 * gg_oracle.c -- TEST INFRASTRUCTURE ONLY.
 *
 * A serial CPU restatement of Gemini's single-partition edge-processing
 * engine (core/graph.hpp) and of its five toolkits (toolkits/*.cpp).  Only the
 * tests, the smoke check and the CPU-baseline leg of the benchmark may load
 * this library, and only as the checker; the product never calls it.
 *
 * Pinned against the reference itself: tests/golden/ holds outputs of the
 * unmodified reference toolkits (built from their sources by
 * oracle/build_ref.sh) on small graphs, and tests/test_oracle_golden.py checks
 * this file against them.
 *
 * Semantics restated here, with the reference lines they follow:
 *  - Graph build: load_directed (core/graph.hpp:771-1339) groups edges by
 *    source (CSR, "outgoing") and by destination (CSC, "incoming");
 *    load_undirected_from_directed (core/graph.hpp:349-757) adds the reversed
 *    copy of every record, counts both endpoints in the degree and aliases
 *    CSC = CSR.  `edges` is the number of file records in both cases
 *    (core/graph.hpp:360,782).  The reference's neighbour order inside one
 *    list is whatever its racing fetch_add fill produced; here lists are
 *    sorted by neighbour id, ties kept in record order (the order the GPU
 *    build produces too).
 *  - process_vertices (core/graph.hpp:1406-1469): sum of f(v) over set bits.
 *  - process_edges (core/graph.hpp:1492-1867): active_edges = sum of
 *    out_degree over the active set (:1503-1508); sparse iff
 *    active_edges < edges / 20 (:1509).  Both modes run every signal before
 *    any slot (messages are buffered, :1541-1556, :1755-1793), so a slot
 *    never sees state written in the same call by another slot's signal:
 *    every message is computed from the state at the start of the call.
 *  - Sparse slots run only for vertices with at least one out-edge
 *    (:1625); dense signals run only for vertices with in-degree > 0 (:1755).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
  uint32_t V;
  uint64_t E;      /* file records: the `edges` of the switch */
  uint64_t nadj;   /* adjacency entries per direction (2E when symmetric) */
  int weighted;
  int symmetric;
  uint64_t *out_off;
  uint32_t *out_nbr;
  float *out_w;
  uint32_t *out_deg;
  uint64_t *in_off;
  uint32_t *in_nbr;
  float *in_w;
  uint32_t *in_deg;
} orc_graph;

/* One record per process_edges call. */
typedef struct {
  int capacity;
  int count;
  int32_t *mode;          /* 0 = sparse (push), 1 = dense (pull) */
  uint64_t *active_edges; /* the switch's left-hand side */
  uint64_t *activated;    /* popcount of the slot-written active set (or V for PageRank) */
} orc_trace;

static void trace_add(orc_trace *t, int mode, uint64_t active_edges, uint64_t activated) {
  if (!t) return;
  if (t->count < t->capacity) {
    t->mode[t->count] = mode;
    t->active_edges[t->count] = active_edges;
    t->activated[t->count] = activated;
  }
  t->count += 1;
}

/* ---- bitmaps: 64-bit words, bit v%64 of word v/64 (core/bitmap.hpp:20-21) ---- */
static uint64_t *bm_new(uint32_t V) { return (uint64_t *)calloc((size_t)V / 64 + 1, 8); }
static void bm_clear(uint64_t *b, uint32_t V) { memset(b, 0, ((size_t)V / 64 + 1) * 8); }
static int bm_get(const uint64_t *b, uint32_t v) { return (int)((b[v >> 6] >> (v & 63)) & 1u); }
static void bm_set(uint64_t *b, uint32_t v) { b[v >> 6] |= 1ull << (v & 63); }
static uint64_t bm_count(const uint64_t *b, uint32_t V) {
  uint64_t c = 0;
  for (size_t i = 0; i <= (size_t)V / 64; i++) c += (uint64_t)__builtin_popcountll(b[i]);
  return c;
}

static int cmp_u64(const void *a, const void *b) {
  uint64_t x = *(const uint64_t *)a, y = *(const uint64_t *)b;
  return x < y ? -1 : (x > y ? 1 : 0);
}

/* Builds one direction: entries grouped by major[], sorted by minor[], ties in
 * entry order.  A stable counting pass groups the entries by major; each list
 * is then sorted on (minor << 32 | position in the list), which keeps equal
 * minors in entry order. */
static void build_dir(uint32_t V, uint64_t n, const uint32_t *major, const uint32_t *minor,
                      const float *w, uint64_t **off_out, uint32_t **nbr_out, float **w_out) {
  uint64_t *off = (uint64_t *)calloc((size_t)V + 1, sizeof(uint64_t));
  for (uint64_t i = 0; i < n; i++) off[major[i] + 1] += 1;
  for (uint32_t v = 0; v < V; v++) off[v + 1] += off[v];
  uint64_t *fill = (uint64_t *)malloc(sizeof(uint64_t) * ((size_t)V + 1));
  memcpy(fill, off, sizeof(uint64_t) * ((size_t)V + 1));
  uint64_t *order = (uint64_t *)malloc(sizeof(uint64_t) * (n ? n : 1));
  for (uint64_t i = 0; i < n; i++) order[fill[major[i]]++] = i;
  free(fill);
  uint32_t *nbr = (uint32_t *)malloc(sizeof(uint32_t) * (n ? n : 1));
  float *ww = w ? (float *)malloc(sizeof(float) * (n ? n : 1)) : NULL;
  uint64_t *keys = NULL;
  uint64_t cap = 0;
  for (uint32_t v = 0; v < V; v++) {
    uint64_t lo = off[v], len = off[v + 1] - lo;
    if (len > cap) {
      cap = len;
      keys = (uint64_t *)realloc(keys, sizeof(uint64_t) * cap);
    }
    for (uint64_t k = 0; k < len; k++) keys[k] = ((uint64_t)minor[order[lo + k]] << 32) | k;
    if (len > 1) qsort(keys, len, sizeof(uint64_t), cmp_u64);
    for (uint64_t k = 0; k < len; k++) {
      uint64_t e = order[lo + (keys[k] & 0xFFFFFFFFull)];
      nbr[lo + k] = minor[e];
      if (ww) ww[lo + k] = w[e];
    }
  }
  free(keys);
  free(order);
  *off_out = off;
  *nbr_out = nbr;
  *w_out = ww;
}

/* Directed: core/graph.hpp:771-1339.  Symmetric: core/graph.hpp:349-757. */
int orc_build(uint32_t V, uint64_t E, const uint32_t *src, const uint32_t *dst, const float *w,
              int symmetric, orc_graph **out) {
  for (uint64_t i = 0; i < E; i++) {
    if (src[i] >= V || dst[i] >= V) return -1;
  }
  orc_graph *g = (orc_graph *)calloc(1, sizeof(orc_graph));
  g->V = V;
  g->E = E;
  g->weighted = w != NULL;
  g->symmetric = symmetric;
  if (!symmetric) {
    g->nadj = E;
    build_dir(V, E, src, dst, w, &g->out_off, &g->out_nbr, &g->out_w);
    build_dir(V, E, dst, src, w, &g->in_off, &g->in_nbr, &g->in_w);
    g->out_deg = (uint32_t *)calloc((size_t)V + 1, 4);
    g->in_deg = (uint32_t *)calloc((size_t)V + 1, 4);
    for (uint64_t i = 0; i < E; i++) {
      g->out_deg[src[i]] += 1;
      g->in_deg[dst[i]] += 1;
    }
  } else {
    /* entry i < E is record i; entry E+i is record i reversed */
    uint64_t n = 2 * E;
    uint32_t *maj = (uint32_t *)malloc(sizeof(uint32_t) * (n ? n : 1));
    uint32_t *min = (uint32_t *)malloc(sizeof(uint32_t) * (n ? n : 1));
    float *ww = w ? (float *)malloc(sizeof(float) * (n ? n : 1)) : NULL;
    for (uint64_t i = 0; i < E; i++) {
      maj[i] = src[i];
      min[i] = dst[i];
      maj[E + i] = dst[i];
      min[E + i] = src[i];
      if (ww) ww[i] = ww[E + i] = w[i];
    }
    g->nadj = n;
    build_dir(V, n, maj, min, ww, &g->out_off, &g->out_nbr, &g->out_w);
    free(maj);
    free(min);
    free(ww);
    g->out_deg = (uint32_t *)calloc((size_t)V + 1, 4);
    for (uint64_t i = 0; i < E; i++) {
      g->out_deg[src[i]] += 1;
      g->out_deg[dst[i]] += 1;
    }
    g->in_off = g->out_off;
    g->in_nbr = g->out_nbr;
    g->in_w = g->out_w;
    g->in_deg = g->out_deg;
  }
  *out = g;
  return 0;
}

void orc_free(orc_graph *g) {
  if (!g) return;
  if (!g->symmetric) {
    free(g->in_off);
    free(g->in_nbr);
    free(g->in_w);
    free(g->in_deg);
  }
  free(g->out_off);
  free(g->out_nbr);
  free(g->out_w);
  free(g->out_deg);
  free(g);
}

uint64_t orc_num_adj(const orc_graph *g) { return g->nadj; }

/* Copies one direction (incoming != 0: CSC) out for structure checks. */
void orc_get_adj(const orc_graph *g, int incoming, uint64_t *off, uint32_t *nbr, float *w,
                 uint32_t *deg) {
  const uint64_t *o = incoming ? g->in_off : g->out_off;
  const uint32_t *n = incoming ? g->in_nbr : g->out_nbr;
  const float *ww = incoming ? g->in_w : g->out_w;
  const uint32_t *d = incoming ? g->in_deg : g->out_deg;
  if (off) memcpy(off, o, sizeof(uint64_t) * ((size_t)g->V + 1));
  if (nbr) memcpy(nbr, n, sizeof(uint32_t) * g->nadj);
  if (w && ww) memcpy(w, ww, sizeof(float) * g->nadj);
  if (deg) memcpy(deg, d, sizeof(uint32_t) * g->V);
}

/* transpose(): core/graph.hpp:759-769 */
static void orc_transpose(orc_graph *g) {
  uint64_t *to = g->out_off; g->out_off = g->in_off; g->in_off = to;
  uint32_t *tn = g->out_nbr; g->out_nbr = g->in_nbr; g->in_nbr = tn;
  float *tw = g->out_w; g->out_w = g->in_w; g->in_w = tw;
  uint32_t *td = g->out_deg; g->out_deg = g->in_deg; g->in_deg = td;
}

static uint64_t active_edges_of(const orc_graph *g, const uint64_t *active) {
  uint64_t s = 0;
  for (uint32_t v = 0; v < g->V; v++)
    if (bm_get(active, v)) s += g->out_deg[v];
  return s;
}

static int is_sparse(const orc_graph *g, uint64_t active_edges) { return active_edges < g->E / 20; }

/* ------------------------------------------------------------------ BFS */
/* toolkits/bfs.cpp:22-109 */
int orc_bfs(const orc_graph *g, uint32_t root, uint32_t *parent, orc_trace *tr) {
  uint32_t V = g->V;
  if (root >= V) return -1;
  uint64_t *visited = bm_new(V), *ain = bm_new(V), *aout = bm_new(V);
  bm_set(visited, root);
  bm_set(ain, root);
  for (uint32_t v = 0; v < V; v++) parent[v] = V;
  parent[root] = root;
  uint64_t active_vertices = 1;
  int iters = 0;
  while (active_vertices > 0) {
    bm_clear(aout, V);
    uint64_t ae = active_edges_of(g, ain);
    int sparse = is_sparse(g, ae);
    if (sparse) {
      for (uint32_t v = 0; v < V; v++) {
        if (!bm_get(ain, v)) continue;
        for (uint64_t e = g->out_off[v]; e < g->out_off[v + 1]; e++) {
          uint32_t d = g->out_nbr[e];
          if (parent[d] == V) {
            parent[d] = v;
            bm_set(aout, d);
          }
        }
      }
    } else {
      for (uint32_t v = 0; v < V; v++) {
        if (g->in_deg[v] == 0 || bm_get(visited, v)) continue;
        for (uint64_t e = g->in_off[v]; e < g->in_off[v + 1]; e++) {
          uint32_t s = g->in_nbr[e];
          if (bm_get(ain, s)) {
            if (parent[v] == V) {
              parent[v] = s;
              bm_set(aout, v);
            }
            break;
          }
        }
      }
    }
    active_vertices = bm_count(aout, V);
    trace_add(tr, sparse ? 0 : 1, ae, active_vertices);
    for (size_t i = 0; i <= (size_t)V / 64; i++) visited[i] |= aout[i];
    uint64_t *t = ain; ain = aout; aout = t;
    iters++;
  }
  free(visited);
  free(ain);
  free(aout);
  return iters;
}

/* ------------------------------------------------------------- PageRank */
/* toolkits/pagerank.cpp:26-129; d = 0.85 (pagerank.cpp:24).  deltas[i] is
 * the value printed as delta(i). */
int orc_pagerank(const orc_graph *g, int iterations, double *curr_out, double *deltas,
                 orc_trace *tr) {
  const double d = 0.85;
  uint32_t V = g->V;
  double *curr = (double *)malloc(sizeof(double) * ((size_t)V + 1));
  double *next = (double *)malloc(sizeof(double) * ((size_t)V + 1));
  double delta = 0;
  for (uint32_t v = 0; v < V; v++) {
    curr[v] = 1.0;
    if (g->out_deg[v] > 0) curr[v] /= g->out_deg[v];
    delta += 1.0;
  }
  delta /= V;
  for (int i = 0; i < iterations; i++) {
    if (deltas) deltas[i] = delta;
    for (uint32_t v = 0; v < V; v++) next[v] = 0;
    uint64_t ae = 0;
    for (uint32_t v = 0; v < V; v++) ae += g->out_deg[v];
    int sparse = is_sparse(g, ae);
    if (sparse) {
      for (uint32_t v = 0; v < V; v++) {
        double msg = curr[v];
        for (uint64_t e = g->out_off[v]; e < g->out_off[v + 1]; e++) next[g->out_nbr[e]] += msg;
      }
    } else {
      for (uint32_t v = 0; v < V; v++) {
        if (g->in_deg[v] == 0) continue;
        double sum = 0;
        for (uint64_t e = g->in_off[v]; e < g->in_off[v + 1]; e++) sum += curr[g->in_nbr[e]];
        next[v] += sum;
      }
    }
    trace_add(tr, sparse ? 0 : 1, ae, V);
    delta = 0;
    if (i == iterations - 1) {
      for (uint32_t v = 0; v < V; v++) next[v] = 1 - d + d * next[v];
    } else {
      for (uint32_t v = 0; v < V; v++) {
        next[v] = 1 - d + d * next[v];
        if (g->out_deg[v] > 0) {
          next[v] /= g->out_deg[v];
          delta += fabs(next[v] - curr[v]) * g->out_deg[v];
        } else {
          delta += fabs(next[v] - curr[v]);
        }
      }
    }
    delta /= V;
    double *t = curr; curr = next; next = t;
  }
  memcpy(curr_out, curr, sizeof(double) * V);
  free(curr);
  free(next);
  return iterations;
}

/* ------------------------------------------------------------------- CC */
/* toolkits/cc.cpp:22-88, on the symmetric graph (cc.cpp:121). */
int orc_cc(const orc_graph *g, uint32_t *label, orc_trace *tr) {
  uint32_t V = g->V;
  uint64_t *ain = bm_new(V), *aout = bm_new(V);
  uint32_t *msg = (uint32_t *)malloc(sizeof(uint32_t) * ((size_t)V + 1));
  for (uint32_t v = 0; v < V; v++) {
    label[v] = v;
    bm_set(ain, v);
  }
  uint64_t active_vertices = V;
  int iters = 0;
  while (active_vertices > 0) {
    bm_clear(aout, V);
    uint64_t ae = active_edges_of(g, ain);
    int sparse = is_sparse(g, ae);
    if (sparse) {
      for (uint32_t v = 0; v < V; v++) msg[v] = label[v]; /* signals read pre-call state */
      for (uint32_t v = 0; v < V; v++) {
        if (!bm_get(ain, v)) continue;
        uint32_t m = msg[v];
        for (uint64_t e = g->out_off[v]; e < g->out_off[v + 1]; e++) {
          uint32_t d = g->out_nbr[e];
          if (m < label[d]) {
            label[d] = m;
            bm_set(aout, d);
          }
        }
      }
    } else {
      for (uint32_t v = 0; v < V; v++) {
        uint32_t m = v;
        if (g->in_deg[v] > 0) {
          for (uint64_t e = g->in_off[v]; e < g->in_off[v + 1]; e++) {
            uint32_t s = g->in_nbr[e];
            if (label[s] < m) m = label[s];
          }
        }
        msg[v] = m;
      }
      for (uint32_t v = 0; v < V; v++) {
        if (msg[v] < v && msg[v] < label[v]) {
          label[v] = msg[v];
          bm_set(aout, v);
        }
      }
    }
    active_vertices = bm_count(aout, V);
    trace_add(tr, sparse ? 0 : 1, ae, active_vertices);
    uint64_t *t = ain; ain = aout; aout = t;
    iters++;
  }
  free(ain);
  free(aout);
  free(msg);
  return iters;
}

/* ----------------------------------------------------------------- SSSP */
/* toolkits/sssp.cpp:24-90; INF = 1e9 (sssp.cpp:33). */
int orc_sssp(const orc_graph *g, uint32_t root, float *dist, orc_trace *tr) {
  uint32_t V = g->V;
  if (root >= V || !g->weighted) return -1;
  const float INF = (float)1e9;
  uint64_t *ain = bm_new(V), *aout = bm_new(V);
  float *msg = (float *)malloc(sizeof(float) * ((size_t)V + 1));
  for (uint32_t v = 0; v < V; v++) dist[v] = INF;
  dist[root] = 0;
  bm_set(ain, root);
  uint64_t active_vertices = 1;
  int iters = 0;
  while (active_vertices > 0) {
    bm_clear(aout, V);
    uint64_t ae = active_edges_of(g, ain);
    int sparse = is_sparse(g, ae);
    if (sparse) {
      for (uint32_t v = 0; v < V; v++) msg[v] = dist[v];
      for (uint32_t v = 0; v < V; v++) {
        if (!bm_get(ain, v)) continue;
        float m = msg[v];
        for (uint64_t e = g->out_off[v]; e < g->out_off[v + 1]; e++) {
          uint32_t d = g->out_nbr[e];
          float relax = m + g->out_w[e];
          if (relax < dist[d]) {
            dist[d] = relax;
            bm_set(aout, d);
          }
        }
      }
    } else {
      for (uint32_t v = 0; v < V; v++) {
        float m = INF;
        if (g->in_deg[v] > 0) {
          for (uint64_t e = g->in_off[v]; e < g->in_off[v + 1]; e++) {
            float relax = dist[g->in_nbr[e]] + g->in_w[e];
            if (relax < m) m = relax;
          }
        }
        msg[v] = m;
      }
      for (uint32_t v = 0; v < V; v++) {
        if ((double)msg[v] < 1e9 && msg[v] < dist[v]) {
          dist[v] = msg[v];
          bm_set(aout, v);
        }
      }
    }
    active_vertices = bm_count(aout, V);
    trace_add(tr, sparse ? 0 : 1, ae, active_vertices);
    uint64_t *t = ain; ain = aout; aout = t;
    iters++;
  }
  free(ain);
  free(aout);
  free(msg);
  return iters;
}

/* ------------------------------------------------------------------- BC */
/* toolkits/bc.cpp:24-196 (compute; COMPACT = 0).  dep receives
 * `dependencies`, inv receives `inv_num_paths` (the array the toolkit frees
 * last, bc.cpp:192-193). */
int orc_bc(const orc_graph *g0, uint32_t root, double *dep, double *inv, orc_trace *tr) {
  /* transpose() acts on a private copy of the handles, so that several
   * threads may run BC on one graph */
  orc_graph gl = *g0;
  orc_graph *g = &gl;
  uint32_t V = g->V;
  if (root >= V) return -1;
  size_t words = (size_t)V / 64 + 1;
  uint64_t *visited = bm_new(V);
  int cap = 64, nlev = 0;
  uint64_t **levels = (uint64_t **)malloc(sizeof(uint64_t *) * cap);
  double *np = inv; /* num_paths becomes inv_num_paths in place (bc.cpp:103) */
  double *msg = (double *)malloc(sizeof(double) * ((size_t)V + 1));
  for (uint32_t v = 0; v < V; v++) np[v] = 0.0;
  np[root] = 1.0;
  uint64_t *ain = bm_new(V);
  bm_set(ain, root);
  bm_set(visited, root);
  levels[nlev++] = ain;
  uint64_t active_vertices = 1;
  int calls = 0;
  while (active_vertices > 0) {
    uint64_t *aout = bm_new(V);
    uint64_t ae = active_edges_of(g, ain);
    int sparse = is_sparse(g, ae);
    if (sparse) {
      for (uint32_t v = 0; v < V; v++) {
        if (!bm_get(ain, v)) continue;
        double m = np[v];
        for (uint64_t e = g->out_off[v]; e < g->out_off[v + 1]; e++) {
          uint32_t d = g->out_nbr[e];
          if (!bm_get(visited, d)) {
            if (np[d] == 0) bm_set(aout, d);
            np[d] += m;
          }
        }
      }
    } else {
      for (uint32_t v = 0; v < V; v++) {
        msg[v] = 0;
        if (g->in_deg[v] == 0 || bm_get(visited, v)) continue;
        double s = 0;
        for (uint64_t e = g->in_off[v]; e < g->in_off[v + 1]; e++) {
          uint32_t u = g->in_nbr[e];
          if (bm_get(ain, u)) s += np[u];
        }
        msg[v] = s;
      }
      for (uint32_t v = 0; v < V; v++) {
        if (msg[v] > 0 && !bm_get(visited, v)) {
          bm_set(aout, v);
          np[v] += msg[v];
        }
      }
    }
    active_vertices = bm_count(aout, V);
    trace_add(tr, sparse ? 0 : 1, ae, active_vertices);
    calls++;
    for (size_t i = 0; i < words; i++) visited[i] |= aout[i];
    if (nlev == cap) {
      cap *= 2;
      levels = (uint64_t **)realloc(levels, sizeof(uint64_t *) * cap);
    }
    levels[nlev++] = aout;
    ain = aout;
  }
  for (uint32_t v = 0; v < V; v++) {
    np[v] = 1 / np[v];
    dep[v] = 0;
  }
  bm_clear(visited, V);
  {
    uint64_t *last = levels[nlev - 1];
    for (uint32_t v = 0; v < V; v++)
      if (bm_get(last, v)) {
        bm_set(visited, v);
        dep[v] += np[v];
      }
  }
  orc_transpose(g);
  while (nlev > 1) {
    uint64_t *act = levels[nlev - 1];
    uint64_t ae = active_edges_of(g, act);
    int sparse = is_sparse(g, ae);
    if (sparse) {
      for (uint32_t v = 0; v < V; v++) {
        if (!bm_get(act, v)) continue;
        double m = dep[v];
        for (uint64_t e = g->out_off[v]; e < g->out_off[v + 1]; e++) {
          uint32_t d = g->out_nbr[e];
          if (!bm_get(visited, d)) dep[d] += m;
        }
      }
    } else {
      for (uint32_t v = 0; v < V; v++) {
        msg[v] = 0;
        if (g->in_deg[v] == 0 || bm_get(visited, v)) continue;
        double s = 0;
        for (uint64_t e = g->in_off[v]; e < g->in_off[v + 1]; e++) {
          uint32_t u = g->in_nbr[e];
          if (bm_get(act, u)) s += dep[u];
        }
        msg[v] = s;
      }
      for (uint32_t v = 0; v < V; v++) {
        if (g->in_deg[v] > 0 && !bm_get(visited, v)) dep[v] += msg[v];
      }
    }
    trace_add(tr, sparse ? 0 : 1, ae, 0);
    calls++;
    free(levels[nlev - 1]);
    nlev--;
    uint64_t *lv = levels[nlev - 1];
    for (uint32_t v = 0; v < V; v++)
      if (bm_get(lv, v)) {
        bm_set(visited, v);
        dep[v] += np[v];
      }
  }
  for (uint32_t v = 0; v < V; v++) dep[v] = (dep[v] - np[v]) / np[v];
  orc_transpose(g);
  for (int i = 0; i < nlev; i++) free(levels[i]);
  free(levels);
  free(visited);
  free(msg);
  return calls;
}

/* ---- seeded synthetic edge lists (inputs of the CPU baseline and tests) ----
 *
 * Restates the benchmark's input generator so that the reference can be fed
 * the same bytes without the product library.  Counter-based: record e
 * depends only on (seed, e).
 *   key          = mix64(seed ^ 0x5851F42D4C957F2D)
 *   draw64(e, j) = mix64(key + (e * 64 + j) * 0x9E3779B97F4A7C15)  (mod 2^64)
 * mix64 is the SplitMix64 finaliser (Steele, Lea, Flood, OOPSLA 2014).
 * R-MAT (Chakrabarti, Zhan, Faloutsos, SDM 2004), a=.57 b=.19 c=.19 d=.05:
 * level l (most significant bit first) takes 32 bits of draw64(e, l/2) (low
 * half for even l, high for odd l); u >= floor(.76*2^32) sets the source bit,
 * floor(.57*2^32) <= u < floor(.76*2^32) or u >= floor(.95*2^32) the
 * destination bit.  Weight: (low32(draw64(e, 16)) >> 8) * 2^-24.
 * Grid n x n: per vertex v = r*n+c in row-major order the records (v,v+1),
 * (v+1,v) when c+1 < n, then (v,v+n), (v+n,v) when r+1 < n.
 * Records are the reference's packed EdgeUnit (core/type.hpp:27-41): two
 * uint32 words, plus the float32 weight as a third word when weighted. */
static uint64_t orc_mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

static uint64_t orc_draw(uint64_t key, uint64_t e, uint32_t j) {
  return orc_mix64(key + (e * 64u + j) * 0x9E3779B97F4A7C15ull);
}

static uint32_t orc_weight_bits(uint64_t key, uint64_t e) {
  float w = (float)((uint32_t)orc_draw(key, e, 16) >> 8) * (1.0f / 16777216.0f);
  uint32_t bits;
  memcpy(&bits, &w, 4);
  return bits;
}

/* Records [first, first + count) of R-MAT `scale` into out (2 or 3 words each). */
void orc_rmat_records(uint32_t scale, uint64_t seed, int weighted, uint64_t first, uint64_t count,
                      uint32_t *out) {
  const uint32_t ta = 2448131358u, tab = 3264175144u, tabc = 4080218931u;
  uint64_t key = orc_mix64(seed ^ 0x5851F42D4C957F2Dull);
  int words = weighted ? 3 : 2;
  for (uint64_t i = 0; i < count; i++) {
    uint64_t e = first + i;
    uint32_t s = 0, d = 0;
    uint64_t draw = 0;
    for (uint32_t l = 0; l < scale; l++) {
      if ((l & 1u) == 0) draw = orc_draw(key, e, l >> 1);
      uint32_t u = (l & 1u) ? (uint32_t)(draw >> 32) : (uint32_t)draw;
      s = (s << 1) | (u >= tab ? 1u : 0u);
      d = (d << 1) | (((u >= ta && u < tab) || u >= tabc) ? 1u : 0u);
    }
    out[i * words] = s;
    out[i * words + 1] = d;
    if (weighted) out[i * words + 2] = orc_weight_bits(key, e);
  }
}

uint64_t orc_grid_count(uint32_t n) { return n < 2 ? 0 : 4ull * n * (n - 1); }

/* Records [first, first + count) of the n x n grid.  Rows r < n-1 hold
 * 4n-2 records (4 per vertex, 2 for the last column), the last row 2(n-1). */
void orc_grid_records(uint32_t n, uint64_t seed, int weighted, uint64_t first, uint64_t count,
                      uint32_t *out) {
  uint64_t key = orc_mix64(seed ^ 0x5851F42D4C957F2Dull);
  int words = weighted ? 3 : 2;
  uint64_t row_len = 4ull * n - 2;
  for (uint64_t i = 0; i < count; i++) {
    uint64_t e = first + i, r = e / row_len, k = e % row_len, c, slot;
    if (r + 1 < n) {
      c = k / 4;
      slot = k % 4;
      if (c + 1 == n) slot += 2;
    } else {
      c = k / 2;
      slot = k % 2;
    }
    uint64_t v = r * n + c, a = v, b = slot < 2 ? v + 1 : v + n;
    if (slot & 1) { uint64_t t = a; a = b; b = t; }
    out[i * words] = (uint32_t)a;
    out[i * words + 1] = (uint32_t)b;
    if (weighted) out[i * words + 2] = orc_weight_bits(key, e);
  }
}

/* deg[src] += 1 for every record (words = 2 or 3 per record). */
void orc_count_out_degree(const uint32_t *rec, uint64_t n, int words, uint32_t *deg) {
  for (uint64_t i = 0; i < n; i++) deg[rec[i * (uint64_t)words]] += 1;
}

/* Levels of a parent tree rooted at `root` (-1 unreached).  Returns 0, or -1
 * when the root is not its own parent, a parent is out of range or
 * unreached, or the array holds a cycle. */
int orc_tree_levels(const uint32_t *parent, uint32_t V, uint32_t root, int32_t *level) {
  if (root >= V || parent[root] != root) return -1;
  for (uint32_t v = 0; v < V; v++) level[v] = parent[v] < V ? -2 : -1;  /* -2: reached, level unknown */
  level[root] = 0;
  uint32_t *stack = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)(V ? V : 1));
  int rc = 0;
  for (uint32_t v = 0; v < V && rc == 0; v++) {
    if (level[v] != -2) continue;
    /* walk up to a vertex of known level, then assign on the way back */
    uint32_t top = 0, u = v;
    while (level[u] == -2) {
      if (top >= V) { rc = -1; break; }     /* longer than V: a cycle */
      stack[top++] = u;
      level[u] = -3;                          /* on the current path */
      u = parent[u];
      if (u >= V) { rc = -1; break; }
    }
    if (rc) break;
    if (level[u] < 0) { rc = -1; break; }    /* -3: cycle; -1: unreached parent */
    int32_t base = level[u];
    while (top > 0) level[stack[--top]] = ++base;
  }
  free(stack);
  return rc;
}

/* Number of reached vertices v != root whose tree edge (parent[v], v) is not
 * an edge of the graph (in-lists are sorted by neighbour id). */
uint64_t orc_tree_bad_edges(const orc_graph *g, const uint32_t *parent, uint32_t root) {
  uint64_t bad = 0;
  for (uint32_t v = 0; v < g->V; v++) {
    uint32_t p = parent[v];
    if (v == root || p >= g->V) continue;
    uint64_t lo = g->in_off[v], hi = g->in_off[v + 1];
    while (lo < hi) {
      uint64_t mid = lo + (hi - lo) / 2;
      if (g->in_nbr[mid] < p) lo = mid + 1; else hi = mid;
    }
    if (lo == g->in_off[v + 1] || g->in_nbr[lo] != p) bad++;
  }
  return bad;
}
