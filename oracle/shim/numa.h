/*
 * One-node stand-in for <numa.h>, used ONLY to compile the Gemini reference
 * toolkits on a host without libnuma.  Test infrastructure.
 *
 * Every allocation is an anonymous mmap so that numa_free (munmap) also
 * accepts the arrays that Graph::alloc_vertex_array maps itself
 * (core/graph.hpp:229-243).
 *
 * Result extraction: the toolkits print summaries only, but every vertex
 * array they free passes through numa_free(array, sizeof(T) * vertices)
 * (core/graph.hpp:242).  When GG_REF_DUMP_DIR is set, each freed buffer is
 * written to $GG_REF_DUMP_DIR/dump_<seq>.bin before it is unmapped, so the
 * full result arrays of a reference run can be compared with the oracle.
 * GG_REF_DUMP_MAX (default 64) bounds the number of dumps.
 * GG_REF_THREADS overrides the thread count the reference sees.
 *
 * A driver may also set gg_shim_free_observer to read each freed buffer
 * (after the toolkit's timed region, before the unmap): oracle/ref_driver.cpp
 * uses it to count the edges a BFS run traversed from its parent array.
 */
#ifndef GG_SHIM_NUMA_H
#define GG_SHIM_NUMA_H

#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/mman.h>
#include <unistd.h>

struct bitmask {
  unsigned long size;
  unsigned long *maskp;
};

static inline int numa_available(void) { return 0; }

static inline int numa_num_configured_cpus(void) {
  const char *env = getenv("GG_REF_THREADS");
  if (env && atoi(env) > 0) return atoi(env);
  long n = sysconf(_SC_NPROCESSORS_ONLN);
  return n > 0 ? (int)n : 1;
}

static inline int numa_num_configured_nodes(void) { return 1; }

static inline struct bitmask *numa_parse_nodestring(const char *) {
  static unsigned long word = 1;
  static struct bitmask mask = {1, &word};
  return &mask;
}

static inline void numa_set_interleave_mask(struct bitmask *) {}
static inline int numa_run_on_node(int) { return 0; }
static inline void numa_tonode_memory(void *, size_t, int) {}

static inline void *gg_shim_map(size_t size) {
  if (size == 0) size = 1;
  void *p = mmap(NULL, size, PROT_READ | PROT_WRITE, MAP_PRIVATE | MAP_ANONYMOUS, -1, 0);
  return p == MAP_FAILED ? NULL : p;
}

static inline void *numa_alloc_onnode(size_t size, int) { return gg_shim_map(size); }
static inline void *numa_alloc_interleaved(size_t size) { return gg_shim_map(size); }

static inline void *numa_realloc(void *old_addr, size_t old_size, size_t new_size) {
  void *p = gg_shim_map(new_size);
  if (p && old_addr) {
    memcpy(p, old_addr, old_size < new_size ? old_size : new_size);
    munmap(old_addr, old_size ? old_size : 1);
  }
  return p;
}

static void (*gg_shim_free_observer)(const void *start, size_t size) = 0;

static inline void numa_free(void *start, size_t size) {
  static int seq = 0;
  if (gg_shim_free_observer) gg_shim_free_observer(start, size);
  const char *dir = getenv("GG_REF_DUMP_DIR");
  const char *max_env = getenv("GG_REF_DUMP_MAX");
  int max_dumps = max_env ? atoi(max_env) : 64;
  if (dir && seq < max_dumps) {
    char path[4096];
    snprintf(path, sizeof(path), "%s/dump_%03d.bin", dir, seq);
    FILE *f = fopen(path, "wb");
    if (f) {
      fwrite(start, 1, size, f);
      fclose(f);
    }
  }
  seq += 1;
  munmap(start, size ? size : 1);
}

#endif
