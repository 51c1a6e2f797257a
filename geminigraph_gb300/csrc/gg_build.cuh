// Graph build internals shared by the in-core build (gg_store.cu) and the
// partitioned build (gg_partition.cu).  Not part of the C ABI.
#ifndef GG_BUILD_CUH
#define GG_BUILD_CUH

#include <vector>

#include "gg_common.cuh"

namespace gg {

// Bits of the largest vertex id (at least 1): keys pack (major << b) | minor.
int bits_for(uint32_t V);

// Stable LSD radix sort of n keys (and optional 32-bit values) on the low
// key_bits bits, ping-ponging between (k0, v0) and (k1, v1); *kres / *vres
// name the buffers holding the result.
int radix_sort(gg_graph *g, uint64_t *k0, uint32_t *v0, uint64_t *k1, uint32_t *v1, size_t n, int key_bits,
               uint64_t **kres, uint32_t **vres);

// Neighbour / weight storage in device memory, or in mapped pinned host memory.
int adj_alloc(gg_graph *g, bool host, void **p, size_t bytes);

// Degrees, the deg > 0 bitmap and the bins of a direction whose offsets are written.
int finish_dir(gg_graph *g, Dir *d);

// The in-core build from E records in device memory.
int build_from_device_records(gg_graph *g, const uint32_t *rec, uint64_t E);

// Largest force_partitions the build options accept.
constexpr int32_t OC_MAX_FORCED = 256;

// In-core or partitioned, and for the partitioned build its range and group
// capacities (entries), from the device-memory budget.
int build_plan(gg_graph *g, uint64_t E, bool rec_on_device, const gg_build_options *opt, bool *partitioned,
               uint64_t *cap, uint64_t *gcap);

// Builds both directions from E records readable by the device at rec.
int build_records(gg_graph *g, const uint32_t *rec, uint64_t E, bool partitioned, uint64_t cap, uint64_t gcap,
                  gg_build_options *opt);

// Device buffers freed together when the build returns.
struct DevScratch {
  std::vector<void *> p;
  DevScratch() = default;
  DevScratch(const DevScratch &) = delete;
  DevScratch &operator=(const DevScratch &) = delete;
  ~DevScratch() {
    for (void *q : p) cudaFree(q);
  }
  template <typename T>
  int get(T **out, size_t count) {
    void *q = nullptr;
    GG_CUDA(cudaMalloc(&q, count ? count * sizeof(T) : 16));
    p.push_back(q);
    *out = (T *)q;
    return GG_OK;
  }
};

}  // namespace gg

#endif
