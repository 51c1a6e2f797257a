// Partitioned graph build (the out-of-core load).
//
// core/graph.hpp:805-821 streams the edge file in CHUNKSIZE pieces so the
// whole edge list is never resident at once.  The partitioned build keeps
// the records where they are (host memory, pinned or registered for the
// build, read by the kernels over NVLink-C2C; or device memory) and builds
// each direction in ranges of its major ids: one pass counts degrees (both
// directions of a directed graph at once), one counts the entries of every
// (range, tile) pair, then groups of consecutive ranges are compacted, one
// pass over the records per group, stably and in tile order, and each range
// is sorted by the in-core build's stable radix sort on its range-relative
// key and copied into its slice of the final arrays.  Both builds sort stably
// on (major, minor) from the same entry order (records forward, then
// reversed for symmetric graphs), so the adjacency, weights included, is
// identical.  Device memory beyond the graph itself is bounded by the group
// buffer, one range's sort buffer and the count table.

#include <algorithm>
#include <vector>

#include "gg_build.cuh"
#include "gg_common.cuh"
#include "gg_scan.cuh"

namespace gg {

constexpr int OC_THREADS = 256;
constexpr int OC_TILE = 4096;                     // entries per block
constexpr int OC_WARP = OC_TILE / (OC_THREADS / 32);  // 512 consecutive entries per warp
constexpr int OC_ROUNDS = OC_WARP / 32;           // 16
// Greedy ranges of at most cap entries: two neighbouring ranges together hold
// more than cap (else they would be one), so n entries make at most
// 2n/cap + 1 ranges; 1024 covers every forced count up to 256.
constexpr uint32_t OC_MAX_PARTS = 1024;

// Entry j of the build order.  mode 0: major = src; 1: major = dst;
// 2 (symmetric): j < E forward, j >= E record j - E reversed.
struct EntrySrc {
  const uint32_t *rec;
  uint64_t E;
  int words;
  int mode;
  __device__ __forceinline__ void ids(uint64_t j, uint32_t &maj, uint32_t &mnr) const {
    const bool rev = j >= E;
    const uint64_t r = rev ? j - E : j;
    const uint32_t s = rec[r * words], d = rec[r * words + 1];
    const bool swap = mode == 1 || (mode == 2 && rev);
    maj = swap ? d : s;
    mnr = swap ? s : d;
  }
  __device__ __forceinline__ uint32_t weight_bits(uint64_t j) const {
    const uint64_t r = j >= E ? j - E : j;
    return words == 3 ? rec[r * words + 2] : 0u;
  }
};

// The counting passes read the records over the link: each thread first
// loads all its entries of a 4096-entry tile (16 independent loads in
// flight, as the compaction does), then counts them.
constexpr uint32_t OC_NO_KEY = 0xFFFFFFFFu;

__global__ void __launch_bounds__(OC_THREADS) oc_degree(EntrySrc src, uint64_t nv, uint32_t V,
                                                        uint32_t *__restrict__ cnt, unsigned *err) {
  const uint64_t base = (uint64_t)blockIdx.x * OC_TILE;
  uint32_t maj[OC_ROUNDS], mnr[OC_ROUNDS];
#pragma unroll
  for (int r = 0; r < OC_ROUNDS; r++) {
    const uint64_t j = base + (uint64_t)r * OC_THREADS + threadIdx.x;
    maj[r] = OC_NO_KEY;
    mnr[r] = 0;
    if (j < nv) src.ids(j, maj[r], mnr[r]);
  }
  const uint64_t left = nv > base ? nv - base : 0;
#pragma unroll
  for (int r = 0; r < OC_ROUNDS; r++) {
    if ((uint64_t)r * OC_THREADS + threadIdx.x >= left) continue;
    if (maj[r] >= V || mnr[r] >= V)
      atomicOr(err, 1u);
    else
      atomicAdd(&cnt[maj[r]], 1u);
  }
}

// Both directions' degrees of a directed graph in one pass over the records.
__global__ void __launch_bounds__(OC_THREADS) oc_degree_both(const uint32_t *__restrict__ rec, uint64_t E, int words,
                                                             uint32_t V, uint32_t *__restrict__ out_cnt,
                                                             uint32_t *__restrict__ in_cnt, unsigned *err) {
  const uint64_t base = (uint64_t)blockIdx.x * OC_TILE;
  uint32_t sv[OC_ROUNDS], dv[OC_ROUNDS];
#pragma unroll
  for (int r = 0; r < OC_ROUNDS; r++) {
    const uint64_t j = base + (uint64_t)r * OC_THREADS + threadIdx.x;
    sv[r] = dv[r] = OC_NO_KEY;
    if (j < E) {
      sv[r] = rec[j * words];
      dv[r] = rec[j * words + 1];
    }
  }
  const uint64_t left = E > base ? E - base : 0;
#pragma unroll
  for (int r = 0; r < OC_ROUNDS; r++) {
    if ((uint64_t)r * OC_THREADS + threadIdx.x >= left) continue;
    if (sv[r] >= V || dv[r] >= V) {
      atomicOr(err, 1u);
    } else {
      atomicAdd(&out_cnt[sv[r]], 1u);
      atomicAdd(&in_cnt[dv[r]], 1u);
    }
  }
}

struct U32AsU64 {
  const uint32_t *p;
  __device__ __forceinline__ uint64_t operator()(size_t i) const { return p[i]; }
};

// One thread: greedy ranges [bounds[k], bounds[k+1]) of at most cap entries
// (a single longer list is a range of its own).  *nparts = 0 when more than
// max_parts ranges would be needed.
__global__ void oc_bounds(const uint64_t *__restrict__ off, uint32_t V, uint64_t cap, uint32_t max_parts,
                          uint32_t *__restrict__ bounds, uint64_t *__restrict__ base, uint32_t *nparts) {
  if (blockIdx.x || threadIdx.x) return;
  uint32_t a = 0, k = 0;
  bounds[0] = 0;
  base[0] = 0;
  while (a < V) {
    if (k == max_parts) {
      *nparts = 0;
      return;
    }
    const uint64_t lim = off[a] + cap;
    uint32_t lo = a + 1, hi = V;
    if (off[lo] > lim) {
      hi = lo;
    } else {
      while (lo < hi) {  // largest b in [a+1, V] with off[b] <= lim
        const uint32_t mid = lo + (hi - lo + 1) / 2;
        if (off[mid] <= lim)
          lo = mid;
        else
          hi = mid - 1;
      }
    }
    k++;
    bounds[k] = hi;
    base[k] = off[hi];
    a = hi;
  }
  *nparts = k;
}

__device__ __forceinline__ uint32_t oc_part_of(const uint32_t *sb, uint32_t nparts, uint32_t maj) {
  uint32_t lo = 0, hi = nparts - 1;
  while (lo < hi) {
    const uint32_t mid = (lo + hi + 1) / 2;
    if (sb[mid] <= maj)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

// counts[p * ntiles + t] = entries of tile t whose major id lies in range p.
__global__ void __launch_bounds__(OC_THREADS) oc_count(EntrySrc src, uint64_t nv, const uint32_t *__restrict__ bounds,
                                                       uint32_t nparts, uint32_t ntiles, uint32_t *__restrict__ counts) {
  __shared__ uint32_t sb[OC_MAX_PARTS + 1];
  __shared__ uint32_t hist[OC_MAX_PARTS];
  for (uint32_t i = threadIdx.x; i <= nparts; i += OC_THREADS) sb[i] = bounds[i];
  for (uint32_t i = threadIdx.x; i < nparts; i += OC_THREADS) hist[i] = 0;
  __syncthreads();
  const uint64_t base = (uint64_t)blockIdx.x * OC_TILE;
  uint32_t maj[OC_ROUNDS];
#pragma unroll
  for (int r = 0; r < OC_ROUNDS; r++) {
    const uint64_t j = base + (uint64_t)r * OC_THREADS + threadIdx.x;
    uint32_t mnr;
    maj[r] = OC_NO_KEY;
    if (j < nv) src.ids(j, maj[r], mnr);
  }
  const uint64_t left = nv > base ? nv - base : 0;
#pragma unroll
  for (int r = 0; r < OC_ROUNDS; r++)
    if ((uint64_t)r * OC_THREADS + threadIdx.x < left) atomicAdd(&hist[oc_part_of(sb, nparts, maj[r])], 1u);
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < nparts; i += OC_THREADS) counts[(size_t)i * ntiles + blockIdx.x] = hist[i];
}

// Entries of the ranges p0 .. p0+m-1 (one group, m <= OC_GROUP), in build
// order within each range: warp w of tile t owns entries
// [t*4096 + w*512, +512); an entry of range p lands at
//   (base[p] - base[p0])                          the range's place in the group
// + scanned[p*ntiles + t] - scanned[p*ntiles]     earlier tiles' entries of p
// + entries of p in lower warps of the tile, then in earlier rounds and
//   lower lanes of its own warp (peers found by __match_any_sync).
// Keys are (major - lo_p, minor).  Writes at or past cap (records changed
// under the build) are dropped.
constexpr uint32_t OC_GROUP = 32;
constexpr uint32_t OC_NONE = 0xFFFFFFFFu;

__global__ void __launch_bounds__(OC_THREADS) oc_scatter(EntrySrc src, uint64_t nv, const uint32_t *__restrict__ bounds,
                                                         const uint64_t *__restrict__ base, uint32_t p0, uint32_t m,
                                                         int bits, const uint32_t *__restrict__ scanned,
                                                         const uint32_t *__restrict__ counts, uint32_t ntiles,
                                                         uint64_t cap, uint64_t *__restrict__ keys,
                                                         uint32_t *__restrict__ vals) {
  __shared__ uint32_t sb[OC_GROUP + 1];
  __shared__ uint32_t wcnt[OC_THREADS / 32][OC_GROUP];
  __shared__ uint64_t wpos[OC_THREADS / 32][OC_GROUP];
  __shared__ int any;
  if (threadIdx.x == 0) any = 0;
  for (uint32_t i = threadIdx.x; i < (OC_THREADS / 32) * OC_GROUP; i += OC_THREADS) (&wcnt[0][0])[i] = 0;
  for (uint32_t i = threadIdx.x; i <= m; i += OC_THREADS) sb[i] = bounds[p0 + i];
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < m; i += OC_THREADS)
    if (counts[(size_t)(p0 + i) * ntiles + blockIdx.x]) any = 1;
  __syncthreads();
  if (!any) return;  // no entry of the group in this tile (uniform over the block)
  const unsigned w = threadIdx.x >> 5, lane = lane_id();
  const uint64_t tb = (uint64_t)blockIdx.x * OC_TILE + (uint64_t)w * OC_WARP;
  const uint32_t lo = sb[0], hi = sb[m];
  uint32_t maj[OC_ROUNDS], mnr[OC_ROUNDS], rg[OC_ROUNDS];
#pragma unroll
  for (int r = 0; r < OC_ROUNDS; r++) {
    const uint64_t j = tb + (uint64_t)r * 32 + lane;
    maj[r] = mnr[r] = 0;
    rg[r] = OC_NONE;
    if (j < nv) {
      src.ids(j, maj[r], mnr[r]);
      if (maj[r] >= lo && maj[r] < hi) rg[r] = oc_part_of(sb, m, maj[r]);
    }
    const unsigned peers = __match_any_sync(GG_FULL, rg[r]);
    if (rg[r] != OC_NONE && lane == (unsigned)(__ffs(peers) - 1)) wcnt[w][rg[r]] += __popc(peers);
    __syncwarp();
  }
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < (OC_THREADS / 32) * m; i += OC_THREADS) {
    const uint32_t ww = i / m, q = i % m;
    const size_t row = (size_t)(p0 + q) * ntiles;
    uint64_t pos = (base[p0 + q] - base[p0]) + (scanned[row + blockIdx.x] - scanned[row]);
    for (uint32_t x = 0; x < ww; x++) pos += wcnt[x][q];
    wpos[ww][q] = pos;
  }
  __syncthreads();
#pragma unroll
  for (int r = 0; r < OC_ROUNDS; r++) {
    const unsigned peers = __match_any_sync(GG_FULL, rg[r]);
    const bool leader = lane == (unsigned)(__ffs(peers) - 1);
    if (rg[r] != OC_NONE) {
      const uint64_t at = wpos[w][rg[r]] + __popc(peers & lanemask_lt());
      if (at < cap) {
        keys[at] = ((uint64_t)(maj[r] - sb[rg[r]]) << bits) | mnr[r];
        if (vals) vals[at] = src.weight_bits(tb + (uint64_t)r * 32 + lane);
      }
    }
    __syncwarp();
    if (rg[r] != OC_NONE && leader) wpos[w][rg[r]] += __popc(peers);
    __syncwarp();
  }
}

// One block per 4096-entry tile.
static unsigned oc_grid(uint64_t n) { return (unsigned)((n + OC_TILE - 1) / OC_TILE); }

__global__ void oc_emit(const uint64_t *__restrict__ ks, const uint32_t *__restrict__ vs, uint64_t n, int bits,
                        uint32_t *__restrict__ nbr, uint32_t *__restrict__ w) {
  const uint64_t mask = (1ull << bits) - 1;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    nbr[i] = (uint32_t)(ks[i] & mask);
    if (w) w[i] = vs[i];
  }
}

// Sort-buffer bytes per entry of a range: two key buffers, two value
// buffers when weighted, the radix sort's per-tile digit counts.
static uint64_t oc_entry_bytes(int weighted) { return 16 + (weighted ? 8 : 0) + 1; }

// One direction by ranges of at most cap entries (force_parts > 0: ranges of
// ceil(entries / force_parts)), compacted gcap entries per pass over the
// records.  rec is readable by the device.
// The direction's final offsets, degrees and adjacency (n entries).
static int oc_alloc_dir(gg_graph *g, Dir *d, uint64_t n) {
  const uint32_t V = g->V;
  const bool host = g->adj_host != 0;
  GG_CUDA(cudaMalloc(&d->off, sizeof(uint64_t) * ((size_t)V + 1)));
  GG_CUDA(cudaMalloc(&d->deg, sizeof(uint32_t) * ((size_t)V + 1)));
  g->graph_bytes += sizeof(uint64_t) * ((size_t)V + 1) + sizeof(uint32_t) * ((size_t)V + 1);
  const size_t npad = (n + 64) / 64 * 64;
  GG_TRY(adj_alloc(g, host, (void **)&d->nbr, sizeof(uint32_t) * npad));
  GG_CUDA(cudaMemsetAsync(d->nbr + n, 0, sizeof(uint32_t) * (npad - n), g->stream));
  if (g->weighted) GG_TRY(adj_alloc(g, host, (void **)&d->w, sizeof(float) * (n ? n : 1)));
  return GG_OK;
}

// counted: d->deg already holds the degrees (both directions of a directed
// graph are counted in one pass); else this call counts them.  The direction
// is allocated by oc_alloc_dir.
static int build_dir_partitioned(gg_graph *g, const uint32_t *rec, uint64_t E, int mode, Dir *d, uint64_t cap,
                                 uint64_t gcap, uint32_t force_parts, bool counted, uint32_t *parts_out,
                                 uint32_t *groups_out) {
  const uint32_t V = g->V;
  const int words = g->weighted ? 3 : 2;
  const uint64_t n = mode == 2 ? 2 * E : E;
  const int bits = bits_for(V);
  EntrySrc src{rec, E, words, mode};

  // degrees -> offsets
  DevScratch tmp;
  unsigned *err = nullptr;
  uint64_t *scan64 = nullptr;
  uint32_t *bounds = nullptr, *nparts_dev = nullptr;
  uint64_t *base_dev = nullptr;
  GG_TRY(tmp.get(&err, 1));
  GG_TRY(tmp.get(&scan64, scan_scratch_elems(V) + 1));
  GG_TRY(tmp.get(&bounds, OC_MAX_PARTS + 1));
  GG_TRY(tmp.get(&base_dev, OC_MAX_PARTS + 1));
  GG_TRY(tmp.get(&nparts_dev, 1));
  GG_CUDA(cudaMemsetAsync(err, 0, sizeof(unsigned), g->stream));
  if (!counted) {
    GG_CUDA(cudaMemsetAsync(d->deg, 0, sizeof(uint32_t) * ((size_t)V + 1), g->stream));
    if (n) {
      oc_degree<<<oc_grid(n), OC_THREADS, 0, g->stream>>>(src, n, V, d->deg, err);
      GG_CUDA(cudaGetLastError());
    }
  }
  unsigned herr = 0;
  GG_CUDA(cudaMemcpyAsync(&herr, err, sizeof(unsigned), cudaMemcpyDeviceToHost, g->stream));
  GG_CUDA(cudaStreamSynchronize(g->stream));
  if (herr) {
    set_error("an edge names a vertex id >= vertices (%u)", V);
    return GG_ERR_RANGE;
  }
  GG_CUDA((exclusive_scan<uint64_t, U32AsU64>(U32AsU64{d->deg}, V, d->off, scan64, g->stream, nullptr)));

  // ranges
  if (force_parts) {
    cap = (n + force_parts - 1) / force_parts;
    gcap = 4 * cap;
  }
  if (cap == 0) cap = 1;
  *groups_out = 0;
  oc_bounds<<<1, 1, 0, g->stream>>>(d->off, V, cap, OC_MAX_PARTS, bounds, base_dev, nparts_dev);
  GG_CUDA(cudaGetLastError());
  uint32_t nparts = 0;
  GG_CUDA(cudaMemcpyAsync(&nparts, nparts_dev, sizeof(uint32_t), cudaMemcpyDeviceToHost, g->stream));
  GG_CUDA(cudaStreamSynchronize(g->stream));
  if (nparts == 0) {
    set_error("build budget too small: more than %u ranges of %llu entries per direction", OC_MAX_PARTS,
              (unsigned long long)cap);
    return GG_ERR_NOMEM;
  }
  std::vector<uint32_t> hb(nparts + 1);
  std::vector<uint64_t> hbase(nparts + 1);
  GG_CUDA(cudaMemcpy(hb.data(), bounds, sizeof(uint32_t) * (nparts + 1), cudaMemcpyDeviceToHost));
  GG_CUDA(cudaMemcpy(hbase.data(), base_dev, sizeof(uint64_t) * (nparts + 1), cudaMemcpyDeviceToHost));
  uint64_t maxnp = 0;
  for (uint32_t p = 0; p < nparts; p++) maxnp = std::max<uint64_t>(maxnp, hbase[p + 1] - hbase[p]);
  *parts_out = nparts;

  if (n) {
    const uint64_t ntiles64 = (n + OC_TILE - 1) / OC_TILE;
    const uint32_t ntiles = (uint32_t)ntiles64;
    const size_t ncounts = (size_t)nparts * ntiles;
    uint32_t *counts = nullptr, *scanned = nullptr, *scan32 = nullptr;
    GG_TRY(tmp.get(&counts, ncounts));
    GG_TRY(tmp.get(&scanned, ncounts + 1));
    GG_TRY(tmp.get(&scan32, scan_scratch_elems(ncounts) + 1));
    oc_count<<<oc_grid(n), OC_THREADS, 0, g->stream>>>(src, n, bounds, nparts, ntiles, counts);
    GG_CUDA(cudaGetLastError());
    GG_CUDA((exclusive_scan<uint32_t, ArrayIn<uint32_t>>(ArrayIn<uint32_t>{counts}, ncounts, scanned, scan32,
                                                         g->stream, nullptr)));
    // groups: consecutive ranges (at most OC_GROUP) holding at most gcap
    // entries together, compacted by one pass over the records
    std::vector<uint32_t> gstart{0};
    uint64_t gmax = 0, gsum = 0;
    for (uint32_t p = 0; p < nparts; p++) {
      const uint64_t np = hbase[p + 1] - hbase[p];
      if (p > gstart.back() && (p - gstart.back() == OC_GROUP || gsum + np > gcap)) {
        gstart.push_back(p);
        gsum = 0;
      }
      gsum += np;
      gmax = std::max(gmax, gsum);
    }
    gstart.push_back(nparts);
    *groups_out = (uint32_t)gstart.size() - 1;
    uint64_t *k0 = nullptr, *k1 = nullptr;
    uint32_t *v0 = nullptr, *v1 = nullptr;
    GG_TRY(tmp.get(&k0, gmax));
    GG_TRY(tmp.get(&k1, maxnp));
    if (g->weighted) {
      GG_TRY(tmp.get(&v0, gmax));
      GG_TRY(tmp.get(&v1, maxnp));
    }
    for (size_t gi = 0; gi + 1 < gstart.size(); gi++) {
      const uint32_t p0 = gstart[gi], p1 = gstart[gi + 1];
      const uint64_t gn = hbase[p1] - hbase[p0];
      if (gn == 0) continue;
      oc_scatter<<<ntiles, OC_THREADS, 0, g->stream>>>(src, n, bounds, base_dev, p0, p1 - p0, bits, scanned, counts,
                                                       ntiles, gn, k0, v0);
      GG_CUDA(cudaGetLastError());
      for (uint32_t p = p0; p < p1; p++) {
        const uint64_t np = hbase[p + 1] - hbase[p];
        if (np == 0) continue;
        const uint64_t at = hbase[p] - hbase[p0];
        uint64_t *ks;
        uint32_t *vs;
        GG_TRY(radix_sort(g, k0 + at, v0 ? v0 + at : nullptr, k1, v1, np, bits + bits_for(hb[p + 1] - hb[p]), &ks,
                          &vs));
        oc_emit<<<grid_for(np, 256, g->num_sms, 16), 256, 0, g->stream>>>(
            ks, vs, np, bits, d->nbr + hbase[p], d->w ? (uint32_t *)d->w + hbase[p] : nullptr);
        GG_CUDA(cudaGetLastError());
      }
    }
  }
  return finish_dir(g, d);
}

// Device bytes of the built graph (both directions, bins estimated at
// 12 B per vertex), without the adjacency when it lives on the host.
static uint64_t graph_estimate(uint32_t V, uint64_t n, int weighted, int symmetric, int adj_host) {
  const uint64_t npad = (n + 64) / 64 * 64;
  uint64_t per_dir = ((uint64_t)V + 1) * 12 + (uint64_t)V / 8 + (uint64_t)V * 12;
  if (!adj_host) per_dir += npad * 4 + (weighted ? n * 4 : 0);
  return per_dir * (symmetric ? 1 : 2);
}

// Chooses the build: in-core when its working set (records copied to the
// device unless already there, two key and value buffers, radix counts) fits
// the budget, else ranges of cap entries.  budget 0: free device memory less
// the graph and a reserve.
int build_plan(gg_graph *g, uint64_t E, bool rec_on_device, const gg_build_options *opt, bool *partitioned,
                      uint64_t *cap, uint64_t *gcap) {
  const uint64_t n = g->symmetric ? 2 * E : E;
  const uint64_t unit = g->weighted ? 12 : 8;
  const uint64_t in_core = (rec_on_device ? 0 : E * unit) + n * oc_entry_bytes(g->weighted);
  uint64_t budget = opt ? opt->build_budget : 0;
  if (budget == 0) {
    size_t free_b = 0, total_b = 0;
    GG_CUDA(cudaMemGetInfo(&free_b, &total_b));
    const uint64_t graph = graph_estimate(g->V, n, g->weighted, g->symmetric, g->adj_host);
    const uint64_t reserve = ((uint64_t)1 << 30) + total_b / 32;
    budget = free_b > graph + reserve ? free_b - graph - reserve : 0;
  }
  const bool force = opt && opt->force_partitions > 0;
  *partitioned = force || in_core > budget;
  *cap = 0;
  *gcap = 0;
  if (!*partitioned) return GG_OK;
  if (force) return GG_OK;
  // (range, tile) counts and their scan (8 B per tile and range) + the
  // offsets scan; then a group buffer of G entries (key + value) and one
  // range's sort buffer and digit counts, ranges of at most G/4 entries.
  // Greedy ranges of at most cap entries number at most 2n/cap + 1, so the
  // count table is sized for that many (at least 64), refined until the
  // table and cap agree: every pass that grows the table recomputes cap, and
  // the table only grows, up to OC_MAX_PARTS, so the loop ends.  (A list
  // longer than cap is still a range of its own, sorted in a buffer of its
  // length, which can exceed the budget.)
  const uint64_t tiles = (n + OC_TILE - 1) / OC_TILE;
  const uint64_t kv = 8 + (g->weighted ? 4 : 0);
  uint64_t ranges = 64;
  for (;;) {
    const uint64_t fixed = (uint64_t)g->V * 8 + tiles * 8 * ranges + (64ull << 20);
    const uint64_t avail = budget > fixed ? budget - fixed : 0;
    *gcap = avail * 4 / (4 * kv + kv + 1);
    *cap = *gcap / 4;
    if (*cap == 0) break;
    const uint64_t need = std::min<uint64_t>(2 * n / *cap + 1, OC_MAX_PARTS);
    if (need <= ranges) break;
    ranges = need;
  }
  if (*cap < (1ull << 16) && *cap < n) {
    set_error("build needs %llu device bytes beyond the graph; %llu available", (unsigned long long)in_core,
              (unsigned long long)budget);
    return GG_ERR_NOMEM;
  }
  return GG_OK;
}

// Builds both directions from E records readable by the device at rec.
int build_records(gg_graph *g, const uint32_t *rec, uint64_t E, bool partitioned, uint64_t cap,
                         uint64_t gcap, gg_build_options *opt) {
  if (opt) {
    opt->partitions = 1;
    opt->record_passes = 1;
  }
  if (!partitioned) return build_from_device_records(g, rec, E);
  g->E = E;
  const uint64_t n = g->symmetric ? 2 * E : E;
  g->nadj = n;
  if (n >= 0xFFFFFFFFull) {
    set_error("%llu adjacency entries per direction: the device sort supports < 2^32", (unsigned long long)n);
    return GG_ERR_TOO_LARGE;
  }
  const uint32_t force = opt && opt->force_partitions > 0 ? (uint32_t)opt->force_partitions : 0;
  uint32_t parts = 0, passes = 0;
  DevScratch tmp;
  GG_TRY(oc_alloc_dir(g, &g->out, n));
  if (!g->symmetric) GG_TRY(oc_alloc_dir(g, &g->in, n));
  if (!g->symmetric) {
    // out- and in-degrees from one pass over the records, into the graph's own arrays
    unsigned *err = nullptr;
    GG_TRY(tmp.get(&err, 1));
    GG_CUDA(cudaMemsetAsync(g->out.deg, 0, sizeof(uint32_t) * ((size_t)g->V + 1), g->stream));
    GG_CUDA(cudaMemsetAsync(g->in.deg, 0, sizeof(uint32_t) * ((size_t)g->V + 1), g->stream));
    GG_CUDA(cudaMemsetAsync(err, 0, sizeof(unsigned), g->stream));
    if (E) {
      oc_degree_both<<<oc_grid(E), OC_THREADS, 0, g->stream>>>(rec, E, g->weighted ? 3 : 2, g->V, g->out.deg, g->in.deg,
                                                          err);
      GG_CUDA(cudaGetLastError());
    }
    unsigned herr = 0;
    GG_CUDA(cudaMemcpyAsync(&herr, err, sizeof(unsigned), cudaMemcpyDeviceToHost, g->stream));
    GG_CUDA(cudaStreamSynchronize(g->stream));
    if (herr) {
      set_error("an edge names a vertex id >= vertices (%u)", g->V);
      return GG_ERR_RANGE;
    }
    passes += 1;
  }
  for (int pass = 0; pass < (g->symmetric ? 1 : 2); pass++) {
    const int mode = g->symmetric ? 2 : pass;
    uint32_t pp = 0, groups = 0;
    GG_TRY(build_dir_partitioned(g, rec, E, mode, pass == 0 ? &g->out : &g->in, cap, gcap, force, !g->symmetric,
                                 &pp, &groups));
    parts = std::max(parts, pp);
    // range counts and one compaction per group (and the degrees of a symmetric graph)
    passes += 1 + groups + (g->symmetric ? 1 : 0);
  }
  if (g->symmetric) g->in = g->out;
  if (opt) {
    opt->partitions = parts;
    opt->record_passes = passes;
  }
  return GG_OK;
}

}  // namespace gg
