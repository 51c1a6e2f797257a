// Device-wide exclusive scan (three phases, no inter-block waiting) and the
// block-level scan it is built from.
#ifndef GG_SCAN_CUH
#define GG_SCAN_CUH

#include "gg_common.cuh"

namespace gg {

constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 8;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

template <typename T>
struct ArrayIn {
  const T *p;
  __device__ __forceinline__ T operator()(size_t i) const { return p[i]; }
};

// Degree of queue entry i: deg[q[i]].
struct QueueDegreeIn {
  const uint32_t *q;
  const uint32_t *deg;
  __device__ __forceinline__ unsigned long long operator()(size_t i) const {
    return (unsigned long long)deg[q[i]];
  }
};

// Exclusive block scan of one value per thread; returns the block total.
// Every thread of the block must call it.
template <typename T>
__device__ __forceinline__ T block_exclusive_scan(T x, T *excl) {
  constexpr int NW = SCAN_THREADS / 32;
  __shared__ T s_warp[NW + 1];
  unsigned lane = lane_id(), w = threadIdx.x >> 5;
  T incl = x;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T y = __shfl_up_sync(GG_FULL, incl, o);
    if (lane >= (unsigned)o) incl += y;
  }
  if (lane == 31) s_warp[w] = incl;
  __syncthreads();
  if (threadIdx.x == 0) {
    T run = 0;
#pragma unroll
    for (int i = 0; i < NW; i++) {
      T t = s_warp[i];
      s_warp[i] = run;
      run += t;
    }
    s_warp[NW] = run;
  }
  __syncthreads();
  *excl = s_warp[w] + incl - x;
  T total = s_warp[NW];
  __syncthreads();
  return total;
}

template <typename T, typename In>
__global__ void __launch_bounds__(SCAN_THREADS) scan_reduce_tiles(In in, size_t n, T *tile_sums) {
  size_t base = (size_t)blockIdx.x * SCAN_TILE + (size_t)threadIdx.x * SCAN_ITEMS;
  T s = 0;
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; k++) {
    size_t i = base + k;
    if (i < n) s += in(i);
  }
  T excl;
  T tot = block_exclusive_scan<T>(s, &excl);
  if (threadIdx.x == 0) tile_sums[blockIdx.x] = tot;
}

template <typename T, typename In>
__global__ void __launch_bounds__(SCAN_THREADS) scan_tiles(In in, size_t n, const T *tile_offsets, T *out) {
  size_t base = (size_t)blockIdx.x * SCAN_TILE + (size_t)threadIdx.x * SCAN_ITEMS;
  T v[SCAN_ITEMS];
  T s = 0;
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; k++) {
    size_t i = base + k;
    v[k] = i < n ? in(i) : T(0);
    s += v[k];
  }
  T excl;
  T tot = block_exclusive_scan<T>(s, &excl);
  T off = tile_offsets ? tile_offsets[blockIdx.x] : T(0);
  T run = off + excl;
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; k++) {
    size_t i = base + k;
    if (i < n) out[i] = run;
    run += v[k];
  }
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) out[n] = off + tot;
}

// The same two tile kernels with the element count n in device memory (a
// step of a captured loop, whose length the host does not see): launched
// over n_max / SCAN_TILE + 1 tiles; tiles past n add 0 and return at once,
// and the tile holding index n writes out[n].
template <typename T, typename In>
__global__ void __launch_bounds__(SCAN_THREADS) scan_reduce_tiles_dn(In in, const uint32_t *n_dev, T *tile_sums) {
  const size_t n = *n_dev;
  const size_t base = (size_t)blockIdx.x * SCAN_TILE + (size_t)threadIdx.x * SCAN_ITEMS;
  if ((size_t)blockIdx.x * SCAN_TILE >= n) {
    if (threadIdx.x == 0) tile_sums[blockIdx.x] = 0;
    return;
  }
  T s = 0;
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; k++) {
    size_t i = base + k;
    if (i < n) s += in(i);
  }
  T excl;
  T tot = block_exclusive_scan<T>(s, &excl);
  if (threadIdx.x == 0) tile_sums[blockIdx.x] = tot;
}

template <typename T, typename In>
__global__ void __launch_bounds__(SCAN_THREADS) scan_tiles_dn(In in, const uint32_t *n_dev, const T *tile_offsets,
                                                              T *out) {
  const size_t n = *n_dev;
  if ((size_t)blockIdx.x * SCAN_TILE > n) return;
  const size_t base = (size_t)blockIdx.x * SCAN_TILE + (size_t)threadIdx.x * SCAN_ITEMS;
  T v[SCAN_ITEMS];
  T s = 0;
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; k++) {
    size_t i = base + k;
    v[k] = i < n ? in(i) : T(0);
    s += v[k];
  }
  T excl;
  T tot = block_exclusive_scan<T>(s, &excl);
  T off = tile_offsets ? tile_offsets[blockIdx.x] : T(0);
  T run = off + excl;
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; k++) {
    size_t i = base + k;
    if (i < n) out[i] = run;
    run += v[k];
  }
  if (blockIdx.x == n / SCAN_TILE && threadIdx.x == 0) out[n] = off + tot;
}

inline size_t scan_scratch_elems_impl(size_t n) {
  size_t tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
  if (tiles <= 1) return 0;
  return 2 * tiles + 1 + scan_scratch_elems_impl(tiles);
}

template <typename T, typename In>
cudaError_t exclusive_scan(In in, size_t n, T *out, T *scratch, cudaStream_t s, int *launches) {
  size_t tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
  if (tiles == 0) tiles = 1;
  if (tiles == 1) {
    scan_tiles<T, In><<<1, SCAN_THREADS, 0, s>>>(in, n, nullptr, out);
    if (launches) *launches += 1;
    return cudaGetLastError();
  }
  T *sums = scratch;
  T *offs = scratch + tiles;
  scan_reduce_tiles<T, In><<<(unsigned)tiles, SCAN_THREADS, 0, s>>>(in, n, sums);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  e = exclusive_scan<T, ArrayIn<T>>(ArrayIn<T>{sums}, tiles, offs, scratch + 2 * tiles + 1, s, launches);
  if (e != cudaSuccess) return e;
  scan_tiles<T, In><<<(unsigned)tiles, SCAN_THREADS, 0, s>>>(in, n, offs, out);
  if (launches) *launches += 2;
  return cudaGetLastError();
}

// Exclusive scan of in(i) for i < *n_dev (at most n_max) into out[0..n]:
// the launch shape depends on n_max only, so it can be captured once and
// replayed for any n.  scratch must hold scan_scratch_elems(n_max + 1).
template <typename T, typename In>
cudaError_t exclusive_scan_dn(In in, const uint32_t *n_dev, size_t n_max, T *out, T *scratch, cudaStream_t s,
                              int *launches) {
  const size_t tiles = n_max / SCAN_TILE + 1;
  if (tiles == 1) {
    scan_tiles_dn<T, In><<<1, SCAN_THREADS, 0, s>>>(in, n_dev, nullptr, out);
    if (launches) *launches += 1;
    return cudaGetLastError();
  }
  T *sums = scratch;
  T *offs = scratch + tiles;
  scan_reduce_tiles_dn<T, In><<<(unsigned)tiles, SCAN_THREADS, 0, s>>>(in, n_dev, sums);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  e = exclusive_scan<T, ArrayIn<T>>(ArrayIn<T>{sums}, tiles, offs, scratch + 2 * tiles + 1, s, launches);
  if (e != cudaSuccess) return e;
  scan_tiles_dn<T, In><<<(unsigned)tiles, SCAN_THREADS, 0, s>>>(in, n_dev, offs, out);
  if (launches) *launches += 2;
  return cudaGetLastError();
}

}  // namespace gg

#endif
