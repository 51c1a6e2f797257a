// Seeded synthetic edge lists, shared by the host generator (C++ threads)
// and the device generator (CUDA).  Counter-based: record e depends only on
// (seed, e), so any range of records can be produced independently and the
// host file and the device buffer are bit-identical.
//
//   key          = mix64(seed ^ 0x5851F42D4C957F2D)
//   draw64(e, j) = mix64(key + (e * 64 + j) * 0x9E3779B97F4A7C15)   (mod 2^64)
//
// mix64 is the SplitMix64 finaliser (Steele, Lea, Flood, OOPSLA 2014).
// R-MAT (Chakrabarti, Zhan, Faloutsos, SDM 2004), a=0.57 b=0.19 c=0.19
// d=0.05: level l (most significant bit first) compares 32 bits of
// draw64(e, l/2) (low half for even l, high half for odd l) with
// floor(p * 2^32) thresholds; b sets the destination bit, c the source bit,
// d both.  Weight of record e: (low32(draw64(e, 16)) >> 8) * 2^-24, uniform
// on [0, 1) and exact in float.
// Grid n x n, vertex r*n+c: per vertex in row-major order the records
// (v,v+1),(v+1,v) when c+1<n, then (v,v+n),(v+n,v) when r+1<n.
#ifndef GG_GEN_H
#define GG_GEN_H

#include <stdint.h>

#if defined(__CUDACC__)
#define GG_HD __host__ __device__ __forceinline__
#else
#define GG_HD static inline
#endif

#define GG_RMAT_TA 2448131358u  /* floor(0.57 * 2^32) */
#define GG_RMAT_TAB 3264175144u /* floor(0.76 * 2^32) */
#define GG_RMAT_TABC 4080218931u /* floor(0.95 * 2^32) */

GG_HD uint64_t gg_mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

GG_HD uint64_t gg_gen_key(uint64_t seed) { return gg_mix64(seed ^ 0x5851F42D4C957F2Dull); }

GG_HD uint64_t gg_draw64(uint64_t key, uint64_t e, uint32_t j) {
  return gg_mix64(key + (e * 64u + j) * 0x9E3779B97F4A7C15ull);
}

GG_HD float gg_gen_weight(uint64_t key, uint64_t e) {
  uint32_t lo = (uint32_t)gg_draw64(key, e, 16);
  return (float)(lo >> 8) * (1.0f / 16777216.0f);
}

GG_HD void gg_rmat_edge(uint64_t key, uint32_t scale, uint64_t e, uint32_t *src, uint32_t *dst) {
  uint32_t s = 0, d = 0;
  uint64_t draw = 0;
  for (uint32_t l = 0; l < scale; l++) {
    if ((l & 1u) == 0) draw = gg_draw64(key, e, l >> 1);
    uint32_t u = (l & 1u) ? (uint32_t)(draw >> 32) : (uint32_t)draw;
    uint32_t sbit = u >= GG_RMAT_TAB ? 1u : 0u;
    uint32_t dbit = ((u >= GG_RMAT_TA && u < GG_RMAT_TAB) || u >= GG_RMAT_TABC) ? 1u : 0u;
    s |= sbit << (scale - 1 - l);
    d |= dbit << (scale - 1 - l);
  }
  *src = s;
  *dst = d;
}

// Grid record e of an n x n grid (n >= 2).  Vertex v = r*n+c owns
// 2*[c+1<n] + 2*[r+1<n] consecutive records; rows r < n-1 own 4n-2 records
// (4 per vertex except 2 for the last column), the last row 2(n-1).
GG_HD void gg_grid_edge(uint32_t n, uint64_t e, uint32_t *src, uint32_t *dst) {
  uint64_t per_row = 4ull * n - 2;
  uint64_t r = e / per_row;
  uint64_t k = e - r * per_row;
  uint64_t c, slot;
  if (r < (uint64_t)n - 1) {
    c = k / 4;
    slot = k - c * 4;
    if (c == (uint64_t)n - 1) slot += 2;  // last column: only the down pair
  } else {
    c = k / 2;
    slot = k - c * 2;  // last row: only the right pair
  }
  uint64_t v = r * n + c;
  uint64_t a, b;
  if (slot < 2) { a = v; b = v + 1; } else { a = v; b = v + n; }
  if (slot & 1) { uint64_t t = a; a = b; b = t; }
  *src = (uint32_t)a;
  *dst = (uint32_t)b;
}

GG_HD uint64_t gg_grid_count(uint32_t n) { return n < 2 ? 0 : 4ull * n * (n - 1); }

#endif
