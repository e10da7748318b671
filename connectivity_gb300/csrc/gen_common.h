// Seeded synthetic-graph primitives shared by the host and the device
// generators, so that a graph built on the GPU and the same graph built on
// the CPU are identical edge for edge.
//
// Only integer arithmetic is used here: the R-MAT quadrant choice compares a
// 32-bit random word with integer thresholds, so no floating-point rounding
// can differ between x86-64, aarch64 and the GPU.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define GB_HD __host__ __device__ __forceinline__
#else
#define GB_HD static inline
#endif

// splitmix64 finaliser (Steele, Lea and Flood, "Fast splittable pseudorandom
// number generators", OOPSLA 2014).
GB_HD uint64_t gb_mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// Counter-based random word for (seed, i, j): a pure function, so edge i can
// be generated by any thread in any order.
GB_HD uint64_t gb_rand64(uint64_t seed, uint64_t i, uint64_t j) {
  return gb_mix64(gb_mix64(seed ^ (i * 0xD1B54A32D192ED03ull)) ^
                  (j * 0x8CB92BA72F3D8DD7ull));
}

// R-MAT thresholds as 32-bit fixed point: quadrant (0,0) if r < ta, (0,1) if
// r < tab, (1,0) if r < tabc, else (1,1).
typedef struct gb_rmat_thr {
  uint32_t ta, tab, tabc;
} gb_rmat_thr;

// Edge i of an R-MAT graph with 2^scale vertices: one 32-bit word per
// recursion level, most significant bit first.
GB_HD void gb_rmat_edge(uint64_t seed, uint64_t i, int scale, gb_rmat_thr t,
                        uint32_t* src, uint32_t* dst) {
  uint32_t s = 0, d = 0;
  uint64_t r = 0;
  for (int l = 0; l < scale; ++l) {
    if ((l & 1) == 0) r = gb_rand64(seed, i, (uint64_t)(l >> 1));
    uint32_t w = (l & 1) ? (uint32_t)(r >> 32) : (uint32_t)r;
    uint32_t sb = w >= t.tab;                       // lower half: (1,0),(1,1)
    uint32_t db = (w >= t.ta && w < t.tab) || w >= t.tabc;  // right: (0,1),(1,1)
    s = (s << 1) | sb;
    d = (d << 1) | db;
  }
  *src = s;
  *dst = d;
}

// Orientation of lattice edge (u, v): 0 = u->v, 1 = v->u, 2 = both, 3 = none,
// each with probability 1/4.
GB_HD uint32_t gb_grid_orient(uint64_t seed, uint64_t u, uint32_t axis) {
  return (uint32_t)(gb_rand64(seed ^ 0x6A09E667F3BCC909ull, u, axis) >> 62);
}
