/*
 * oracle/gen.c -- seeded R-MAT edge lists for the CPU side of the checks.
 *
 * TEST INFRASTRUCTURE ONLY.  The reference arm of the benchmark and the CPU
 * baselines generate their graphs here, so that timing the reference never
 * loads the product library.  The edges equal the product's generator's
 * (tests compare the digests); the construction is independent of it: edges
 * are bucketed by source with a counting pass, then each bucket is sorted
 * and de-duplicated on its own, where the product sorts 64-bit keys.
 *
 * The graph: edge_factor * n candidate edges i = 0 .. m0-1 drawn at scale
 * ceil(log2 n).  Each recursion level l (most significant bit first) uses one
 * 32-bit word: the low half of R(seed, i, l/2) for even l, its high half for
 * odd l, where R(seed, i, j) = mix(mix(seed ^ i*K1) ^ j*K2) and mix is the
 * splitmix64 finaliser (Steele, Lea and Flood, OOPSLA 2014).  The word w
 * picks quadrant (0,0) when w < A, (0,1) when w < A+B, (1,0) when
 * w < A+B+C, else (1,1), with A, A+B, A+B+C the probabilities in 32-bit
 * fixed point (rounded to nearest, clamped at 2^32-1).  Self-loops, ids >= n
 * and duplicates are dropped; the list is sorted by (source, target).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <omp.h>

static inline uint64_t orc_mix(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

static inline uint64_t orc_word64(uint64_t seed, uint64_t i, uint64_t j) {
  return orc_mix(orc_mix(seed ^ (i * 0xD1B54A32D192ED03ull)) ^ (j * 0x8CB92BA72F3D8DD7ull));
}

static uint32_t orc_fixed32(double x) {
  if (x <= 0.0) return 0u;
  double v = x * 4294967296.0;
  if (v >= 4294967295.0) return 4294967295u;
  return (uint32_t)(v + 0.5);
}

static void orc_rmat_pair(uint64_t seed, uint64_t i, int scale, uint32_t ta, uint32_t tab,
                          uint32_t tabc, uint32_t* src, uint32_t* dst) {
  uint32_t s = 0, d = 0;
  uint64_t r = 0;
  for (int l = 0; l < scale; ++l) {
    if ((l & 1) == 0) r = orc_word64(seed, i, (uint64_t)(l >> 1));
    const uint32_t w = (l & 1) ? (uint32_t)(r >> 32) : (uint32_t)r;
    uint32_t row, col;
    if (w < ta) { row = 0; col = 0; }
    else if (w < tab) { row = 0; col = 1; }
    else if (w < tabc) { row = 1; col = 0; }
    else { row = 1; col = 1; }
    s = (s << 1) | row;
    d = (d << 1) | col;
  }
  *src = s;
  *dst = d;
}

static int cmp_i32(const void* a, const void* b) {
  const int32_t x = *(const int32_t*)a, y = *(const int32_t*)b;
  return (x > y) - (x < y);
}

/* R-MAT edge list on n vertices (see the file header).  *src / *dst are
 * malloc'd (free with orc_free).  Returns 0, or -1 on bad arguments or a
 * failed allocation. */
int orc_rmat_edges(int32_t n, int32_t edge_factor, uint64_t seed, double a, double b, double c,
                   int64_t* m_out, int32_t** src_out, int32_t** dst_out) {
  if (n < 1 || edge_factor < 1 || !m_out || !src_out || !dst_out) return -1;
  int scale = 1;
  while (scale < 31 && (1ll << scale) < (long long)n) ++scale;
  const int64_t m0 = (int64_t)edge_factor * n;
  const uint32_t ta = orc_fixed32(a), tab = orc_fixed32(a + b), tabc = orc_fixed32(a + b + c);
  const int nt = omp_get_max_threads();
  int64_t* cnt = (int64_t*)calloc((size_t)n + 1, sizeof(int64_t));
  int32_t* bucket = (int32_t*)malloc((size_t)(m0 > 0 ? m0 : 1) * sizeof(int32_t));
  if (!cnt || !bucket) { free(cnt); free(bucket); return -1; }
  /* pass 1: out-degree of every source among the kept candidates */
#pragma omp parallel for schedule(static) num_threads(nt)
  for (int64_t i = 0; i < m0; ++i) {
    uint32_t s, d;
    orc_rmat_pair(seed, (uint64_t)i, scale, ta, tab, tabc, &s, &d);
    if (s != d && s < (uint32_t)n && d < (uint32_t)n)
      __atomic_fetch_add(&cnt[s + 1], 1, __ATOMIC_RELAXED);
  }
  for (int32_t v = 0; v < n; ++v) cnt[v + 1] += cnt[v];
  int64_t* fill = (int64_t*)malloc((size_t)n * sizeof(int64_t));
  if (!fill) { free(cnt); free(bucket); return -1; }
  memcpy(fill, cnt, (size_t)n * sizeof(int64_t));
  /* pass 2: targets into their source's bucket (any order) */
#pragma omp parallel for schedule(static) num_threads(nt)
  for (int64_t i = 0; i < m0; ++i) {
    uint32_t s, d;
    orc_rmat_pair(seed, (uint64_t)i, scale, ta, tab, tabc, &s, &d);
    if (s != d && s < (uint32_t)n && d < (uint32_t)n) {
      const int64_t at = __atomic_fetch_add(&fill[s], 1, __ATOMIC_RELAXED);
      bucket[at] = (int32_t)d;
    }
  }
  /* each bucket sorted and de-duplicated in place; kept counts in fill[] */
#pragma omp parallel for schedule(dynamic, 4096) num_threads(nt)
  for (int32_t v = 0; v < n; ++v) {
    int32_t* p = bucket + cnt[v];
    const int64_t len = cnt[v + 1] - cnt[v];
    if (len > 1) qsort(p, (size_t)len, sizeof(int32_t), cmp_i32);
    int64_t k = 0;
    for (int64_t j = 0; j < len; ++j)
      if (k == 0 || p[k - 1] != p[j]) p[k++] = p[j];
    fill[v] = k;
  }
  int64_t* at = (int64_t*)malloc(((size_t)n + 1) * sizeof(int64_t));
  if (!at) { free(cnt); free(fill); free(bucket); return -1; }
  at[0] = 0;
  for (int32_t v = 0; v < n; ++v) at[v + 1] = at[v] + fill[v];
  const int64_t m = at[n];
  int32_t* s = (int32_t*)malloc((size_t)(m > 0 ? m : 1) * sizeof(int32_t));
  int32_t* d = (int32_t*)malloc((size_t)(m > 0 ? m : 1) * sizeof(int32_t));
  if (!s || !d) { free(s); free(d); free(cnt); free(fill); free(bucket); free(at); return -1; }
#pragma omp parallel for schedule(dynamic, 4096) num_threads(nt)
  for (int32_t v = 0; v < n; ++v) {
    const int32_t* p = bucket + cnt[v];
    for (int64_t j = 0; j < fill[v]; ++j) {
      s[at[v] + j] = v;
      d[at[v] + j] = p[j];
    }
  }
  free(cnt); free(fill); free(bucket); free(at);
  *m_out = m;
  *src_out = s;
  *dst_out = d;
  return 0;
}

void orc_free(void* p) { free(p); }
