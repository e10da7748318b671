// Device CSR construction (create_csr, multistep/scc_main.cpp:127-191) and the
// device R-MAT generator.
//
// The reference builds its CSR with a serial counting sort that keeps the
// input order of each vertex's edges.  Here the same order comes from a
// stable LSD radix sort of (key = endpoint, value = other endpoint) pairs
// (CUB DeviceRadixSort, a library sort: construction is outside the timed
// region, as in the reference), followed by an offsets kernel that writes
// off[v] at every boundary of the sorted keys.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_select.cuh>

#include "gb_internal.cuh"
#include "gen_common.h"

#include <algorithm>
#include <cstring>

namespace gb {
namespace {

__global__ void k_check_ids(const int32_t* a, const int32_t* b, int64_t m, int32_t n, int* bad) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t x = a[i], y = b[i];
    if (x < 0 || x >= n || y < 0 || y >= n) {
      atomicOr(bad, 1);
      return;
    }
  }
}

// off[v] = first index i with key[i] >= v, for v in [0, n]; keys sorted.
__global__ void k_offsets(const uint32_t* key, int64_t m, int32_t n, int64_t* off) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i <= m;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t prev = i == 0 ? -1 : (int64_t)key[i - 1];
    const int64_t cur = i == m ? (int64_t)n : (int64_t)key[i];
    for (int64_t v = prev + 1; v <= cur; ++v) off[v] = i;
  }
}

__global__ void k_widen(const uint32_t* in, int64_t* out, int64_t count) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (int64_t)in[i];
}

__global__ void k_rmat_keys(uint64_t seed, int64_t m0, int scale, uint32_t n, gb_rmat_thr thr,
                            uint64_t self, uint64_t* keys) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m0;
       i += (int64_t)gridDim.x * blockDim.x) {
    uint32_t s, d;
    gb_rmat_edge(seed, (uint64_t)i, scale, thr, &s, &d);
    keys[i] = (s == d || s >= n || d >= n) ? self : (((uint64_t)s << scale) | d);
  }
}

// Batch generator: edge index i of the concatenation of every graph's ef*n
// candidate edges.  Each thread walks a run of kRun consecutive indices,
// locating its graph once.  Keys hold global ids.
constexpr int kRun = 64;
__global__ void k_batch_keys(int64_t etotal, const int64_t* ebase, const int64_t* vbase,
                             const int32_t* nv, const int32_t* scale, const uint64_t* seeds,
                             int32_t count, gb_rmat_thr thr, int id_bits, uint64_t* keys) {
  const uint64_t self = (1ull << (2 * id_bits)) - 1ull;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r * kRun < etotal;
       r += (int64_t)gridDim.x * blockDim.x) {
    int64_t i = r * kRun;
    const int64_t end = i + kRun < etotal ? i + kRun : etotal;
    int lo = 0, hi = count;  // last graph with ebase[g] <= i
    while (hi - lo > 1) {
      const int mid = (lo + hi) / 2;
      if (ebase[mid] <= i) lo = mid; else hi = mid;
    }
    int gr = lo;
    for (; i < end; ++i) {
      while (gr + 1 < count && ebase[gr + 1] <= i) ++gr;
      uint32_t s, d;
      gb_rmat_edge(seeds[gr], (uint64_t)(i - ebase[gr]), scale[gr], thr, &s, &d);
      const uint32_t n = (uint32_t)nv[gr];
      if (s == d || s >= n || d >= n) {
        keys[i] = self;
      } else {
        const uint64_t vb = (uint64_t)vbase[gr];
        keys[i] = ((vb + s) << id_bits) | (vb + d);
      }
    }
  }
}

__global__ void k_split_bits(const uint64_t* keys, int64_t m, int id_bits, int32_t* src,
                             int32_t* dst) {
  const uint64_t mask = (1ull << id_bits) - 1ull;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m;
       i += (int64_t)gridDim.x * blockDim.x) {
    src[i] = (int32_t)(keys[i] >> id_bits);
    dst[i] = (int32_t)(keys[i] & mask);
  }
}

__global__ void k_fill_gid(int32_t n, const int64_t* vbase, int32_t count, int32_t* gid) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (int64_t)gridDim.x * blockDim.x) {
    int lo = 0, hi = count;
    while (hi - lo > 1) {
      const int mid = (lo + hi) / 2;
      if (vbase[mid] <= v) lo = mid; else hi = mid;
    }
    gid[v] = lo;
  }
}

// Every edge must stay inside its graph.
__global__ void k_check_within(const int32_t* s, const int32_t* d, int64_t m, const int32_t* gid,
                               int* bad) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m;
       i += (int64_t)gridDim.x * blockDim.x)
    if (gid[s[i]] != gid[d[i]]) atomicOr(bad, 1);
}

__global__ void k_max_degree(int32_t n, const int64_t* off, unsigned long long* out) {
  unsigned long long best = 0;
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (int64_t)gridDim.x * blockDim.x) {
    const unsigned long long d = (unsigned long long)(off[v + 1] - off[v]);
    if (d > best) best = d;
  }
  if (best) atomicMax(out, best);
}

__global__ void k_split(const uint64_t* keys, int64_t m, int scale, int32_t* src, int32_t* dst) {
  const uint64_t mask = (1ull << scale) - 1ull;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m;
       i += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t k = keys[i];
    src[i] = (int32_t)(k >> scale);
    dst[i] = (int32_t)(k & mask);
  }
}

__global__ void k_check_csr(int32_t n, int64_t m, const int64_t* off, const int32_t* adj, int* bad) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  for (int64_t v = t0; v <= n; v += stride) {
    const int64_t o = off[v];
    if ((v == 0 && o != 0) || (v == n && o != m) || (v < n && off[v + 1] < o)) atomicOr(bad, 1);
  }
  for (int64_t e = t0; e < m; e += stride) {
    const int32_t x = adj[e];
    if (x < 0 || x >= n) atomicOr(bad, 1);
  }
}

// Every id of adj[0, count) in [0, n).
__global__ void k_check_adj_ids(const int32_t* __restrict__ adj, int64_t count, int32_t n,
                                int* bad) {
  bool ok = true;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < count;
       e += (int64_t)gridDim.x * blockDim.x)
    ok = ok && (uint32_t)adj[e] < (uint32_t)n;
  if (!__all_sync(0xffffffffu, ok) && (threadIdx.x & 31) == 0) atomicOr(bad, 1);
}

// Ingest of the reference's 32-bit CSR from host memory the device reads
// directly (pinned): offsets are widened to int64 and checked (off[0] == 0,
// off[n] == m, non-decreasing), ids are checked against [0, n), in the same
// pass that moves the bytes, so the host link is crossed once and nothing
// is read again on the device.
__global__ void k_ingest_off(const uint32_t* __restrict__ h, int64_t* __restrict__ d, int32_t n,
                             int64_t m, int* bad) {
  const int lane = threadIdx.x & 31;
  for (int64_t base = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) & ~(int64_t)31; base <= n;
       base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = base + lane;
    const uint32_t x = i <= n ? h[i] : 0u;
    uint32_t nx = __shfl_down_sync(0xffffffffu, x, 1);
    if (lane == 31 && i + 1 <= n) nx = h[i + 1];
    if (i <= n) {
      d[i] = (int64_t)x;
      if ((i == 0 && x != 0u) || (i == n && (int64_t)x != m) || (i < n && nx < x)) atomicOr(bad, 1);
    }
  }
}
__global__ void k_ingest_adj(const int32_t* __restrict__ h, int32_t* __restrict__ d, int64_t m,
                             int32_t n, int* bad) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  bool ok = true;
  if (((reinterpret_cast<uintptr_t>(h) | reinterpret_cast<uintptr_t>(d)) & 15u) == 0u) {
    const int64_t m4 = m / 4;
    const int4* h4 = reinterpret_cast<const int4*>(h);
    int4* d4 = reinterpret_cast<int4*>(d);
    for (int64_t i = t0; i < m4; i += stride) {
      const int4 v = h4[i];
      d4[i] = v;
      ok = ok && (uint32_t)v.x < (uint32_t)n && (uint32_t)v.y < (uint32_t)n &&
           (uint32_t)v.z < (uint32_t)n && (uint32_t)v.w < (uint32_t)n;
    }
    for (int64_t e = m4 * 4 + t0; e < m; e += stride) {
      const int32_t v = h[e];
      d[e] = v;
      ok = ok && (uint32_t)v < (uint32_t)n;
    }
  } else {
    for (int64_t e = t0; e < m; e += stride) {
      const int32_t v = h[e];
      d[e] = v;
      ok = ok && (uint32_t)v < (uint32_t)n;
    }
  }
  if (!__all_sync(0xffffffffu, ok) && (threadIdx.x & 31) == 0) atomicOr(bad, 1);
}

// ---------------------------------------------------------------------------
// In-lists derived from the out-CSR.
//
// The reference's run_scc takes both CSRs of the graph (graph struct,
// multistep/scc_main.cpp:75-86, both built by create_csr, :127-191).  The
// in-CSR is the out-CSR transposed, so a caller that hands over both moves
// every edge across the host link twice.  Here only the out-CSR and the
// in-offsets cross it: k_place_in reads the out-adjacency in tiles of kTile
// edges (from host memory the device maps, or from device memory), stores
// it, finds each edge's source by a max-scan of the tile's list heads, and
// writes the source into the target's in-list at the next free slot (an
// atomic on a per-vertex cursor that starts at the list's first slot).
// Targets with at least kHubDeg in-edges (a bitmap made with the offsets)
// take their slots once per tile: the tile's edges to them are counted in a
// shared hash table, one atomic per (tile, target) reserves a run of slots
// and the edges take consecutive slots of it, so a hub with hundreds of
// thousands of in-edges sees one atomic per tile instead of one per edge.
// Each block loads its next tile before it works on the current one, so the
// host link stays busy while the block places edges.
//
// The order within an in-list is the order of the atomics, not the caller's
// (no label depends on it).  Slots stay below m, so no write leaves the
// array; in-offsets that are not those of the out-CSR's transpose leave some
// cursor off its list's end, which k_check_cursors reports (*bad).  With
// every cursor at its list's end, every vertex received exactly its
// in-degree of placements, all inside its own list.
// ---------------------------------------------------------------------------
constexpr int kPT = 256;                 // threads per block
constexpr int kPE = 8;                   // edges per thread
constexpr int kTile = kPT * kPE;         // edges per tile
constexpr uint32_t kHubDeg = 2048;       // in-degree from which slots are reserved per tile
constexpr int kHashBits = 9;
constexpr int kHash = 1 << kHashBits;    // shared hash entries
constexpr int kProbe = 8;                // linear probes before the per-edge atomic
constexpr uint32_t kNoSlot = 0xffffffffu;

// Tile position of a thread's edge k: two runs of four consecutive edges, so
// the tile is read as 16-byte words with consecutive threads on consecutive
// words.
__device__ __forceinline__ int tile_pos(int k) {
  return (k >> 2) * 4 * kPT + 4 * (int)threadIdx.x + (k & 3);
}

// In-offsets: widened into off (int64), cursor[v] = off[v] (each list's
// first free slot), hub bit of v = in-degree >= kHubDeg; checked as
// k_ingest_off checks.
__global__ void k_ingest_in_off(const uint32_t* __restrict__ h, int32_t n, int64_t m,
                                int64_t* __restrict__ off, uint32_t* __restrict__ cursor,
                                uint32_t* __restrict__ hub_bits, int* bad) {
  const int lane = threadIdx.x & 31;
  for (int64_t base = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) & ~(int64_t)31; base <= n;
       base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = base + lane;
    const uint32_t x = i <= n ? h[i] : 0u;
    uint32_t nx = __shfl_down_sync(0xffffffffu, x, 1);
    if (lane == 31 && i + 1 <= n) nx = h[i + 1];
    const unsigned hub = __ballot_sync(0xffffffffu, i < n && nx >= x && nx - x >= kHubDeg);
    if (lane == 0 && base < n) hub_bits[base >> 5] = hub;
    if (i <= n) {
      off[i] = (int64_t)x;
      if (i < n) cursor[i] = x;
      if ((i == 0 && x != 0u) || (i == n && (int64_t)x != m) || (i < n && nx < x)) atomicOr(bad, 1);
    }
  }
}

// tile_src[t] = the vertex whose out-list holds edge t * kTile.  Skipped once
// the offsets were found bad; indexes stay below `tiles` whatever they hold.
__global__ void k_tile_heads(int32_t n, int64_t tiles, const int64_t* __restrict__ off,
                             int32_t* __restrict__ tile_src, const int* bad) {
  if (*(volatile const int*)bad) return;
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < n;
       u += (int64_t)gridDim.x * blockDim.x) {
    const int64_t a = off[u], b = off[u + 1];
    if (a < 0) continue;
    for (int64_t t = (a + kTile - 1) / kTile; t < tiles && t * kTile < b; ++t)
      tile_src[t] = (int32_t)u;
  }
}

// Every cursor must have reached its list's end.
__global__ void k_check_cursors(int32_t n, const int64_t* __restrict__ off,
                                const uint32_t* __restrict__ cursor, int* bad) {
  bool ok = true;
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (int64_t)gridDim.x * blockDim.x)
    ok = ok && (int64_t)cursor[v] == off[v + 1];
  if (!__all_sync(0xffffffffu, ok) && (threadIdx.x & 31) == 0) atomicOr(bad, 1);
}

__global__ void __launch_bounds__(kPT) k_place_in(
    const int32_t* __restrict__ src_adj, int32_t* __restrict__ out_adj, int64_t m, int32_t n,
    const int64_t* __restrict__ out_off, const uint32_t* __restrict__ hub_bits,
    uint32_t* __restrict__ cursor, const int32_t* __restrict__ tile_src,
    int32_t* __restrict__ in_adj, int32_t t_split, const int32_t* __restrict__ src_in,
    int64_t tail0, int* bad) {
  __shared__ int32_t head[kTile];
  __shared__ int32_t hkey[kHash];
  __shared__ uint32_t hval[kHash];  // a target's edge count in the tile, then its first slot
  __shared__ int32_t wmax[kPT / 32];
  __shared__ int s_skip;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  // bad offsets (either CSR): nothing is placed, nothing is indexed by them
  if (tid == 0) s_skip = *(volatile const int*)bad;
  __syncthreads();
  if (s_skip) return;
  // Placement tiles (the out-adjacency) and copy tiles (the in-lists from
  // tail0 on, copied as given) are interleaved evenly in one tile order, so
  // the blocks mix device-bound placement with link-bound copies.  Copy
  // tiles start at the first multiple of four from tail0; the elements
  // before it go with copy tile 0.
  const int64_t P = (m + kTile - 1) / kTile;
  const int64_t ca = tail0 < m ? ((tail0 + 3) & ~(int64_t)3) : m;
  const int64_t Q = ca < m ? (m - ca + kTile - 1) / kTile : 0;
  const int64_t U = P + Q;
  const bool vec =
      ((reinterpret_cast<uintptr_t>(src_adj) | reinterpret_cast<uintptr_t>(out_adj)) & 15u) == 0;
  const bool tvec = Q > 0 && ((reinterpret_cast<uintptr_t>(src_in + ca) |
                               reinterpret_cast<uintptr_t>(in_adj + ca)) & 15u) == 0;
  const bool store = src_adj != out_adj;
  const uint32_t slot_cap = (uint32_t)m;
  bool ok = true;
  // tile u: a copy tile when the even interleave puts one there
  auto kind_of = [&](int64_t u, bool& copy, int64_t& t, int64_t& e0, int& len, bool& full,
                     const int32_t*& src) {
    const int64_t cq = Q ? u * Q / U : 0;
    copy = Q && (u + 1) * Q / U > cq;
    t = copy ? cq : u - cq;
    e0 = copy ? ca + t * kTile : t * kTile;
    len = (int)(m - e0 < kTile ? m - e0 : kTile);
    full = len == kTile && (copy ? tvec : vec);
    src = (copy ? src_in : src_adj) + e0;
  };
  int64_t u = blockIdx.x;
  // the next full tile's words, loaded one tile ahead
  int4 n0 = make_int4(0, 0, 0, 0), n1 = n0;
  if (u < U) {
    bool cp, fl;
    int64_t tt, ee;
    int ll;
    const int32_t* sp;
    kind_of(u, cp, tt, ee, ll, fl, sp);
    if (fl) {
      n0 = reinterpret_cast<const int4*>(sp)[tid];
      n1 = reinterpret_cast<const int4*>(sp)[kPT + tid];
    }
  }
  for (; u < U; u += gridDim.x) {
    bool copy, full;
    int64_t t, e0;
    int len;
    const int32_t* src;
    kind_of(u, copy, t, e0, len, full, src);
    // 1. the tile's words
    int32_t w[kPE];
    if (full) {
      const int4 q0 = n0, q1 = n1;
      if (u + gridDim.x < U) {
        bool cp, fl;
        int64_t tt, ee;
        int ll;
        const int32_t* sp;
        kind_of(u + gridDim.x, cp, tt, ee, ll, fl, sp);
        if (fl) {
          n0 = reinterpret_cast<const int4*>(sp)[tid];
          n1 = reinterpret_cast<const int4*>(sp)[kPT + tid];
        }
      }
      if (copy || store) {
        int4* d4 = reinterpret_cast<int4*>((copy ? in_adj : out_adj) + e0);
        __stcs(d4 + tid, q0);
        __stcs(d4 + kPT + tid, q1);
      }
      w[0] = q0.x; w[1] = q0.y; w[2] = q0.z; w[3] = q0.w;
      w[4] = q1.x; w[5] = q1.y; w[6] = q1.z; w[7] = q1.w;
    } else {
      int32_t* dst = (copy ? in_adj : out_adj) + e0;
#pragma unroll
      for (int k = 0; k < kPE; ++k) {
        const int p = tile_pos(k);
        w[k] = p < len ? src[p] : 0;
        if (p < len && (copy || store)) dst[p] = w[k];
      }
    }
    if (copy) {
      // ids of copied in-lists are checked here; copy tile 0 also takes the
      // elements from tail0 up to the first copy tile
#pragma unroll
      for (int k = 0; k < kPE; ++k)
        if (tile_pos(k) < len && (uint32_t)w[k] >= (uint32_t)n) ok = false;
      if (t == 0 && tid < ca - tail0) {
        const int32_t x = src_in[tail0 + tid];
        in_adj[tail0 + tid] = x;
        if ((uint32_t)x >= (uint32_t)n) ok = false;
      }
      continue;
    }
    // 2. sources: every out-list starting inside the tile marks its first
    // position, the list holding edge e0 marks position 0; a max-scan then
    // gives every position its list's vertex
    for (int i = tid; i < kTile; i += kPT) head[i] = -1;
    for (int i = tid; i < kHash; i += kPT) {
      hkey[i] = -1;
      hval[i] = 0u;
    }
    __syncthreads();
    const int32_t u0 = tile_src[t];
    if (u0 < 0 || u0 >= n) {
      ok = false;  // not reached with checked offsets
    } else {
      const int64_t e1 = e0 + len;
      for (int64_t u = (int64_t)u0 + tid; u < n; u += kPT) {
        const int64_t a = out_off[u];
        if (a >= e1) break;
        if (out_off[u + 1] > a) atomicMax(&head[a > e0 ? (int)(a - e0) : 0], (int32_t)u);
      }
    }
    __syncthreads();
    {
      int32_t x[kPE];
      int32_t run = -1;
#pragma unroll
      for (int k = 0; k < kPE; ++k) {
        run = max(run, head[tid * kPE + k]);
        x[k] = run;
      }
      int32_t inc = run;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int32_t y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc = max(inc, y);
      }
      int32_t pre = __shfl_up_sync(0xffffffffu, inc, 1);
      if (lane == 0) pre = -1;
      if (lane == 31) wmax[wid] = inc;
      __syncthreads();
      for (int i = 0; i < wid; ++i) pre = max(pre, wmax[i]);
#pragma unroll
      for (int k = 0; k < kPE; ++k) head[tid * kPE + k] = max(pre, x[k]);
    }
    __syncthreads();
    // 3. slots.  A thread's loads come first (sources, hub bits), then its
    // hub edges are counted in the shared table, then the other edges'
    // atomics are issued together and only then their stores, so its eight
    // atomics are in flight at once.
    int32_t us[kPE];
    uint32_t info[kPE];  // hub edge: (table entry << 16) | rank in the tile
#pragma unroll
    for (int k = 0; k < kPE; ++k) {
      const int p = tile_pos(k);
      const bool id_ok = p < len && (uint32_t)w[k] < (uint32_t)n;
      if (p < len && !id_ok) ok = false;
      const bool in = id_ok && w[k] < t_split;  // targets from t_split on are copied
      us[k] = in ? head[p] : -1;
      if (in && us[k] < 0) ok = false;
      info[k] = in ? __ldg(hub_bits + (w[k] >> 5)) : 0u;
    }
#pragma unroll
    for (int k = 0; k < kPE; ++k) {
      const int32_t v = w[k];
      const bool hub = us[k] >= 0 && ((info[k] >> (v & 31)) & 1u);
      info[k] = kNoSlot;
      if (!hub) continue;
      uint32_t h = ((uint32_t)v * 2654435761u) >> (32 - kHashBits);
      int probe = 0;
      for (; probe < kProbe; ++probe) {
        const int32_t k0 = atomicCAS(&hkey[h], -1, v);
        if (k0 == -1 || k0 == v) break;
        h = (h + 1) & (kHash - 1);
      }
      if (probe < kProbe) info[k] = (h << 16) | atomicAdd(&hval[h], 1u);
    }
    uint32_t slot[kPE];
#pragma unroll
    for (int k = 0; k < kPE; ++k)
      slot[k] = (us[k] >= 0 && info[k] == kNoSlot) ? atomicAdd(&cursor[w[k]], 1u) : kNoSlot;
#pragma unroll
    for (int k = 0; k < kPE; ++k)
      if (slot[k] < slot_cap) __stcs(in_adj + slot[k], us[k]);
    __syncthreads();
    for (int h = tid; h < kHash; h += kPT) {
      const uint32_t c = hval[h];
      if (c == 0u) continue;
      const uint32_t base = atomicAdd(&cursor[hkey[h]], c);
      hval[h] = (uint64_t)base + c <= (uint64_t)slot_cap ? base : kNoSlot;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kPE; ++k) {
      if (info[k] == kNoSlot) continue;
      const uint32_t b = hval[info[k] >> 16];
      if (b != kNoSlot) __stcs(in_adj + b + (info[k] & 0xffffu), us[k]);
    }
    __syncthreads();
  }
  if (!__all_sync(0xffffffffu, ok) && lane == 0) atomicOr(bad, 1);
}

// Pivot keys: out*in (kind 0) or degree (kind 1).
__device__ __forceinline__ unsigned long long pivot_key(const int64_t* out_off, const int64_t* in_off,
                                                        int kind, int64_t v) {
  const unsigned long long o = (unsigned long long)(out_off[v + 1] - out_off[v]);
  const unsigned long long i = in_off ? (unsigned long long)(in_off[v + 1] - in_off[v]) : 0ull;
  return kind == 0 ? o * i : o + i;
}
__global__ void k_pivot_max(int32_t n, const int64_t* out_off, const int64_t* in_off, int kind,
                            unsigned long long* best) {
  unsigned long long k = 0;
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (int64_t)gridDim.x * blockDim.x) {
    const unsigned long long x = pivot_key(out_off, in_off, kind, v);
    if (x > k) k = x;
  }
  if (k) atomicMax(best, k);
}
__global__ void k_pivot_min(int32_t n, const int64_t* out_off, const int64_t* in_off, int kind,
                            const unsigned long long* best, int* id) {
  const unsigned long long b = *best;
  if (b == 0ull) return;
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (int64_t)gridDim.x * blockDim.x) {
    if (pivot_key(out_off, in_off, kind, v) == b) {
      atomicMin(id, (int)v);
      return;
    }
  }
}

__global__ void k_latch(const Ctl* c, int* sticky) {
  if (c->err != 0 && sticky[0] == 0) {
    sticky[0] = c->err;
    sticky[1] = c->err_where;
  }
}

// Degree key of the hint rule: the total degree itself below 32, above it
// eight steps per power of two (the exponent and the next three bits), so
// that every key fits a byte and the key array (n bytes) stays in the L2
// while the adjacency streams past it.  Non-decreasing in the degree.
__device__ __forceinline__ uint8_t degree_key(long long d) {
  if (d < 32) return (uint8_t)(d < 0 ? 0 : d);
  int e = 63 - __clzll((unsigned long long)d);
  if (e > 30) e = 30;
  const long long dd = d < (1ll << 31) ? d : (1ll << 31) - 1;
  return (uint8_t)(32 + 8 * (e - 5) + (int)((dd >> (e - 3)) & 7));
}

__global__ void k_degree_key(int32_t n, const int64_t* out_off, const int64_t* in_off,
                             uint8_t* key) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (int64_t)gridDim.x * blockDim.x) {
    long long d = out_off[v + 1] - out_off[v];
    if (in_off) d += in_off[v + 1] - in_off[v];
    key[v] = degree_key(d);
  }
}

// The pull hint of a vertex: its neighbour of largest degree key, the first
// one in adjacency order on ties (-1 without neighbours).  Vertices are
// taken in three tiers by degree:
//   <= kHintThread neighbours: one thread, eight loads in flight at a time
//      (most vertices of a power-law graph);
//   <= kHintWarp: appended to `mid`, then half a warp per vertex in
//      k_hint_mid (two vertices per warp, eight loads in flight per lane);
//   more: the vertex gets an ordinal in `heavy` and its list is cut into
//      chunks of kHintChunk entries, each appended to `chunk`; a warp per
//      chunk in k_hint_heavy folds the chunk's best (key, position) into the
//      ordinal's slot with a 64-bit atomicMax, and k_hint_slots turns the
//      slots into hints.  A hub's list is then spread over many warps.
// Appends to the middle and heavy lists take one atomic per warp.  Walking
// the middle tier inside the pass that finds it, or cutting the adjacency
// into pieces of 32 consecutive vertices, leaves long tails: R-MAT puts its
// high-degree vertices at neighbouring ids.
constexpr int kHintThread = 32;
constexpr int kHintWarp = 2048;
constexpr int kHintBlock = 256;
constexpr int kHintThreadWU = 8;  // loads in flight per thread, thread tier
constexpr int kHintMidWU = 8;     // per lane, middle tier
constexpr int kHintHeavyWU = 8;   // and heavy tier
constexpr int kHintChunk = 32 * kHintHeavyWU * 4;  // 1,024 entries: four rounds of a warp

// (key, position) packed so that the larger key wins and, between equal
// keys, the earlier position: 16 bits of position in the middle tier
// (lists of at most kHintWarp entries), 48 in the heavy tier.
__device__ __forceinline__ uint32_t mid_pack(int32_t key, int32_t e) {
  return ((uint32_t)key << 16) | (0xFFFFu - (uint32_t)e);
}
constexpr uint64_t kHintPos48 = (1ull << 48) - 1;
__device__ __forceinline__ uint64_t heavy_pack(int32_t key, int64_t e) {
  return ((uint64_t)key << 48) | (kHintPos48 - (uint64_t)e);
}

// One side of the hint build: a CSR and the hints it gets.  Both sides go
// through each tier in one launch; a listed vertex of the in-side is stored
// as ~v.
struct HintSide {
  const int64_t* off;
  const int32_t* adj;
  int32_t* hint;
};

// The lists the first pass fills.  count: [0] middle vertices, [1] heavy
// vertices (ordinals), [2] heavy chunks.
struct HintLists {
  int32_t* mid;
  int32_t* heavy;                // tag of each heavy ordinal
  unsigned long long* slot;      // packed best of each heavy ordinal (zeroed)
  int64_t* chunk;                // (ordinal << 32) | chunk index
  unsigned long long* count;
  int64_t heavy_cap, chunk_cap;  // bounds the sizes guarantee (checked anyway)
};

__device__ __forceinline__ HintSide side_of(int32_t x, const HintSide s0, const HintSide s1) {
  return x < 0 ? s1 : s0;
}

__global__ void __launch_bounds__(kHintBlock) k_hint(int32_t n, int sides, HintSide s0,
                                                     HintSide s1, const uint8_t* deg,
                                                     HintLists L) {
  const int lane = threadIdx.x & 31;
  const unsigned below = (1u << lane) - 1u;
  const int64_t total = (int64_t)sides * n;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  // the bound is tested on the warp's first vertex, so that every lane of a
  // warp takes part in the appends' ballots
  for (int64_t b = (int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31); b < total;
       b += stride) {
    const int64_t v2 = b + lane;
    const bool live = v2 < total;
    const bool in = v2 >= n;
    const int64_t v = in ? v2 - n : v2;
    const HintSide S = in ? s1 : s0;
    int64_t s = 0, d = 0;
    if (live) {
      s = S.off[v];
      d = S.off[v + 1] - s;
    }
    const int32_t tag = in ? ~(int32_t)v : (int32_t)v;
    const bool heavy = live && d > kHintWarp;
    const bool middle = live && d > kHintThread && !heavy;
    const unsigned bm = __ballot_sync(0xffffffffu, middle);
    if (bm) {
      const int leader = __ffs(bm) - 1;
      unsigned long long base = 0;
      if (lane == leader) base = atomicAdd(&L.count[0], (unsigned long long)__popc(bm));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (middle) L.mid[base + __popc(bm & below)] = tag;
    }
    const unsigned bh = __ballot_sync(0xffffffffu, heavy);
    if (bh) {
      const int leader = __ffs(bh) - 1;
      unsigned long long base = 0;
      if (lane == leader) base = atomicAdd(&L.count[1], (unsigned long long)__popc(bh));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (heavy) {
        const int64_t j = (int64_t)base + __popc(bh & below);
        const int64_t c = (d + kHintChunk - 1) / kHintChunk;
        const int64_t c0 = (int64_t)atomicAdd(&L.count[2], (unsigned long long)c);
        if (j < L.heavy_cap) {
          L.heavy[j] = tag;
          for (int64_t q = 0; q < c && c0 + q < L.chunk_cap; ++q)
            L.chunk[c0 + q] = (j << 32) | q;
        }
      }
    }
    if (live && d <= kHintThread) {
      int32_t best_d = -1, best_a = -1;
      for (int64_t e = 0; e < d; e += kHintThreadWU) {
        int32_t a[kHintThreadWU], k[kHintThreadWU];
#pragma unroll
        for (int q = 0; q < kHintThreadWU; ++q) a[q] = e + q < d ? S.adj[s + e + q] : -1;
#pragma unroll
        for (int q = 0; q < kHintThreadWU; ++q) k[q] = a[q] >= 0 ? (int32_t)deg[a[q]] : -1;
#pragma unroll
        for (int q = 0; q < kHintThreadWU; ++q)
          if (k[q] > best_d) {
            best_d = k[q];
            best_a = a[q];
          }
      }
      S.hint[v] = best_a;
    }
  }
}

// Half a warp per middle-tier vertex, two vertices per warp, the list
// spread over every warp.  A half-warp reads the tag and offsets of its next
// vertex before it walks the current one, so that those loads overlap.
__global__ void __launch_bounds__(kHintBlock) k_hint_mid(HintSide s0, HintSide s1,
                                                         const uint8_t* deg, const int32_t* mid,
                                                         const unsigned long long* nmid) {
  const int lane = threadIdx.x & 31, hl = lane & 15;
  const int64_t halves = (int64_t)gridDim.x * (blockDim.x >> 4);
  const int64_t nm = (int64_t)*nmid;
  int64_t b = (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 2;
  int32_t x = 0, d = 0;
  int64_t s = 0;
  if (b + (lane >> 4) < nm) {
    x = mid[b + (lane >> 4)];
    const HintSide S = side_of(x, s0, s1);
    const int32_t v = x < 0 ? ~x : x;
    s = S.off[v];
    d = (int32_t)(S.off[v + 1] - s);
  }
  for (; b < nm; b += halves) {
    const int64_t i = b + (lane >> 4);
    const bool live = i < nm;
    const int32_t v = x < 0 ? ~x : x;
    const HintSide S = side_of(x, s0, s1);
    const int64_t cs = s;
    const int32_t cd = d;
    // the next vertex's header
    x = 0;
    d = 0;
    s = 0;
    if (i + halves < nm) {
      x = mid[i + halves];
      const HintSide N = side_of(x, s0, s1);
      const int32_t vn = x < 0 ? ~x : x;
      s = N.off[vn];
      d = (int32_t)(N.off[vn + 1] - s);
    }
    uint32_t best = 0;
    for (int32_t e = hl; e < cd; e += 16 * kHintMidWU) {
      int32_t a[kHintMidWU];
#pragma unroll
      for (int q = 0; q < kHintMidWU; ++q) a[q] = e + 16 * q < cd ? S.adj[cs + e + 16 * q] : -1;
#pragma unroll
      for (int q = 0; q < kHintMidWU; ++q)
        if (a[q] >= 0) best = max(best, mid_pack(deg[a[q]], e + 16 * q));
    }
    for (int o = 8; o; o >>= 1) best = max(best, __shfl_xor_sync(0xffffffffu, best, o));
    if (live && hl == 0) S.hint[v] = S.adj[cs + (int32_t)(0xFFFFu - (best & 0xFFFFu))];
  }
}

// A warp per chunk of a heavy vertex's list: the chunk's best folded into
// the vertex's slot.
__global__ void __launch_bounds__(kHintBlock, 8) k_hint_heavy(HintSide s0, HintSide s1,
                                                           const uint8_t* deg, HintLists L) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  const int64_t nc = min((int64_t)L.count[2], L.chunk_cap);
  for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < nc; i += warps) {
    const int64_t c = L.chunk[i];
    const int64_t j = c >> 32;
    const int32_t x = L.heavy[j];
    const int32_t v = x < 0 ? ~x : x;
    const HintSide S = side_of(x, s0, s1);
    const int64_t s = S.off[v], d = S.off[v + 1] - s;
    const int64_t e0 = (c & 0xffffffffll) * kHintChunk;
    const int64_t e1 = min(d, e0 + kHintChunk);
    unsigned long long best = 0;
    for (int64_t e = e0 + lane; e < e1; e += 32 * kHintHeavyWU) {
      int32_t a[kHintHeavyWU];
#pragma unroll
      for (int q = 0; q < kHintHeavyWU; ++q) a[q] = e + 32 * q < e1 ? S.adj[s + e + 32 * q] : -1;
#pragma unroll
      for (int q = 0; q < kHintHeavyWU; ++q)
        if (a[q] >= 0) best = max(best, (unsigned long long)heavy_pack(deg[a[q]], e + 32 * q));
    }
    for (int o = 16; o; o >>= 1) best = max(best, __shfl_xor_sync(0xffffffffu, best, o));
    if (lane == 0) atomicMax(&L.slot[j], best);
  }
}

// Heavy ordinals' slots -> hints.
__global__ void k_hint_slots(HintSide s0, HintSide s1, HintLists L) {
  const int64_t nh = min((int64_t)L.count[1], L.heavy_cap);
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < nh;
       j += (int64_t)gridDim.x * blockDim.x) {
    const int32_t x = L.heavy[j];
    const int32_t v = x < 0 ? ~x : x;
    const HintSide S = side_of(x, s0, s1);
    const unsigned long long best = L.slot[j];  // non-zero once a chunk folded in
    const uint64_t e = kHintPos48 - (best & kHintPos48);
    S.hint[v] = best ? S.adj[S.off[v] + (int64_t)e] : -1;
  }
}

// Blocks of `threads` threads of kernel k resident at once on the current
// device (at least one per SM).
template <typename K>
int resident_grid(K k, int threads) {
  int dev = 0, sms = 152, per = 1;
  if (cudaGetDevice(&dev) == cudaSuccess)
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k, threads, 0) != cudaSuccess || per < 1)
    per = 1;
  cudaGetLastError();
  return sms * per;
}

int bits_for(int32_t n) {
  int b = 1;
  while (b < 32 && (1ll << b) < (long long)n) ++b;
  return b;
}

int grid_for(int64_t work) {
  int64_t g = (work + 255) / 256;
  if (g > 152 * 32) g = 152 * 32;
  if (g < 1) g = 1;
  return (int)g;
}

// Sort (key, value) pairs by key (stable) and write CSR offsets + adjacency.
cudaError_t one_side(int32_t n, int64_t m, const int32_t* key, const int32_t* val, int64_t* off,
                     int32_t* adj, uint32_t* tmp_keys, cudaStream_t s) {
  size_t bytes = 0;
  const int bits = bits_for(n);
  cudaError_t e = cub::DeviceRadixSort::SortPairs(
      nullptr, bytes, reinterpret_cast<const uint32_t*>(key), tmp_keys, val, adj, m, 0, bits, s);
  if (e != cudaSuccess) return e;
  void* temp = nullptr;
  e = cudaMallocAsync(&temp, bytes ? bytes : 16, s);
  if (e != cudaSuccess) return e;
  e = cub::DeviceRadixSort::SortPairs(temp, bytes, reinterpret_cast<const uint32_t*>(key),
                                      tmp_keys, val, adj, m, 0, bits, s);
  cudaFreeAsync(temp, s);
  if (e != cudaSuccess) return e;
  k_offsets<<<grid_for(m + 1), 256, 0, s>>>(tmp_keys, m, n, off);
  return cudaGetLastError();
}

}  // namespace

cudaError_t build_csr(int32_t n, int64_t m, const int32_t* d_src, const int32_t* d_dst,
                      int64_t* out_off, int32_t* out_adj, int64_t* in_off, int32_t* in_adj,
                      cudaStream_t s, bool* ids_ok) {
  *ids_ok = true;
  int* bad = nullptr;
  cudaError_t e = cudaMallocAsync(&bad, sizeof(int), s);
  if (e != cudaSuccess) return e;
  cudaMemsetAsync(bad, 0, sizeof(int), s);
  if (m > 0) k_check_ids<<<grid_for(m), 256, 0, s>>>(d_src, d_dst, m, n, bad);
  int hbad = 0;
  cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, s);
  cudaFreeAsync(bad, s);
  e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return e;
  if (hbad) {
    *ids_ok = false;
    return cudaSuccess;
  }
  uint32_t* tmp = nullptr;
  e = cudaMallocAsync(&tmp, (size_t)(m > 0 ? m : 1) * sizeof(uint32_t), s);
  if (e != cudaSuccess) return e;
  e = one_side(n, m, d_src, d_dst, out_off, out_adj, tmp, s);
  if (e == cudaSuccess && in_off != nullptr) e = one_side(n, m, d_dst, d_src, in_off, in_adj, tmp, s);
  cudaFreeAsync(tmp, s);
  return e;
}

cudaError_t check_csr(int32_t n, int64_t m, const int64_t* off, const int32_t* adj,
                      cudaStream_t s, int* bad) {
  int* d = nullptr;
  cudaError_t e = cudaMallocAsync(&d, sizeof(int), s);
  if (e != cudaSuccess) return e;
  cudaMemsetAsync(d, 0, sizeof(int), s);
  k_check_csr<<<grid_for((m > n ? m : n) + 1), 256, 0, s>>>(n, m, off, adj, d);
  cudaMemcpyAsync(bad, d, sizeof(int), cudaMemcpyDeviceToHost, s);
  cudaFreeAsync(d, s);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return cudaStreamSynchronize(s);
}

cudaError_t check_ids_flag(int32_t n, const int32_t* adj, int64_t count, int* d_bad,
                           cudaStream_t s) {
  if (count <= 0) return cudaSuccess;
  k_check_adj_ids<<<grid_for(count), 256, 0, s>>>(adj, count, n, d_bad);
  return cudaGetLastError();
}

cudaError_t check_csr_flag(int32_t n, int64_t m, const int64_t* off, const int32_t* adj,
                           int* d_bad, cudaStream_t s) {
  k_check_csr<<<grid_for((m > n ? m : n) + 1), 256, 0, s>>>(n, m, off, adj, d_bad);
  return cudaGetLastError();
}

cudaError_t ingest_csr32(int32_t n, int64_t m, const uint32_t* h_off, const int32_t* h_adj,
                         int64_t* off, int32_t* adj, int* d_bad, cudaStream_t s) {
  k_ingest_off<<<grid_for((int64_t)n + 1), 256, 0, s>>>(h_off, off, n, m, d_bad);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || m == 0) return e;
  k_ingest_adj<<<grid_for(m / 4 + 1), 256, 0, s>>>(h_adj, adj, m, n, d_bad);
  return cudaGetLastError();
}

cudaError_t ingest_csr32_derive_in(int32_t n, int64_t m, const uint32_t* h_out_off,
                                   const int32_t* h_out_adj, const uint32_t* h_in_off,
                                   int64_t* out_off, int32_t* out_adj, int64_t* in_off,
                                   int32_t* in_adj, int32_t t_split, const int32_t* h_in_adj,
                                   int64_t tail0, int* d_bad, cudaStream_t s) {
  if (m >= (1ll << 31) || t_split < 0 || t_split > n || tail0 < 0 || tail0 > m ||
      (tail0 < m && h_in_adj == nullptr))
    return cudaErrorInvalidValue;
  k_ingest_off<<<grid_for((int64_t)n + 1), 256, 0, s>>>(h_out_off, out_off, n, m, d_bad);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  const int64_t tiles = (m + kTile - 1) / kTile;
  const int64_t words = ((int64_t)n + 31) / 32;
  // cursors (n), hub bits (words), tile heads (tiles)
  uint32_t* tmp = nullptr;
  e = cudaMallocAsync(&tmp, ((size_t)n + (size_t)words + (size_t)tiles + 1) * 4, s);
  if (e != cudaSuccess) return e;
  uint32_t* cursor = tmp;
  uint32_t* hub_bits = cursor + n;
  int32_t* tile_src = reinterpret_cast<int32_t*>(hub_bits + words);
  k_ingest_in_off<<<grid_for((int64_t)n + 1), 256, 0, s>>>(h_in_off, n, m, in_off, cursor,
                                                           hub_bits, d_bad);
  e = cudaGetLastError();
  if (e == cudaSuccess && m > 0) {
    cudaMemsetAsync(tile_src, 0xff, (size_t)tiles * 4, s);
    k_tile_heads<<<grid_for(n), 256, 0, s>>>(n, tiles, out_off, tile_src, d_bad);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && m > 0) {
    static int blocks[64] = {0};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) dev = 0;
    if (blocks[dev] == 0) {
      int per_sm = 0, sms = 0;
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_place_in, kPT, 0);
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      blocks[dev] = (per_sm > 0 ? per_sm : 1) * (sms > 0 ? sms : 1);
    }
    // placement tiles and the copy tiles of the in-lists from tail0 on
    const int64_t ca = tail0 < m ? ((tail0 + 3) & ~(int64_t)3) : m;
    const int64_t units = tiles + (ca < m ? (m - ca + kTile - 1) / kTile : 0);
    const int g = (int)(units < blocks[dev] ? units : blocks[dev]);
    k_place_in<<<g, kPT, 0, s>>>(h_out_adj, out_adj, m, n, out_off, hub_bits, cursor, tile_src,
                                 in_adj, t_split, h_in_adj, tail0, d_bad);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && t_split > 0) {
    k_check_cursors<<<grid_for(t_split), 256, 0, s>>>(t_split, in_off, cursor, d_bad);
    e = cudaGetLastError();
  }
  cudaFreeAsync(tmp, s);
  return e;
}

cudaError_t pivot_device(int32_t n, const int64_t* out_off, const int64_t* in_off, int kind,
                         cudaStream_t s, int32_t* pivot) {
  unsigned long long* best = nullptr;
  cudaError_t e = cudaMallocAsync(&best, 16, s);
  if (e != cudaSuccess) return e;
  int* id = reinterpret_cast<int*>(best + 1);
  cudaMemsetAsync(best, 0, 8, s);
  cudaMemsetAsync(id, 0x7f, 4, s);
  if (n > 0) {
    k_pivot_max<<<grid_for(n), 256, 0, s>>>(n, out_off, in_off, kind, best);
    k_pivot_min<<<grid_for(n), 256, 0, s>>>(n, out_off, in_off, kind, best, id);
  }
  unsigned long long hb[2] = {0, 0};
  cudaMemcpyAsync(hb, best, 16, cudaMemcpyDeviceToHost, s);
  cudaFreeAsync(best, s);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return e;
  int hid;
  std::memcpy(&hid, &hb[1], sizeof(int));
  *pivot = hb[0] == 0ull ? -1 : hid;
  return cudaSuccess;
}

cudaError_t batch_edges_device(int32_t count, const int32_t* h_n, const int32_t* h_ef,
                               const uint64_t* h_seeds, gb_rmat_thr thr, int id_bits,
                               const int64_t* h_vbase, int32_t** d_src, int32_t** d_dst,
                               int64_t* m_out, cudaStream_t s) {
  // per graph: scale, candidate edge base
  int32_t* hs = new int32_t[count];
  int64_t* heb = new int64_t[count + 1];
  heb[0] = 0;
  for (int g = 0; g < count; ++g) {
    int sc = 1;
    while (sc < 31 && (1ll << sc) < (long long)h_n[g]) ++sc;
    hs[g] = sc;
    heb[g + 1] = heb[g] + (int64_t)h_ef[g] * h_n[g];
  }
  const int64_t etotal = heb[count];
  int64_t *d_eb = nullptr, *d_vb = nullptr, *nsel = nullptr;
  int32_t *d_nv = nullptr, *d_sc = nullptr;
  uint64_t *d_seed = nullptr, *a = nullptr, *b = nullptr;
  cudaError_t e = cudaMallocAsync(&d_eb, (count + 1) * 8, s);
  if (e == cudaSuccess) e = cudaMallocAsync(&d_vb, (count + 1) * 8, s);
  if (e == cudaSuccess) e = cudaMallocAsync(&d_nv, count * 4, s);
  if (e == cudaSuccess) e = cudaMallocAsync(&d_sc, count * 4, s);
  if (e == cudaSuccess) e = cudaMallocAsync(&d_seed, count * 8, s);
  if (e == cudaSuccess) e = cudaMallocAsync(&nsel, 8, s);
  if (e == cudaSuccess) e = cudaMallocAsync(&a, (size_t)(etotal > 0 ? etotal : 1) * 8, s);
  if (e == cudaSuccess) e = cudaMallocAsync(&b, (size_t)(etotal > 0 ? etotal : 1) * 8, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_eb, heb, (count + 1) * 8, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_vb, h_vbase, (count + 1) * 8, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_nv, h_n, count * 4, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_sc, hs, count * 4, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_seed, h_seeds, count * 8, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  delete[] hs;
  delete[] heb;
  int64_t k = 0;
  if (e == cudaSuccess && etotal > 0) {
    k_batch_keys<<<grid_for((etotal + kRun - 1) / kRun), 256, 0, s>>>(
        etotal, d_eb, d_vb, d_nv, d_sc, d_seed, count, thr, id_bits, a);
    size_t bytes = 0, bytes2 = 0;
    cub::DeviceRadixSort::SortKeys(nullptr, bytes, a, b, etotal, 0, 2 * id_bits, s);
    cub::DeviceSelect::Unique(nullptr, bytes2, b, a, nsel, etotal, s);
    if (bytes2 > bytes) bytes = bytes2;
    void* temp = nullptr;
    e = cudaMallocAsync(&temp, bytes ? bytes : 16, s);
    if (e == cudaSuccess) e = cub::DeviceRadixSort::SortKeys(temp, bytes, a, b, etotal, 0, 2 * id_bits, s);
    if (e == cudaSuccess) e = cub::DeviceSelect::Unique(temp, bytes, b, a, nsel, etotal, s);
    cudaFreeAsync(temp, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&k, nsel, 8, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e == cudaSuccess && k > 0) {
      uint64_t last = 0;
      e = cudaMemcpyAsync(&last, a + (k - 1), 8, cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s);
      if (last == (1ull << (2 * id_bits)) - 1ull) --k;  // the dropped-edge marker
    }
  }
  int32_t *src = nullptr, *dst = nullptr;
  if (e == cudaSuccess) e = cudaMallocAsync(&src, (size_t)(k > 0 ? k : 1) * 4, s);
  if (e == cudaSuccess) e = cudaMallocAsync(&dst, (size_t)(k > 0 ? k : 1) * 4, s);
  if (e == cudaSuccess && k > 0) k_split_bits<<<grid_for(k), 256, 0, s>>>(a, k, id_bits, src, dst);
  cudaFreeAsync(a, s);
  cudaFreeAsync(b, s);
  cudaFreeAsync(d_eb, s);
  cudaFreeAsync(d_vb, s);
  cudaFreeAsync(d_nv, s);
  cudaFreeAsync(d_sc, s);
  cudaFreeAsync(d_seed, s);
  cudaFreeAsync(nsel, s);
  if (e != cudaSuccess) return e;
  *d_src = src;
  *d_dst = dst;
  *m_out = k;
  return cudaGetLastError();
}

cudaError_t batch_gid(int32_t n, const int64_t* d_vbase, int32_t count, int32_t* gid,
                      cudaStream_t s) {
  if (n > 0) k_fill_gid<<<grid_for(n), 256, 0, s>>>(n, d_vbase, count, gid);
  return cudaGetLastError();
}

cudaError_t batch_check_within(const int32_t* src, const int32_t* dst, int64_t m,
                               const int32_t* gid, cudaStream_t s, int* bad) {
  int* d = nullptr;
  cudaError_t e = cudaMallocAsync(&d, sizeof(int), s);
  if (e != cudaSuccess) return e;
  cudaMemsetAsync(d, 0, sizeof(int), s);
  if (m > 0) k_check_within<<<grid_for(m), 256, 0, s>>>(src, dst, m, gid, d);
  cudaMemcpyAsync(bad, d, sizeof(int), cudaMemcpyDeviceToHost, s);
  cudaFreeAsync(d, s);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return cudaStreamSynchronize(s);
}

cudaError_t max_degree(int32_t n, const int64_t* off, cudaStream_t s, unsigned long long* out) {
  unsigned long long* d = nullptr;
  cudaError_t e = cudaMallocAsync(&d, 8, s);
  if (e != cudaSuccess) return e;
  cudaMemsetAsync(d, 0, 8, s);
  if (n > 0) k_max_degree<<<grid_for(n), 256, 0, s>>>(n, off, d);
  cudaMemcpyAsync(out, d, 8, cudaMemcpyDeviceToHost, s);
  cudaFreeAsync(d, s);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return cudaStreamSynchronize(s);
}

cudaError_t launch_latch(Ctl* ctl, int* sticky, cudaStream_t s) {
  k_latch<<<1, 1, 0, s>>>(ctl, sticky);
  return cudaGetLastError();
}

cudaError_t build_hints(int32_t n, int64_t m, const int64_t* out_off, const int32_t* out_adj,
                        const int64_t* in_off, const int32_t* in_adj, int32_t* hint_out,
                        int32_t* hint_in, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  // the sides to build, the out-side first
  HintSide sd[2];
  int sides = 0;
  if (out_off && hint_out) sd[sides++] = HintSide{out_off, out_adj, hint_out};
  if (in_off && hint_in) sd[sides++] = HintSide{in_off, in_adj, hint_in};
  if (sides == 0) return cudaSuccess;
  if (sides == 1) sd[1] = sd[0];
  // Scratch: the heavy slots and the three counts (zeroed together), the
  // chunks, the middle list (a vertex-side each at most), the heavy tags,
  // then the degree keys (n bytes).  A side holds m entries, so at most
  // 2m / (kHintWarp + 1) vertex-sides are heavy and their lists make at most
  // 2m / kHintChunk + (heavy vertex-sides) chunks.
  const int64_t mm = m > 0 ? m : 0;
  HintLists L;
  L.heavy_cap = std::min<int64_t>(2 * (int64_t)n, 2 * mm / (kHintWarp + 1) + 1);
  L.chunk_cap = 2 * mm / kHintChunk + L.heavy_cap;
  const size_t zero_b = ((size_t)L.heavy_cap + 4) * 8;
  const size_t bytes = zero_b + (size_t)L.chunk_cap * 8 + (size_t)2 * n * 4 +
                       (size_t)L.heavy_cap * 4 + (size_t)n;
  char* buf = nullptr;
  cudaError_t e = cudaMallocAsync(&buf, bytes, s);
  if (e != cudaSuccess) return e;
  L.slot = reinterpret_cast<unsigned long long*>(buf);
  L.count = L.slot + L.heavy_cap;
  L.chunk = reinterpret_cast<int64_t*>(L.count + 4);
  L.mid = reinterpret_cast<int32_t*>(L.chunk + L.chunk_cap);
  L.heavy = L.mid + 2 * (size_t)n;
  uint8_t* deg = reinterpret_cast<uint8_t*>(L.heavy + L.heavy_cap);
  e = cudaMemsetAsync(buf, 0, zero_b, s);
  if (e != cudaSuccess) {
    cudaFreeAsync(buf, s);
    return e;
  }
  k_degree_key<<<grid_for(n), 256, 0, s>>>(n, out_off, in_off, deg);
  // the list passes: as many blocks as are resident at once on the SMs
  static const int gw_mid = resident_grid(k_hint_mid, kHintBlock);
  static const int gw_heavy = resident_grid(k_hint_heavy, kHintBlock);
  // (a side's entries carry its tag; with one side the in-side copy is the
  // out-side's, never tagged)
  k_hint<<<grid_for((int64_t)sides * n), kHintBlock, 0, s>>>(n, sides, sd[0], sd[1], deg, L);
  k_hint_mid<<<gw_mid, kHintBlock, 0, s>>>(sd[0], sd[1], deg, L.mid, L.count);
  k_hint_heavy<<<gw_heavy, kHintBlock, 0, s>>>(sd[0], sd[1], deg, L);
  k_hint_slots<<<grid_for(L.heavy_cap), 256, 0, s>>>(sd[0], sd[1], L);
  cudaFreeAsync(buf, s);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return cudaStreamSynchronize(s);
}

cudaError_t widen_offsets(const uint32_t* in, int64_t* out, int64_t count, cudaStream_t s) {
  if (count > 0) k_widen<<<grid_for(count), 256, 0, s>>>(in, out, count);
  return cudaGetLastError();
}

cudaError_t rmat_edges_device(int32_t n, int edge_factor, uint64_t seed, gb_rmat_thr thr,
                              int32_t** d_src, int32_t** d_dst, int64_t* m_out, cudaStream_t s) {
  int scale = 1;
  while (scale < 31 && (1ll << scale) < (long long)n) ++scale;
  const int64_t m0 = (int64_t)edge_factor * n;
  const uint64_t self = (1ull << (2 * scale)) - 1ull;
  uint64_t *a = nullptr, *b = nullptr;
  int64_t* nsel = nullptr;
  cudaError_t e = cudaMallocAsync(&a, (size_t)m0 * 8, s);
  if (e == cudaSuccess) e = cudaMallocAsync(&b, (size_t)m0 * 8, s);
  if (e == cudaSuccess) e = cudaMallocAsync(&nsel, sizeof(int64_t), s);
  if (e != cudaSuccess) return e;
  k_rmat_keys<<<grid_for(m0), 256, 0, s>>>(seed, m0, scale, (uint32_t)n, thr, self, a);
  size_t bytes = 0, bytes2 = 0;
  cub::DeviceRadixSort::SortKeys(nullptr, bytes, a, b, m0, 0, 2 * scale, s);
  cub::DeviceSelect::Unique(nullptr, bytes2, b, a, nsel, m0, s);
  if (bytes2 > bytes) bytes = bytes2;
  void* temp = nullptr;
  e = cudaMallocAsync(&temp, bytes ? bytes : 16, s);
  if (e == cudaSuccess) e = cub::DeviceRadixSort::SortKeys(temp, bytes, a, b, m0, 0, 2 * scale, s);
  if (e == cudaSuccess) e = cub::DeviceSelect::Unique(temp, bytes, b, a, nsel, m0, s);
  cudaFreeAsync(temp, s);
  int64_t k = 0;
  uint64_t last = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&k, nsel, sizeof(int64_t), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e == cudaSuccess && k > 0) {
    e = cudaMemcpyAsync(&last, a + (k - 1), 8, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (last == self) --k;  // only the self-loop key can equal `self`
  }
  int32_t *src = nullptr, *dst = nullptr;
  if (e == cudaSuccess) e = cudaMallocAsync(&src, (size_t)(k > 0 ? k : 1) * 4, s);
  if (e == cudaSuccess) e = cudaMallocAsync(&dst, (size_t)(k > 0 ? k : 1) * 4, s);
  if (e == cudaSuccess && k > 0) k_split<<<grid_for(k), 256, 0, s>>>(a, k, scale, src, dst);
  cudaFreeAsync(a, s);
  cudaFreeAsync(b, s);
  cudaFreeAsync(nsel, s);
  if (e != cudaSuccess) return e;
  *d_src = src;
  *d_dst = dst;
  *m_out = k;
  return cudaGetLastError();
}

}  // namespace gb
