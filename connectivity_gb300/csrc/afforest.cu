// Connected components of a symmetric CSR read in place from host memory
// (the drop-in gb_run_cc): sampled union-find in which the largest
// component's adjacency past a small sample is never read, so most of the
// CSR does not cross the host link.
//
// cc's graph (cc_main.cpp:72-79 and 102-118) is the mirrored edge list:
// every edge sits in the lists of both its ends.  Union-find over the edges
// with the larger root always hooked under the smaller gives every
// component its smallest id as root, which is the canonical label of the
// reference's cc labels (cc_main.cpp:184-245).  The order of the work
// follows the published Afforest scheme (Sutton, Ben-Nun and Barak, IPDPS
// 2018): every vertex first links to its first kSample neighbours (one:
// measured faster than the scheme's two on R-MAT, whose first neighbours
// are hubs); the most frequent root among a sample of vertices is then
// taken for the largest component, and only the vertices outside it link
// their remaining neighbours.  A vertex inside it may skip them: a neighbour outside the
// component holds the same edge in its own list (the CSR is symmetric) and
// links it from there.
#include <cstdint>

#include "gb_internal.cuh"

namespace gb {
namespace {

constexpr int kSample = 1;          // neighbours every vertex links first
constexpr int kModeSamples = 1024;  // vertices sampled for the largest component
constexpr int kModeHash = 2048;
constexpr int kLinkCap = 1 << 20;   // retries of one link before it reports failure

int af_grid(int64_t work) {
  int64_t g = (work + 255) / 256;
  if (g > 152 * 16) g = 152 * 16;
  if (g < 1) g = 1;
  return (int)g;
}

// Offsets to the device (checked: off[0] == 0, off[n] == m, non-decreasing)
// and every vertex its own parent.
__global__ void k_af_init(const uint32_t* __restrict__ h, int32_t n, int64_t m,
                          uint32_t* __restrict__ off, int32_t* __restrict__ parent, int* bad) {
  const int lane = threadIdx.x & 31;
  for (int64_t base = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) & ~(int64_t)31; base <= n;
       base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = base + lane;
    const uint32_t x = i <= n ? h[i] : 0u;
    uint32_t nx = __shfl_down_sync(0xffffffffu, x, 1);
    if (lane == 31 && i + 1 <= n) nx = h[i + 1];
    if (i <= n) {
      off[i] = x;
      if (i < n) parent[i] = (int32_t)i;
      if ((i == 0 && x != 0u) || (i == n && (int64_t)x != m) || (i < n && nx < x)) atomicOr(bad, 1);
    }
  }
}

// Joins the trees of u and v, the larger root hooked under the smaller
// (the lock-free link of the Afforest scheme).  False after kLinkCap
// retries.
__device__ __forceinline__ bool af_link(int32_t u, int32_t v, int32_t* p) {
  volatile int32_t* vp = p;
  int32_t p1 = vp[u], p2 = vp[v];
  for (int it = 0; p1 != p2; ++it) {
    if (it >= kLinkCap) return false;
    const int32_t high = p1 > p2 ? p1 : p2, low = p1 > p2 ? p2 : p1;
    const int32_t ph = vp[high];
    if (ph == low) return true;
    if (ph == high && atomicCAS(p + high, high, low) == high) return true;
    p1 = vp[vp[high]];
    p2 = vp[low];
  }
  return true;
}

// One or two adjacency lists per vertex (a symmetric CSR; or the out- and
// in-CSR of a directed graph, whose union is symmetric).
template <typename OffT, int NC>
struct UfCsr {
  const OffT* off[NC];
  const int32_t* adj[NC];
};

// Every vertex to the first kSample neighbours of each of its lists, in one
// pass (sampling rounds with a compression between them were measured
// slower: each round reads every vertex's list head again).
template <typename OffT, int NC>
__global__ void k_af_sample(int32_t n, UfCsr<OffT, NC> g, int32_t* parent, int* bad, int* err) {
  if (*(volatile const int*)bad) return;
  bool ok = true, fine = true;
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (int64_t)gridDim.x * blockDim.x) {
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      const OffT a = g.off[c][v], b = g.off[c][v + 1];
      int32_t w[kSample];
#pragma unroll
      for (int j = 0; j < kSample; ++j) w[j] = a + j < b ? g.adj[c][a + j] : -1;
#pragma unroll
      for (int j = 0; j < kSample; ++j) {
        if (a + j >= b) continue;
        if ((uint32_t)w[j] >= (uint32_t)n) {
          ok = false;
          continue;
        }
        fine = af_link((int32_t)v, w[j], parent) && fine;
      }
    }
  }
  if (!ok) atomicOr(bad, 1);
  if (!fine) atomicCAS(err, 0, (int)kErrIterLimit);
}

// Every parent to its root (no link runs at the same time).
__global__ void k_af_compress(int32_t n, int32_t* parent, int* err) {
  bool fine = true;
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (int64_t)gridDim.x * blockDim.x) {
    int32_t r = parent[v];
    int it = 0;
    while (parent[r] != r && it < kLinkCap) {
      r = parent[r];
      ++it;
    }
    if (it >= kLinkCap) fine = false;
    parent[v] = r;
  }
  if (!fine) atomicCAS(err, 0, (int)kErrIterLimit);
}

// The most frequent root among kModeSamples spread vertices (one block).
__global__ void __launch_bounds__(kModeSamples) k_af_mode(int32_t n, const int32_t* parent,
                                                          int32_t* giant) {
  __shared__ int32_t key[kModeHash];
  __shared__ int32_t cnt[kModeHash];
  __shared__ unsigned long long best;
  for (int i = threadIdx.x; i < kModeHash; i += blockDim.x) {
    key[i] = -1;
    cnt[i] = 0;
  }
  if (threadIdx.x == 0) best = 0ull;
  __syncthreads();
  if (n > 0) {
    const int32_t v = (int32_t)(((unsigned long long)threadIdx.x * 2654435761ull + 12345ull) %
                                (unsigned long long)n);
    const int32_t r = parent[v];
    uint32_t h = ((uint32_t)r * 2654435761u) & (kModeHash - 1);
    for (int probe = 0; probe < kModeHash; ++probe) {
      const int32_t k0 = atomicCAS(&key[h], -1, r);
      if (k0 == -1 || k0 == r) {
        const int c = atomicAdd(&cnt[h], 1) + 1;
        // count, then the smaller root on ties
        atomicMax(&best, ((unsigned long long)c << 32) | (0xffffffffu - (uint32_t)r));
        break;
      }
      h = (h + 1) & (kModeHash - 1);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0)
    *giant = best ? (int32_t)(0xffffffffu - (uint32_t)(best & 0xffffffffull)) : -1;
}

// Vertices outside the sampled largest component link their remaining
// neighbours.  A warp takes 32 vertices, finds those that have edges left
// (outside the component), and walks their lists together, a lane per edge;
// a vertex with more than kAfHeavy edges left goes to `heavy`, walked by
// whole blocks in k_af_rest_heavy (a hub that the sample left outside the
// component would otherwise hold one warp for its whole list).
constexpr long long kAfHeavy = 4096;

template <typename OffT, int NC>
__global__ void k_af_rest(int32_t n, UfCsr<OffT, NC> g, int32_t* parent, const int32_t* giant,
                          int32_t* heavy, int32_t* nheavy, int* bad, int* err) {
  if (*(volatile const int*)bad) return;
  const int32_t cg = *giant;
  const int lane = threadIdx.x & 31;
  const int64_t wid = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  bool ok = true, fine = true;
  for (int64_t base = wid * 32; base < n; base += nw * 32) {
    const int64_t v = base + lane;
    long long left = 0;
    if (v < n && ((volatile int32_t*)parent)[v] != cg) {
#pragma unroll
      for (int c = 0; c < NC; ++c) {
        const long long d = (long long)(g.off[c][v + 1] - g.off[c][v]) - kSample;
        left += d > 0 ? d : 0;
      }
    }
    const bool big = left > kAfHeavy;
    if (big) heavy[atomicAdd(nheavy, 1)] = (int32_t)v;
    unsigned mask = __ballot_sync(0xffffffffu, left > 0 && !big);
    while (mask) {
      const int i = __ffs(mask) - 1;
      mask &= mask - 1;
      const int32_t u = (int32_t)(base + i);
#pragma unroll
      for (int c = 0; c < NC; ++c) {
        const OffT a = g.off[c][u], b = g.off[c][u + 1];
        for (OffT e = a + kSample + lane; e < b; e += 32) {
          const int32_t w = g.adj[c][e];
          if ((uint32_t)w >= (uint32_t)n) {
            ok = false;
            continue;
          }
          fine = af_link(u, w, parent) && fine;
        }
      }
    }
  }
  if (!ok) atomicOr(bad, 1);
  if (!fine) atomicCAS(err, 0, (int)kErrIterLimit);
}

template <typename OffT, int NC>
__global__ void k_af_rest_heavy(int32_t n, UfCsr<OffT, NC> g, int32_t* parent,
                                const int32_t* heavy, const int32_t* nheavy, int* bad, int* err) {
  if (*(volatile const int*)bad) return;
  const int nh = *nheavy;
  bool ok = true, fine = true;
  for (int i = blockIdx.x; i < nh; i += gridDim.x) {
    const int32_t u = heavy[i];
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      const OffT a = g.off[c][u], b = g.off[c][u + 1];
      for (OffT e = a + kSample + threadIdx.x; e < b; e += blockDim.x) {
        const int32_t w = g.adj[c][e];
        if ((uint32_t)w >= (uint32_t)n) {
          ok = false;
          continue;
        }
        fine = af_link(u, w, parent) && fine;
      }
    }
  }
  if (!ok) atomicOr(bad, 1);
  if (!fine) atomicCAS(err, 0, (int)kErrIterLimit);
}

__global__ void k_af_self(int32_t n, int32_t* parent) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (int64_t)gridDim.x * blockDim.x)
    parent[v] = (int32_t)v;
}

// The passes after the parents are set: sample, compress, the largest
// component, the rest, compress.
// scratch: [0] the largest component's root, [1] the heavy count, then n
// heavy entries.
template <typename OffT, int NC>
void af_passes(int32_t n, const UfCsr<OffT, NC>& g, int32_t* parent, int32_t* scratch, int* bad,
               int* err, cudaStream_t s) {
  const int gr = af_grid(n);
  cudaMemsetAsync(scratch + 1, 0, 4, s);
  k_af_sample<OffT, NC><<<gr, 256, 0, s>>>(n, g, parent, bad, err);
  k_af_compress<<<gr, 256, 0, s>>>(n, parent, err);
  k_af_mode<<<1, kModeSamples, 0, s>>>(n, parent, scratch);
  k_af_rest<OffT, NC><<<gr, 256, 0, s>>>(n, g, parent, scratch, scratch + 2, scratch + 1, bad, err);
  k_af_rest_heavy<OffT, NC><<<152 * 2, 1024, 0, s>>>(n, g, parent, scratch + 2, scratch + 1, bad,
                                                     err);
  k_af_compress<<<gr, 256, 0, s>>>(n, parent, err);
}

}  // namespace

cudaError_t cc_sampled(int32_t n, int64_t m, const uint32_t* h_off, const int32_t* h_adj,
                       int32_t* labels, int* d_bad, int* d_err, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  if (m >= (1ll << 32) - 16) return cudaErrorInvalidValue;
  uint32_t* off = nullptr;
  cudaError_t e = cudaMallocAsync(&off, ((size_t)2 * n + 3) * 4, s);
  if (e != cudaSuccess) return e;
  int32_t* giant = reinterpret_cast<int32_t*>(off + n + 1);  // and the heavy list
  int32_t* parent = labels;  // the roots become the labels
  k_af_init<<<af_grid((int64_t)n + 1), 256, 0, s>>>(h_off, n, m, off, parent, d_bad);
  if (m > 0) {
    UfCsr<uint32_t, 1> g;
    g.off[0] = off;
    g.adj[0] = h_adj;
    af_passes(n, g, parent, giant, d_bad, d_err, s);
  }
  e = cudaGetLastError();
  cudaFreeAsync(off, s);
  return e;
}

cudaError_t cc_sampled_device(int32_t n, const int64_t* out_off, const int32_t* out_adj,
                              const int64_t* in_off, const int32_t* in_adj, int32_t* labels,
                              int* d_bad, int* d_err, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  int32_t* giant = nullptr;  // and the heavy list
  cudaError_t e = cudaMallocAsync(&giant, ((size_t)n + 2) * 4, s);
  if (e != cudaSuccess) return e;
  k_af_self<<<af_grid(n), 256, 0, s>>>(n, labels);
  if (in_off == nullptr) {
    UfCsr<int64_t, 1> g;
    g.off[0] = out_off;
    g.adj[0] = out_adj;
    af_passes(n, g, labels, giant, d_bad, d_err, s);
  } else {
    UfCsr<int64_t, 2> g;
    g.off[0] = out_off;
    g.adj[0] = out_adj;
    g.off[1] = in_off;
    g.adj[1] = in_adj;
    af_passes(n, g, labels, giant, d_bad, d_err, s);
  }
  e = cudaGetLastError();
  cudaFreeAsync(giant, s);
  return e;
}

}  // namespace gb
