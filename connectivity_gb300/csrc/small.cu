// Connected components of small graphs, one thread block per graph.
//
// A graph of at most kSmallMaxN vertices fits the shared memory of one SM:
// its offsets, labels, flags, live degrees, frontier queues and a prefix
// array (nine int32 per vertex).  One 1024-thread block then runs the whole
// pipeline with block barriers only -- no cooperative grid, no grid
// barrier, no host round trip -- so a small graph costs a few microseconds
// per step instead of a grid-wide step, and a set of small graphs (a batch,
// or the requests of a server) runs as one launch with a block per graph.
//
// SCC (labels: the smallest member id of each component):
//   1. trim to the fixed point (scc_trim_complete, multistep/scc_trim.cpp:
//      141-297): a vertex without a valid in- or out-neighbour (self-loops
//      aside) is a component alone; removals propagate by live-degree
//      counters and a removed-vertex queue;
//   2. FW-BW (scc_fwbw.cpp:47-466) from the valid vertex of largest
//      out x in live degree (lowest id on ties): forward reach, backward
//      reach inside it; their intersection is one component;
//   3. colour rounds (scc_color.cpp:47-373): every vertex takes the
//      smallest id that reaches it (min-colour push to the fixed point),
//      every vertex whose colour is its own id is a root, and the vertices
//      of its colour that reach it (backward search) are its component;
//      after four of them, signature rounds until no vertex is left (the
//      smallest reaching and reached ids inside classes of equal pairs;
//      equal ids label the vertex).
// WCC (cc_main.cpp:184-245): union-find over the edges with hooking of the
// larger root under the smaller, so each root is its component's smallest
// id; no fixed-point loop.
//
// Frontier steps are edge-balanced: the frontier's degrees are scanned, and
// thread t takes edges t, t + 1024, ... of the concatenated edge lists,
// finding its vertex by a binary search over the scan, so a hub's edges are
// spread over the whole block.
//
// The CSR comes either from the caller (a device graph or a batch union,
// whose ids are offset by id_base) or from an edge list, counted and
// scattered here into a caller-provided scratch area (2m ints).
#include <cstdint>

#include "gb_internal.cuh"

namespace gb {
namespace {

constexpr int kST = 1024;
constexpr int kSW = kST / 32;
constexpr uint32_t kValid = 1u, kFw = 2u, kBw = 4u, kInq = 8u;
constexpr int kCtlInts = 160;

// control words (int32 slots of the shared control area)
constexpr int cQn = 0;       // queue lengths [2]
constexpr int cBad = 2;      // an edge id outside [0, n)
constexpr int cStop = 3;     // a loop ran out of steps
constexpr int cRed = 8;      // reductions: up to 3 * kSW words
constexpr int cScan = 112;   // scans: kSW + 1 words

__device__ __forceinline__ int warp_incl(int x) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  return x;
}

// Exclusive prefix sum of a[0..len) in place; returns the total.  Thread t
// owns a contiguous chunk.  Starts and ends with a barrier.
__device__ int32_t block_scan(int32_t* a, int len, int32_t* ctl) {
  __syncthreads();
  const int per = (len + kST - 1) / kST;
  const int lo = min(len, (int)threadIdx.x * per), hi = min(len, lo + per);
  int32_t s = 0;
  for (int i = lo; i < hi; ++i) s += a[i];
  const int inc = warp_incl(s);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int32_t* ws = ctl + cScan;
  if (lane == 31) ws[wid] = inc;
  __syncthreads();
  if (wid == 0) {
    const int v = lane < kSW ? ws[lane] : 0;
    const int vi = warp_incl(v);
    if (lane < kSW) ws[lane] = vi - v;
    if (lane == 31) ws[kSW] = vi;
  }
  __syncthreads();
  int32_t run = ws[wid] + inc - s;
  for (int i = lo; i < hi; ++i) {
    const int32_t x = a[i];
    a[i] = run;
    run += x;
  }
  const int32_t total = ws[kSW];
  __syncthreads();
  return total;
}

// Block sum of x.
__device__ int32_t block_sum(int32_t x, int32_t* ctl) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  __syncthreads();
  if (lane == 0) ctl[cRed + wid] = x;
  __syncthreads();
  int32_t t = 0;
  for (int i = 0; i < kSW; ++i) t += ctl[cRed + i];
  __syncthreads();
  return t;
}

// Block minimum of x.
__device__ int32_t block_min(int32_t x, int32_t* ctl) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o; o >>= 1) x = min(x, __shfl_xor_sync(0xffffffffu, x, o));
  __syncthreads();
  if (lane == 0) ctl[cRed + wid] = x;
  __syncthreads();
  int32_t t = x;
  for (int i = 0; i < kSW; ++i) t = min(t, ctl[cRed + i]);
  __syncthreads();
  return t;
}

// The largest key (then the smallest id) over the block: the pivot rule.
__device__ int32_t block_argmax(long long key, int32_t id, int32_t* ctl) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    const long long k2 = __shfl_xor_sync(0xffffffffu, key, o);
    const int32_t i2 = __shfl_xor_sync(0xffffffffu, id, o);
    if (k2 > key || (k2 == key && i2 < id)) { key = k2; id = i2; }
  }
  long long* rk = reinterpret_cast<long long*>(ctl + cRed);  // kSW long longs
  int32_t* ri = ctl + cRed + 2 * kSW;                          // then kSW ids
  __syncthreads();
  if (lane == 0) { rk[wid] = key; ri[wid] = id; }
  __syncthreads();
  for (int i = 0; i < kSW; ++i)
    if (rk[i] > key || (rk[i] == key && ri[i] < id)) { key = rk[i]; id = ri[i]; }
  __syncthreads();
  return id;
}

struct SmallCsr {
  const int32_t* ooff;  // n + 1 (shared)
  const int32_t* ioff;
  const int32_t* oadj;  // global
  const int32_t* iadj;
  int32_t base;         // subtracted from every adjacency entry
};

// Visits every edge (v, w) of the frontier's adjacency lists, edge-balanced.
// pre: n + 1 ints of scratch.  Ends with a barrier.
template <class F>
__device__ void expand_front(const int32_t* front, int nf, const int32_t* off, const int32_t* adj,
                             int32_t base, int32_t* pre, int32_t* ctl, F f) {
  for (int i = threadIdx.x; i < nf; i += kST) {
    const int32_t v = front[i];
    pre[i] = off[v + 1] - off[v];
  }
  const int32_t total = block_scan(pre, nf, ctl);
  for (int32_t e = threadIdx.x; e < total; e += kST) {
    int lo = 0, hi = nf - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (pre[mid] <= e) lo = mid;
      else hi = mid - 1;
    }
    const int32_t v = front[lo];
    f(v, adj[off[v] + (e - pre[lo])] - base);
  }
  __syncthreads();
}

// Every edge (u, w) of a CSR, edge-balanced over the block (u found by a
// binary search over the offsets).
template <class F>
__device__ void for_each_edge(int n, const int32_t* off, const int32_t* adj, int32_t base, F f) {
  const int32_t m = off[n];
  for (int32_t e = threadIdx.x; e < m; e += kST) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (off[mid] <= e) lo = mid;
      else hi = mid - 1;
    }
    f(lo, adj[e] - base);
  }
}

__device__ __forceinline__ void push(int32_t* q, int32_t* qn, int32_t v) {
  q[atomicAdd(qn, 1)] = v;
}

// Union-find root with path halving.  Parents only ever point at smaller
// ids, so a grandparent read at any time is still an ancestor.
__device__ __forceinline__ int32_t uf_find(int32_t* p, int32_t x) {
  volatile int32_t* vp = p;
  for (;;) {
    const int32_t px = vp[x];
    if (px == x) return x;
    const int32_t ppx = vp[px];
    if (ppx != px) vp[x] = ppx;
    x = px;
  }
}

__device__ __forceinline__ void uf_unite(int32_t* p, int32_t a, int32_t b) {
  for (;;) {
    const int32_t ra = uf_find(p, a), rb = uf_find(p, b);
    if (ra == rb) return;
    const int32_t lo = ra < rb ? ra : rb, hi = ra < rb ? rb : ra;
    if (atomicCAS(&p[hi], hi, lo) == hi) return;
  }
}

template <int KIND>
__global__ void __launch_bounds__(kST, 1) k_small(SmallDesc one, const SmallDesc* many,
                                                  int32_t max_steps, int32_t colour_rounds,
                                                  int* err) {
  extern __shared__ int32_t smem[];
  const SmallDesc D = many ? many[blockIdx.x] : one;
  const int n = D.n;
  if (n <= 0) return;
  const int tid = threadIdx.x;
  int32_t* ctl = smem;
  int32_t* ooff = smem + kCtlInts;
  int32_t* ioff = ooff + (n + 1);
  int32_t* lab = ioff + (n + 1);
  uint32_t* flg = reinterpret_cast<uint32_t*>(lab + n);
  int32_t* cnt_o = reinterpret_cast<int32_t*>(flg + n);
  int32_t* cnt_i = cnt_o + n;
  int32_t* q[2] = {cnt_i + n, cnt_i + 2 * n};
  int32_t* pre = cnt_i + 3 * n;  // n + 1
  int32_t* qn = ctl + cQn;
  const int32_t cap = (int32_t)min((long long)max_steps, 4ll * n + 64);
  if (tid == 0) {
    ctl[cBad] = 0;
    ctl[cStop] = 0;
  }

  // ---- WCC from an edge list: union-find over the edges, no CSR ----------
  if (KIND == 1 && D.out_off == nullptr) {
    for (int v = tid; v < n; v += kST) lab[v] = v;
    __syncthreads();
    for (long long e = tid; e < D.m; e += kST) {
      const int32_t a = D.src[e] - D.id_base, b = D.dst[e] - D.id_base;
      if ((unsigned)a >= (unsigned)n || (unsigned)b >= (unsigned)n) {
        ctl[cBad] = 1;
        continue;
      }
      uf_unite(lab, a, b);
    }
    __syncthreads();
    if (ctl[cBad]) {
      if (tid == 0) atomicCAS(err, 0, (int)kErrInvalid);
      return;
    }
    for (int v = tid; v < n; v += kST) D.labels[v] = uf_find(lab, v);
    return;
  }

  // ---- the CSR ------------------------------------------------------------
  SmallCsr g;
  if (D.out_off != nullptr) {
    const long long ob = D.out_off[0];
    const long long ib = D.in_off ? D.in_off[0] : ob;
    for (int v = tid; v <= n; v += kST) {
      ooff[v] = (int32_t)(D.out_off[v] - ob);
      ioff[v] = D.in_off ? (int32_t)(D.in_off[v] - ib) : ooff[v];
    }
    g.oadj = D.out_adj + ob;
    g.iadj = D.in_off ? D.in_adj + ib : g.oadj;
    g.base = D.id_base;
  } else {
    for (int v = tid; v < n; v += kST) {
      cnt_o[v] = 0;
      cnt_i[v] = 0;
    }
    __syncthreads();
    for (long long e = tid; e < D.m; e += kST) {
      const int32_t a = D.src[e] - D.id_base, b = D.dst[e] - D.id_base;
      if ((unsigned)a >= (unsigned)n || (unsigned)b >= (unsigned)n) {
        ctl[cBad] = 1;
        continue;
      }
      atomicAdd(&cnt_o[a], 1);
      atomicAdd(&cnt_i[b], 1);
    }
    __syncthreads();
    if (ctl[cBad]) {
      if (tid == 0) atomicCAS(err, 0, (int)kErrInvalid);
      return;
    }
    for (int v = tid; v < n; v += kST) {
      ooff[v] = cnt_o[v];
      ioff[v] = cnt_i[v];
    }
    if (tid == 0) {
      ooff[n] = 0;
      ioff[n] = 0;
    }
    block_scan(ooff, n + 1, ctl);
    block_scan(ioff, n + 1, ctl);
    for (int v = tid; v < n; v += kST) {
      cnt_o[v] = ooff[v];
      cnt_i[v] = ioff[v];
    }
    __syncthreads();
    int32_t* so = D.adj_scratch;
    int32_t* si = D.adj_scratch + D.m;
    for (long long e = tid; e < D.m; e += kST) {
      const int32_t a = D.src[e] - D.id_base, b = D.dst[e] - D.id_base;
      so[atomicAdd(&cnt_o[a], 1)] = b;
      si[atomicAdd(&cnt_i[b], 1)] = a;
    }
    __syncthreads();
    g.oadj = so;
    g.iadj = si;
    g.base = 0;
  }
  g.ooff = ooff;
  g.ioff = ioff;

  // ---- WCC on a CSR: union-find over the out-lists ------------------------
  if (KIND == 1) {
    for (int v = tid; v < n; v += kST) lab[v] = v;
    __syncthreads();
    for_each_edge(n, ooff, g.oadj, g.base, [&](int32_t u, int32_t w) { uf_unite(lab, u, w); });
    __syncthreads();
    for (int v = tid; v < n; v += kST) D.labels[v] = uf_find(lab, v);
    return;
  }

  // ---- SCC ----------------------------------------------------------------
  // live degrees without self-loops
  for (int v = tid; v < n; v += kST) {
    cnt_o[v] = ooff[v + 1] - ooff[v];
    cnt_i[v] = ioff[v + 1] - ioff[v];
    flg[v] = kValid;
    lab[v] = -1;
  }
  __syncthreads();
  for_each_edge(n, ooff, g.oadj, g.base, [&](int32_t u, int32_t w) {
    if (u == w) {
      atomicSub(&cnt_o[u], 1);
      atomicSub(&cnt_i[u], 1);
    }
  });
  if (tid == 0) qn[0] = 0;
  __syncthreads();

  // 1. trim to the fixed point
  for (int v = tid; v < n; v += kST) {
    if (cnt_o[v] == 0 || cnt_i[v] == 0) {
      flg[v] = 0;
      lab[v] = v;
      push(q[0], &qn[0], v);
    }
  }
  __syncthreads();
  auto claim_trim = [&](int32_t w, int nx) {
    const uint32_t old = atomicAnd(&flg[w], ~kValid);
    if (old & kValid) {
      lab[w] = w;
      push(q[nx], &qn[nx], w);
    }
  };
  int cur = 0;
  for (int32_t it = 0;; ++it) {
    const int nf = qn[cur];
    if (nf == 0) break;
    if (it >= cap) {
      ctl[cStop] = 1;
      break;
    }
    const int nx = cur ^ 1;
    if (tid == 0) qn[nx] = 0;
    __syncthreads();
    expand_front(q[cur], nf, ooff, g.oadj, g.base, pre, ctl, [&](int32_t v, int32_t w) {
      if (w != v && (flg[w] & kValid) && atomicSub(&cnt_i[w], 1) == 1) claim_trim(w, nx);
    });
    expand_front(q[cur], nf, ioff, g.iadj, g.base, pre, ctl, [&](int32_t v, int32_t w) {
      if (w != v && (flg[w] & kValid) && atomicSub(&cnt_o[w], 1) == 1) claim_trim(w, nx);
    });
    cur = nx;
  }
  __syncthreads();

  // 2. FW-BW from the pivot
  int32_t nvalid;
  {
    long long key = -1;
    int32_t id = 0x7fffffff;
    int32_t cnt = 0;
    for (int v = tid; v < n; v += kST) {
      if (flg[v] & kValid) {
        ++cnt;
        const long long k = (long long)cnt_o[v] * (long long)cnt_i[v];
        if (k > key || (k == key && v < id)) { key = k; id = v; }
      }
    }
    nvalid = block_sum(cnt, ctl);
    const int32_t pivot = block_argmax(key, id, ctl);
    if (nvalid > 0 && !ctl[cStop]) {
      for (int dir = 0; dir < 2; ++dir) {
        if (tid == 0) {
          flg[pivot] |= dir == 0 ? kFw : kBw;
          q[0][0] = pivot;
          qn[0] = 1;
        }
        __syncthreads();
        const int32_t* off = dir == 0 ? ooff : ioff;
        const int32_t* adj = dir == 0 ? g.oadj : g.iadj;
        const uint32_t want = dir == 0 ? kValid : (kValid | kFw);
        const uint32_t mask = dir == 0 ? (kValid | kFw) : (kValid | kFw | kBw);
        const uint32_t bit = dir == 0 ? kFw : kBw;
        cur = 0;
        for (int32_t it = 0;; ++it) {
          const int nf = qn[cur];
          if (nf == 0) break;
          if (it >= cap) {
            ctl[cStop] = 1;
            break;
          }
          const int nx = cur ^ 1;
          if (tid == 0) qn[nx] = 0;
          __syncthreads();
          expand_front(q[cur], nf, off, adj, g.base, pre, ctl, [&](int32_t v, int32_t w) {
            if ((flg[w] & mask) == want && !(atomicOr(&flg[w], bit) & bit))
              push(q[nx], &qn[nx], w);
          });
          cur = nx;
        }
        __syncthreads();
      }
      // the component: smallest member id as its label
      int32_t mn = 0x7fffffff;
      for (int v = tid; v < n; v += kST)
        if ((flg[v] & (kValid | kFw | kBw)) == (kValid | kFw | kBw)) mn = min(mn, v);
      mn = block_min(mn, ctl);
      int32_t cnt2 = 0;
      for (int v = tid; v < n; v += kST) {
        const uint32_t f = flg[v];
        if ((f & (kValid | kFw | kBw)) == (kValid | kFw | kBw)) {
          lab[v] = mn;
          flg[v] = 0;
          ++cnt2;
        } else {
          flg[v] = f & kValid;
        }
      }
      nvalid -= block_sum(cnt2, ctl);
    }
  }

  // 3. colour rounds (at most colour_rounds), then signature rounds for what
  // is left
  int32_t* col = cnt_o;  // live degrees are not needed any more
  int32_t round = 0;
  for (; nvalid > 0 && !ctl[cStop] && round < colour_rounds; ++round) {
    if (round >= cap) {
      ctl[cStop] = 1;
      break;
    }
    if (tid == 0) qn[0] = 0;
    __syncthreads();
    for (int v = tid; v < n; v += kST) {
      if (flg[v] & kValid) {
        col[v] = v;
        flg[v] = kValid | kInq;
        push(q[0], &qn[0], v);
      }
    }
    __syncthreads();
    // min colour pushed along out-edges to the fixed point
    cur = 0;
    for (int32_t it = 0;; ++it) {
      const int nf = qn[cur];
      if (nf == 0) break;
      if (it >= cap) {
        ctl[cStop] = 1;
        break;
      }
      const int nx = cur ^ 1;
      if (tid == 0) qn[nx] = 0;
      for (int i = tid; i < nf; i += kST) atomicAnd(&flg[q[cur][i]], ~kInq);
      __syncthreads();
      expand_front(q[cur], nf, ooff, g.oadj, g.base, pre, ctl, [&](int32_t v, int32_t w) {
        if (!(flg[w] & kValid)) return;
        const int32_t cv = col[v];
        if (col[w] > cv && atomicMin(&col[w], cv) > cv && !(atomicOr(&flg[w], kInq) & kInq))
          push(q[nx], &qn[nx], w);
      });
      cur = nx;
    }
    if (ctl[cStop]) break;
    // roots, then the vertices of each root's colour that reach it
    if (tid == 0) qn[0] = 0;
    __syncthreads();
    for (int v = tid; v < n; v += kST) {
      if ((flg[v] & kValid) && col[v] == v) {
        flg[v] = kValid | kFw;
        push(q[0], &qn[0], v);
      }
    }
    __syncthreads();
    cur = 0;
    for (int32_t it = 0;; ++it) {
      const int nf = qn[cur];
      if (nf == 0) break;
      if (it >= cap) {
        ctl[cStop] = 1;
        break;
      }
      const int nx = cur ^ 1;
      if (tid == 0) qn[nx] = 0;
      __syncthreads();
      expand_front(q[cur], nf, ioff, g.iadj, g.base, pre, ctl, [&](int32_t v, int32_t w) {
        if ((flg[w] & (kValid | kFw)) == kValid && col[w] == col[v] &&
            !(atomicOr(&flg[w], kFw) & kFw))
          push(q[nx], &qn[nx], w);
      });
      cur = nx;
    }
    int32_t cnt3 = 0;
    for (int v = tid; v < n; v += kST) {
      if ((flg[v] & (kValid | kFw)) == (kValid | kFw)) {
        lab[v] = col[v];
        flg[v] = 0;
        ++cnt3;
      }
    }
    nvalid -= block_sum(cnt3, ctl);
  }
  // Signature rounds (a deep condensation, such as a long chain between
  // cycles, would take one colour round per component): each round, fw = the
  // smallest id reaching a vertex and bw = the smallest id it reaches, both
  // inside its class (kept in lab[] while the vertex is valid; one class at
  // first); fw == bw labels the vertex with that id, its SCC's smallest
  // member; the others take the pair as their class.
  if (nvalid > 0 && !ctl[cStop]) {
    int32_t* fw = cnt_o;
    int32_t* bw = cnt_i;
    for (int v = tid; v < n; v += kST)
      if (flg[v] & kValid) lab[v] = 0;
    __syncthreads();
    auto propagate = [&](int32_t* val, const int32_t* off, const int32_t* adj) {
      if (tid == 0) qn[0] = 0;
      __syncthreads();
      for (int v = tid; v < n; v += kST) {
        if (flg[v] & kValid) {
          val[v] = v;
          flg[v] = kValid | kInq;
          push(q[0], &qn[0], v);
        }
      }
      __syncthreads();
      cur = 0;
      for (int32_t it = 0;; ++it) {
        const int nf = qn[cur];
        if (nf == 0) break;
        if (it >= cap) {
          ctl[cStop] = 1;
          break;
        }
        const int nx = cur ^ 1;
        if (tid == 0) qn[nx] = 0;
        for (int i = tid; i < nf; i += kST) atomicAnd(&flg[q[cur][i]], ~kInq);
        __syncthreads();
        expand_front(q[cur], nf, off, adj, g.base, pre, ctl, [&](int32_t v, int32_t w) {
          if (!(flg[w] & kValid) || lab[w] != lab[v]) return;
          const int32_t cv = val[v];
          if (val[w] > cv && atomicMin(&val[w], cv) > cv && !(atomicOr(&flg[w], kInq) & kInq))
            push(q[nx], &qn[nx], w);
        });
        cur = nx;
      }
    };
    for (; nvalid > 0 && !ctl[cStop]; ++round) {
      if (round >= cap) {
        ctl[cStop] = 1;
        break;
      }
      propagate(fw, ooff, g.oadj);
      if (ctl[cStop]) break;
      propagate(bw, ioff, g.iadj);
      if (ctl[cStop]) break;
      int32_t cnt4 = 0;
      for (int v = tid; v < n; v += kST) {
        if (flg[v] & kValid) {
          const int32_t f = fw[v], b = bw[v];
          if (f == b) {
            lab[v] = f;
            flg[v] = 0;
            ++cnt4;
          } else {
            uint32_t x = (uint32_t)f * 0x9E3779B1u;
            x ^= (uint32_t)b * 0x85EBCA77u + 0x7F4A7C15u + (x << 6) + (x >> 2);
            lab[v] = (int32_t)x;
          }
        }
      }
      nvalid -= block_sum(cnt4, ctl);
    }
  }
  __syncthreads();
  if (ctl[cStop]) {
    if (tid == 0) atomicCAS(err, 0, (int)kErrIterLimit);
    return;
  }
  for (int v = tid; v < n; v += kST) D.labels[v] = lab[v];
}

template <int KIND>
cudaError_t launch_k(const SmallDesc& one, const SmallDesc* many, int count, int32_t max_n,
                     int32_t max_steps, int32_t colour_rounds, int* err, cudaStream_t s) {
  // the shared-memory attribute, once per device
  static bool attr_set[64][2] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const size_t smem = small_smem_bytes(max_n);
  if (dev < 0 || dev >= 64 || !attr_set[dev][KIND]) {
    e = cudaFuncSetAttribute(k_small<KIND>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)small_smem_bytes(kSmallMaxN));
    if (e != cudaSuccess) return e;
    if (dev >= 0 && dev < 64) attr_set[dev][KIND] = true;
  }
  k_small<KIND><<<count, kST, smem, s>>>(one, many, max_steps, colour_rounds, err);
  return cudaGetLastError();
}

}  // namespace

size_t small_smem_bytes(int32_t max_n) {
  const size_t n = (size_t)(max_n > 0 ? max_n : 1);
  return (size_t)kCtlInts * 4 + (9 * n + 3) * 4;
}

cudaError_t launch_small(int kind, const SmallDesc& one, const SmallDesc* many, int count,
                         int32_t max_n, int32_t max_steps, int* err, cudaStream_t s,
                         int32_t colour_mode) {
  if (count <= 0) return cudaSuccess;
  if (max_n > kSmallMaxN) return cudaErrorInvalidValue;
  // colour rounds before the signature rounds: all (0), none (1), four (2)
  const int32_t cr = colour_mode == 0 ? 0x7fffffff : (colour_mode == 1 ? 0 : 4);
  return kind == 0 ? launch_k<0>(one, many, count, max_n, max_steps, cr, err, s)
                   : launch_k<1>(one, many, count, max_n, max_steps, cr, err, s);
}

}  // namespace gb
